// ssfft_multi.cu -- a fixed batch of complex transforms of uneven sizes in one submission.
//
// The reference transforms one size per FFT object, so a caller with transforms of many sizes
// loops over objects (signalsmith-fft.h:374-386 per call).  ssfft_multi_* takes the whole list
// once: transforms are grouped by size, each size gets its size-specialised kernel (compiled
// concurrently at creation) and a device table of its transforms' offsets, so the caller's
// layout (transform i at the prefix sum of the sizes before it) needs no reordering.  Execution
// is one CUDA graph whose launches (one per size) sit on up to 8 parallel branches, balanced by
// work, so small sizes fill the GPU together instead of one after another; the graph is
// captured once per (input, output, direction) and replayed.  ssfft_multi_exec_plain issues the
// same launches one after another on the caller's stream, for comparison.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#include "ssfft_host.h"

namespace ssfft {

ssfft_status launch_batch_offs(const Plan *p, int inverse, const void *in, void *out, size_t batch,
                               const long long *d_offs, cudaStream_t s);
ssfft_status plan_prepare_launch(const Plan *p);

namespace {

constexpr int kMaxBranches = 32;

struct Group {
	size_t n = 0, count = 0;
	ssfft_plan_t plan = nullptr;
	long long *d_offs = nullptr;
	double work = 0;
	int branch = 0;
};

struct GraphKey {
	const void *in;
	void *out;
	int inverse;
	bool operator<(const GraphKey &o) const { return std::tie(in, out, inverse) < std::tie(o.in, o.out, o.inverse); }
};

}  // namespace

struct MultiPlan {
	ssfft_dtype dtype = SSFFT_F32;
	int device = 0;
	size_t total = 0;
	std::vector<Group> groups;
	cudaStream_t cap = nullptr;
	int branches = 8;  // parallel graph branches (debug switch multi_branches overrides, up to 32)
	cudaStream_t branch[kMaxBranches] = {};
	cudaEvent_t fork = nullptr, join[kMaxBranches] = {};
	std::mutex mu;
	std::map<GraphKey, cudaGraphExec_t> graphs;

	~MultiPlan() {
		for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
		for (auto &g : groups) {
			if (g.d_offs) cudaFree(g.d_offs);
			if (g.plan) ssfft_plan_destroy(g.plan);
		}
		for (int b = 0; b < kMaxBranches; ++b) {
			if (join[b]) cudaEventDestroy(join[b]);
			if (branch[b]) cudaStreamDestroy(branch[b]);
		}
		if (fork) cudaEventDestroy(fork);
		if (cap) cudaStreamDestroy(cap);
	}

	ssfft_status launch_all(int inverse, const void *in, void *out, cudaStream_t *streams) {
		for (auto &g : groups) {
			ssfft_status st = launch_batch_offs(reinterpret_cast<const Plan *>(g.plan), inverse, in, out, g.count,
			                                    g.d_offs, streams[g.branch]);
			if (st != SSFFT_SUCCESS) return st;
		}
		return SSFFT_SUCCESS;
	}

	ssfft_status capture(const GraphKey &k, cudaGraphExec_t &exec) {
		cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
		if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
		ssfft_status st = SSFFT_SUCCESS;
		e = cudaEventRecord(fork, cap);
		for (int b = 0; b < branches && e == cudaSuccess; ++b) e = cudaStreamWaitEvent(branch[b], fork, 0);
		if (e == cudaSuccess) st = launch_all(k.inverse, k.in, k.out, branch);
		for (int b = 0; b < branches && e == cudaSuccess; ++b) {
			e = cudaEventRecord(join[b], branch[b]);
			if (e == cudaSuccess) e = cudaStreamWaitEvent(cap, join[b], 0);
		}
		cudaGraph_t graph = nullptr;
		cudaError_t e2 = cudaStreamEndCapture(cap, &graph);
		if (e != cudaSuccess) return cuda_fail(e, "multi capture");
		if (st != SSFFT_SUCCESS) {
			if (graph) cudaGraphDestroy(graph);
			return st;
		}
		if (e2 != cudaSuccess) return cuda_fail(e2, "cudaStreamEndCapture");
		e = cudaGraphInstantiate(&exec, graph, 0);
		cudaGraphDestroy(graph);
		if (e != cudaSuccess) return cuda_fail(e, "cudaGraphInstantiate");
		return SSFFT_SUCCESS;
	}
};

}  // namespace ssfft

using namespace ssfft;

extern "C" {

ssfft_status ssfft_multi_create(ssfft_multi_t *out, const size_t *sizes, size_t count, ssfft_dtype dtype) {
	return ssfft_multi_create_ex(out, sizes, count, dtype, nullptr);
}

ssfft_status ssfft_multi_create_ex(ssfft_multi_t *out, const size_t *sizes, size_t count, ssfft_dtype dtype,
                                   const ssfft_plan_options *opt) {
	if (!out || !sizes || count == 0) return SSFFT_ERR_INVALID_VALUE;
	if (opt && opt->radices[0] != 0) return SSFFT_ERR_INVALID_VALUE;  // one radix list cannot fit every size
	if (dtype != SSFFT_F32 && dtype != SSFFT_F64) return SSFFT_ERR_INVALID_VALUE;
	*out = nullptr;
	std::unique_ptr<MultiPlan> m(new MultiPlan());
	m->dtype = dtype;
	cudaError_t e = cudaGetDevice(&m->device);
	if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
	// offsets of every transform (in scalars), grouped by size
	const size_t max_n = dtype == SSFFT_F32 ? (size_t)kMaxSubTransform : (size_t)kMaxSubTransform / 2;
	std::map<size_t, std::vector<long long>> by_size;
	long long off = 0;
	for (size_t i = 0; i < count; ++i) {
		if (sizes[i] == 0 || sizes[i] > max_n) return SSFFT_ERR_UNSUPPORTED;
		by_size[sizes[i]].push_back(off);
		off += 2 * (long long)sizes[i];
	}
	m->total = (size_t)off / 2;
	for (auto &kv : by_size) {
		Group g;
		g.n = kv.first;
		g.count = kv.second.size();
		g.work = (double)g.count * (double)g.n * std::log2((double)std::max<size_t>(g.n, 2));
		m->groups.push_back(g);
	}
	// per-size plans, compiled concurrently
	std::atomic<size_t> next{0};
	std::atomic<int> bad{0};
	std::vector<std::thread> th;
	const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
	const int dev = m->device;
	MultiPlan *mp = m.get();
	for (int t = 0; t < nt; ++t)
		th.emplace_back([&, mp, dev] {
			cudaSetDevice(dev);
			for (size_t i = next++; i < mp->groups.size(); i = next++) {
				Group &g = mp->groups[i];
				if (ssfft_plan_create_ex(&g.plan, g.n, mp->dtype, SSFFT_COMPLEX, g.count, opt) != SSFFT_SUCCESS) bad = 1;
			}
		});
	for (auto &x : th) x.join();
	if (bad) return SSFFT_ERR_UNSUPPORTED;
	for (auto &g : m->groups) {  // every size must run in one CTA (offset-table launches)
		const Plan *p = reinterpret_cast<const Plan *>(g.plan);
		if (p->large) return SSFFT_ERR_UNSUPPORTED;
		// the graph capture must not load modules: compile every kernel a launch may use now
		ssfft_status st = plan_prepare_launch(p);
		if (st != SSFFT_SUCCESS) return st;
	}
	for (auto &g : m->groups) {
		const auto &offs = by_size[g.n];
		e = cudaMalloc(&g.d_offs, offs.size() * sizeof(long long));
		if (e == cudaSuccess)
			e = cudaMemcpy(g.d_offs, offs.data(), offs.size() * sizeof(long long), cudaMemcpyHostToDevice);
		if (e != cudaSuccess) return cuda_fail(e, "multi offsets");
	}
	// branches balanced by work, largest first
	std::vector<size_t> order(m->groups.size());
	for (size_t i = 0; i < order.size(); ++i) order[i] = i;
	std::sort(order.begin(), order.end(), [&](size_t a, size_t b) { return m->groups[a].work > m->groups[b].work; });
	{
		const long long nb_dbg = debug_knob("multi_branches", 0);
		if (nb_dbg > 0) m->branches = (int)std::min<long long>(kMaxBranches, nb_dbg);
	}
	const int nb = m->branches;
	double load[kMaxBranches] = {};
	for (size_t i : order) {
		int best = 0;
		for (int b = 1; b < nb; ++b)
			if (load[b] < load[best]) best = b;
		m->groups[i].branch = best;
		load[best] += m->groups[i].work;
	}
	std::vector<Group> sorted;
	for (size_t i : order) sorted.push_back(m->groups[i]);
	m->groups.swap(sorted);
	e = cudaStreamCreateWithFlags(&m->cap, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaEventCreateWithFlags(&m->fork, cudaEventDisableTiming);
	for (int b = 0; b < nb && e == cudaSuccess; ++b) {
		e = cudaStreamCreateWithFlags(&m->branch[b], cudaStreamNonBlocking);
		if (e == cudaSuccess) e = cudaEventCreateWithFlags(&m->join[b], cudaEventDisableTiming);
	}
	if (e != cudaSuccess) return cuda_fail(e, "multi streams");
	*out = reinterpret_cast<ssfft_multi_t>(m.release());
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_multi_exec(ssfft_multi_t multi, int inverse, const void *d_in, void *d_out, void *stream) {
	if (!multi || !d_in || !d_out) return SSFFT_ERR_INVALID_VALUE;
	MultiPlan *m = reinterpret_cast<MultiPlan *>(multi);
	const size_t align = m->dtype == SSFFT_F32 ? 8 : 16;
	if ((uintptr_t)d_in % align || (uintptr_t)d_out % align) return SSFFT_ERR_INVALID_VALUE;
	std::lock_guard<std::mutex> lock(m->mu);
	GraphKey k{d_in, d_out, inverse ? 1 : 0};
	auto it = m->graphs.find(k);
	if (it == m->graphs.end()) {
		cudaGraphExec_t exec = nullptr;
		ssfft_status st = m->capture(k, exec);
		if (st != SSFFT_SUCCESS) return st;
		if (m->graphs.size() >= 16) {  // bounded cache of captured graphs
			cudaGraphExecDestroy(m->graphs.begin()->second);
			m->graphs.erase(m->graphs.begin());
		}
		it = m->graphs.emplace(k, exec).first;
	}
	cudaError_t e = cudaGraphLaunch(it->second, static_cast<cudaStream_t>(stream));
	if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_multi_exec_plain(ssfft_multi_t multi, int inverse, const void *d_in, void *d_out, void *stream) {
	if (!multi || !d_in || !d_out) return SSFFT_ERR_INVALID_VALUE;
	MultiPlan *m = reinterpret_cast<MultiPlan *>(multi);
	cudaStream_t s[kMaxBranches];
	for (int b = 0; b < kMaxBranches; ++b) s[b] = static_cast<cudaStream_t>(stream);
	return m->launch_all(inverse ? 1 : 0, d_in, d_out, s);
}

ssfft_status ssfft_multi_info(ssfft_multi_t multi, size_t *distinct_sizes, size_t *total_elements) {
	if (!multi) return SSFFT_ERR_INVALID_VALUE;
	MultiPlan *m = reinterpret_cast<MultiPlan *>(multi);
	if (distinct_sizes) *distinct_sizes = m->groups.size();
	if (total_elements) *total_elements = m->total;
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_multi_destroy(ssfft_multi_t multi) {
	if (!multi) return SSFFT_ERR_INVALID_VALUE;
	delete reinterpret_cast<MultiPlan *>(multi);
	return SSFFT_SUCCESS;
}

}  // extern "C"

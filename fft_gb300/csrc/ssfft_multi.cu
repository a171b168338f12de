// ssfft_multi.cu -- a fixed batch of complex transforms of uneven sizes in one submission.
//
// The reference transforms one size per FFT object, so a caller with transforms of many sizes
// loops over objects (signalsmith-fft.h:374-386 per call).  ssfft_multi_* takes the whole list
// once and runs it as a queue of work items:
//   * every distinct size gets its size-specialised schedule (the planner's) and a device table
//     of its transforms' offsets, so the caller's layout (transform i at the prefix sum of the
//     sizes before it) needs no reordering;
//   * sizes whose schedules share a CTA shape (threads per CTA rounded up to a multiple of 128,
//     values per thread, register cap) form a class; one kernel per class (ssfft_cl::queue,
//     compiled concurrently at creation; classes of more than 16 sizes are cut into several)
//     holds its sizes' passes as compile-time members;
//   * a class's transforms are cut into work items of as many transforms as one CTA runs, and
//     the items are queued longest transforms first: CTA b of the class's single launch takes
//     item b, so the long work starts first and the short work fills the last wave;
//   * the class launches are one CUDA graph (parallel branches, largest class first, so CTAs of
//     different classes share the SMs), captured once per (input, output, direction).
// ssfft_multi_exec_plain issues one plain launch per size, one after another on the caller's
// stream, for comparison; the debug switch multi_mode=1 runs the earlier design instead (one
// CUDA graph of per-size launches on parallel branches).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <thread>
#include <tuple>
#include <vector>

#include "ssfft_host.h"

namespace ssfft {

ssfft_status plan_prepare_launch(const Plan *p);

namespace {

constexpr int kMaxBranches = 32;
constexpr int kQueueBucket = 128;     // queue CTAs: threads rounded up to a multiple of this
// Measured on GB300 (32768 transforms log-uniform over 64-16384 points): every split between
// queue classes and per-size launches lands at 0.59-0.62 ms; sizes up to 1024 points in classes
// of four is the fastest (0.595 ms against 0.601 for one launch per size), and classes of long
// sizes or of many sizes are slower (0.88 ms with every size in classes of 16).
constexpr size_t kQueueMembers = 4;   // sizes per queue kernel at most
constexpr size_t kQueueMaxN = 1024;   // longest size run by a queue class (longer: own launch)

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

// One queue class: the sizes whose queue schedules share (CTA threads, values per thread,
// register cap), run by one ssfft_cl::queue launch.
struct QClass {
	ssfft_dtype dtype = SSFFT_F32;
	int cta = 0, emax = 16, minb = 1;
	size_t smem = 0;
	std::vector<size_t> members;   // indices into MultiPlan::groups
	std::vector<Schedule> sch;     // member schedules (per_cta = transforms per work item)
	CUfunction fwd = nullptr, inv = nullptr;
	const int *d_kidx = nullptr;   // member of each item
	const int *d_toff = nullptr;   // item x thread: transform offset in complex elements (-1: none)
	ssfft_cl::QSched *d_sch = nullptr;
	long long nitems = 0;
	long long pf_dist = 0;
	double work = 0;
	int branch = 0;

	std::string name(bool inverse) const {
		std::string r = "ssfft_cl::queue<";
		r += dtype == SSFFT_F32 ? "float" : "double";
		r += std::string(", ") + (inverse ? "true" : "false") + ", " + std::to_string(cta) + ", " + std::to_string(minb);
		for (const Schedule &q : sch) {
			r += ", ssfft_cl::QS<" + std::to_string(q.n) + ", " + std::to_string(q.threads) + ", " +
			     std::to_string(q.smem_stride) + ", " + std::to_string(q.emax);
			for (int x : q.radices) r += ", " + std::to_string(x);
			r += ">";
		}
		return r + ">";
	}
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
	bool queue_mode = true;        // work-item queue kernels (false: one launch per size)
	std::vector<QClass> classes;   // queue mode: sizes up to queue_max_n
	std::vector<size_t> big;       // queue mode: groups above queue_max_n, one launch per size
	size_t queue_max_n = 0;
	void *d_queue = nullptr;       // queue mode: items, per-schedule records and twiddle tables

	~MultiPlan() {
		for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
		if (d_queue) cudaFree(d_queue);
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

	ssfft_status launch_queue(int inverse, const void *in, void *out, cudaStream_t *streams) {
		for (const QClass &c : classes) {
			ssfft_cl::QueueArgs a;
			std::memset(&a, 0, sizeof a);
			a.in = in;
			a.out = out;
			a.kidx = c.d_kidx;
			a.toff = c.d_toff;
			a.nitems = c.nitems;
			a.sch = c.d_sch;
			a.pf_dist = c.pf_dist;
			ssfft_status st = jit_launch(inverse ? c.inv : c.fwd, (unsigned)c.nitems, (unsigned)c.cta, c.smem,
			                             streams[c.branch], &a);
			if (st != SSFFT_SUCCESS) return st;
		}
		for (size_t gi : big) {
			const Group &g = groups[gi];
			ssfft_status st = launch_batch_offs(reinterpret_cast<const Plan *>(g.plan), inverse, in, out, g.count,
			                                    g.d_offs, streams[g.branch]);
			if (st != SSFFT_SUCCESS) return st;
		}
		return SSFFT_SUCCESS;
	}

	ssfft_status launch_all(int inverse, const void *in, void *out, cudaStream_t *streams) {
		if (queue_mode) return launch_queue(inverse, in, out, streams);
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

	ssfft_status build_queue(const std::vector<std::vector<long long>> &elem_offs);
};

// Queue schedule of one size: the planner's schedule (no staged or tensor-core variant), its
// transforms per work item filling a CTA of threads rounded up to kQueueBucket.
static bool queue_schedule(ssfft_dtype dtype, size_t n, size_t count, Schedule &s, int &cta) {
	if (!make_schedule(dtype, (int)n, ssfft_cl::kComplex, false, count, s, 0, nullptr, 0)) return false;
	if (s.staged || s.tc || s.pair) return false;
	// the debug switch queue_bucket overrides the rounding (a multiple of 32; with 32 a class is
	// the planner's own CTA shape rounded to whole warps)
	const long long qb = debug_knob("queue_bucket", kQueueBucket);
	const int bucket = qb >= 32 && qb <= 1024 && qb % 32 == 0 ? (int)qb : kQueueBucket;
	if (bucket < kQueueBucket) {
		cta = (s.threads * s.per_cta + bucket - 1) / bucket * bucket;
		const size_t eb0 = dtype == SSFFT_F32 ? 8 : 16;
		if ((size_t)s.per_cta > count) s.per_cta = (int)std::max<size_t>(1, count);
		s.smem_bytes = (size_t)s.per_cta * (size_t)s.smem_stride * eb0;
		return true;
	}
	cta = (s.threads + bucket - 1) / bucket * bucket;
	const size_t eb = dtype == SSFFT_F32 ? 8 : 16;
	const size_t per = (size_t)s.smem_stride * eb;
	int g = std::max(1, cta / s.threads);
	// at most 48 KiB of shared memory per CTA unless one transform needs more (as the planner)
	while (g > 1 && (size_t)g * per > std::max<size_t>(per, 48 * 1024)) --g;
	if ((size_t)g > count) g = (int)std::max<size_t>(1, count);
	s.per_cta = g;
	s.smem_bytes = (size_t)g * per;
	return true;
}

static size_t qalign(size_t v) { return (v + 255) / 256 * 256; }

// The queue classes of distinct sizes (n, transform count, work), largest class first; members
// index into `sizes`.  No GPU needed.
static ssfft_status form_classes(ssfft_dtype dtype, const std::vector<std::tuple<size_t, size_t, double>> &sizes,
                                 std::vector<QClass> &classes) {
	// classes by (CTA threads, values per thread, register cap of the member's own schedule)
	std::map<std::tuple<int, int, int>, QClass> cls;
	for (size_t gi = 0; gi < sizes.size(); ++gi) {
		Schedule s;
		int cta = 0;
		if (!queue_schedule(dtype, std::get<0>(sizes[gi]), std::get<1>(sizes[gi]), s, cta))
			return SSFFT_ERR_UNSUPPORTED;
		QClass &c = cls[std::make_tuple(cta, s.emax, s.minb)];
		c.dtype = dtype;
		c.cta = cta;
		c.emax = s.emax;
		c.minb = std::max(c.minb, s.minb);
		c.smem = std::max(c.smem, s.smem_bytes);
		c.members.push_back(gi);
		c.sch.push_back(s);
		c.work += std::get<2>(sizes[gi]);
	}
	classes.clear();
	for (auto &kv : cls) {
		// members longest first (the queue's order)
		QClass &c = kv.second;
		std::vector<size_t> ord(c.members.size());
		for (size_t i = 0; i < ord.size(); ++i) ord[i] = i;
		std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) { return c.sch[a].n > c.sch[b].n; });
		std::vector<size_t> mem;
		std::vector<Schedule> sch;
		for (size_t i : ord) {
			mem.push_back(c.members[i]);
			sch.push_back(c.sch[i]);
		}
		// at most kQueueMembers sizes per kernel (debug switch queue_members): each member's passes
		// are fully unrolled, and a kernel holding many of them thrashes the instruction cache
		// (measured on GB300: 16 sizes of 900-2048 points, 0.82 of the copy bandwidth as one-size
		// classes, 0.46 as one 16-size class, no_instruction stalls 5.9 per issue); NVRTC's time
		// also grows faster than the member count
		const long long qm = debug_knob("queue_members", (long long)kQueueMembers);
		const size_t members = qm >= 1 && qm <= 64 ? (size_t)qm : kQueueMembers;
		for (size_t b = 0; b < mem.size(); b += members) {
			QClass part = c;
			part.members.assign(mem.begin() + b, mem.begin() + std::min(mem.size(), b + members));
			part.sch.assign(sch.begin() + b, sch.begin() + std::min(sch.size(), b + members));
			part.smem = 0;
			part.work = 0;
			for (size_t k = 0; k < part.sch.size(); ++k) {
				part.smem = std::max(part.smem, part.sch[k].smem_bytes);
				part.work += std::get<2>(sizes[part.members[k]]);
			}
			classes.push_back(part);
		}
	}
	std::stable_sort(classes.begin(), classes.end(), [](const QClass &a, const QClass &b) { return a.work > b.work; });
	return SSFFT_SUCCESS;
}

// One work item of a class: `count` transforms of member k, its transforms first .. first+count-1.
struct QueueItem {
	int k, count;
	size_t first;
};

// The work items of one class, in queue order: member by member (longest first), each member's
// transforms in groups of its transforms per CTA.
static void class_items(const QClass &c, const std::vector<size_t> &counts, std::vector<QueueItem> &items) {
	items.clear();
	for (size_t k = 0; k < c.sch.size(); ++k) {
		const size_t cnt = counts[c.members[k]];
		const int per = c.sch[k].per_cta;
		for (size_t f = 0; f < cnt; f += (size_t)per)
			items.push_back(QueueItem{(int)k, (int)std::min<size_t>((size_t)per, cnt - f), f});
	}
}

// The device tables of a class queue: kidx[b] = member of item b; toff[b * cta + t] = offset, in
// complex elements, of the transform thread t of item b works on (-1: none).  elem_offs[m] lists
// the element offsets of member-size m's transforms (indexed like `counts`).
static void class_tables(const QClass &c, const std::vector<QueueItem> &items,
                         const std::vector<std::vector<long long>> &elem_offs, std::vector<int> &kidx,
                         std::vector<int> &toff) {
	kidx.resize(items.size());
	toff.assign(items.size() * (size_t)c.cta, -1);
	for (size_t b = 0; b < items.size(); ++b) {
		const QueueItem &it = items[b];
		kidx[b] = it.k;
		const int th = c.sch[it.k].threads;
		const std::vector<long long> &offs = elem_offs[c.members[it.k]];
		for (int t = 0; t < c.cta; ++t) {
			const int g = t / th;
			if (g < it.count) toff[b * (size_t)c.cta + t] = (int)offs[it.first + (size_t)g];
		}
	}
}

ssfft_status MultiPlan::build_queue(const std::vector<std::vector<long long>> &group_offs) {
	// sizes up to queue_max_n go into queue classes; longer ones keep their own launch (a class
	// kernel holding several long fully unrolled transforms thrashes the instruction cache)
	std::vector<std::tuple<size_t, size_t, double>> sizes;
	std::vector<size_t> counts;
	std::vector<std::vector<long long>> elem_offs;
	big.clear();
	for (size_t gi = 0; gi < groups.size(); ++gi) {
		const Group &g = groups[gi];
		if (g.n > queue_max_n) {
			big.push_back(gi);
			continue;
		}
		sizes.emplace_back(g.n, g.count, g.work);
		counts.push_back(g.count);
		elem_offs.push_back(group_offs[gi]);
	}
	ssfft_status fst = form_classes(dtype, sizes, classes);
	if (fst != SSFFT_SUCCESS) return fst;
	const size_t smem_limit = device_smem_limit(device);
	for (const QClass &c : classes)
		if (c.smem > smem_limit) return SSFFT_ERR_UNSUPPORTED;
	// one class kernel per compile, concurrently
	std::atomic<size_t> next{0};
	std::atomic<int> bad{0};
	std::vector<std::thread> th;
	const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
	const int dev = device;
	for (int t = 0; t < nt; ++t)
		th.emplace_back([&, dev] {
			cudaSetDevice(dev);
			for (size_t i = next++; i < classes.size(); i = next++) {
				QClass &c = classes[i];
				std::vector<CUfunction> fns;
				if (jit_kernels({c.name(false), c.name(true)}, c.smem, fns) != SSFFT_SUCCESS) {
					bad = 1;
					continue;
				}
				c.fwd = fns[0];
				c.inv = fns[1];
			}
		});
	for (auto &x : th) x.join();
	if (bad) return SSFFT_ERR_CUDA;
	// device layout: per class its member indices, per-thread offsets and member records; then
	// every member's tables
	std::vector<std::vector<int>> kidx(classes.size()), toff(classes.size());
	std::vector<std::vector<double>> tw_all, roots_all;
	size_t off = 0;
	std::vector<size_t> off_kidx(classes.size()), off_toff(classes.size()), off_sch(classes.size());
	for (size_t ci = 0; ci < classes.size(); ++ci) {
		QClass &c = classes[ci];
		std::vector<QueueItem> items;
		class_items(c, counts, items);
		class_tables(c, items, elem_offs, kidx[ci], toff[ci]);
		for (size_t k = 0; k < c.sch.size(); ++k) {
			std::vector<double> tw, roots;
			schedule_twiddles(c.sch[k], tw, roots);
			tw_all.push_back(tw);
			roots_all.push_back(roots);
		}
		c.nitems = (long long)items.size();
		if (c.nitems > 0x7fffffffLL) return SSFFT_ERR_INVALID_SIZE;
		off_kidx[ci] = off;
		off = qalign(off + kidx[ci].size() * sizeof(int));
		off_toff[ci] = off;
		off = qalign(off + toff[ci].size() * sizeof(int));
		off_sch[ci] = off;
		off = qalign(off + c.sch.size() * sizeof(ssfft_cl::QSched));
	}
	const size_t sb = dtype == SSFFT_F32 ? 4 : 8;
	std::vector<size_t> off_tw(tw_all.size()), off_roots(tw_all.size());
	for (size_t i = 0; i < tw_all.size(); ++i) {
		off_tw[i] = off;
		off = qalign(off + tw_all[i].size() * sb);
		off_roots[i] = off;
		off = qalign(off + roots_all[i].size() * sb);
	}
	const size_t total = std::max<size_t>(off, 256);
	cudaError_t e = cudaMalloc(&d_queue, total);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(multi queue)");
	unsigned char *base = static_cast<unsigned char *>(d_queue);
	std::vector<unsigned char> blob(total, 0);
	size_t mi = 0;
	for (size_t ci = 0; ci < classes.size(); ++ci) {
		QClass &c = classes[ci];
		std::memcpy(blob.data() + off_kidx[ci], kidx[ci].data(), kidx[ci].size() * sizeof(int));
		std::memcpy(blob.data() + off_toff[ci], toff[ci].data(), toff[ci].size() * sizeof(int));
		std::vector<ssfft_cl::QSched> recs(c.sch.size());
		for (size_t k = 0; k < c.sch.size(); ++k, ++mi) {
			recs[k].tw = base + off_tw[mi];
			recs[k].roots = base + off_roots[mi];
			recs[k].n = (long long)c.sch[k].n;
			recs[k].threads = (long long)c.sch[k].threads;
			for (size_t i = 0; i < tw_all[mi].size(); ++i) {
				if (sb == 4) reinterpret_cast<float *>(blob.data() + off_tw[mi])[i] = (float)tw_all[mi][i];
				else reinterpret_cast<double *>(blob.data() + off_tw[mi])[i] = tw_all[mi][i];
			}
			for (size_t i = 0; i < roots_all[mi].size(); ++i) {
				if (sb == 4) reinterpret_cast<float *>(blob.data() + off_roots[mi])[i] = (float)roots_all[mi][i];
				else reinterpret_cast<double *>(blob.data() + off_roots[mi])[i] = roots_all[mi][i];
			}
		}
		std::memcpy(blob.data() + off_sch[ci], recs.data(), recs.size() * sizeof(ssfft_cl::QSched));
		c.d_kidx = reinterpret_cast<const int *>(base + off_kidx[ci]);
		c.d_toff = reinterpret_cast<const int *>(base + off_toff[ci]);
		c.d_sch = reinterpret_cast<ssfft_cl::QSched *>(base + off_sch[ci]);
		// L2 prefetch one wave of resident CTAs ahead, as the batch kernel does
		int sms = 0;
		cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
		const long long resident = (long long)std::min(jit_occupancy(c.fwd, c.cta, c.smem),
		                                                jit_occupancy(c.inv, c.cta, c.smem)) * std::max(1, sms);
		c.pf_dist = debug_knob("prefetch", 1) == 0 ? 0 : resident;
	}
	e = cudaMemcpy(d_queue, blob.data(), total, cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(multi queue)");
	return SSFFT_SUCCESS;
}

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
	// per-size plans, compiled concurrently; they run offset-table launches, which the staged
	// (bulk-copy) kernels do not take, so none stages
	ssfft_plan_options po;
	if (opt) po = *opt;
	else std::memset(&po, 0, sizeof po);
	po.staging = -1;
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
				if (ssfft_plan_create_ex(&g.plan, g.n, mp->dtype, SSFFT_COMPLEX, g.count, &po) != SSFFT_SUCCESS) bad = 1;
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
	// the work-item queue (default), except for the tensor-core precision option (per-size
	// tcgen05 kernels), the debug switch multi_mode=1 (per-size launches) and batches of 2^31
	// complex elements or more (the queue's offsets are 32-bit element counts)
	m->queue_mode = debug_knob("multi_mode", 0) != 1 && !(opt && opt->precision == SSFFT_PRECISION_SPLIT_BF16) &&
	                m->total < ((size_t)1 << 31);
	if (m->queue_mode) {
		m->queue_max_n = (size_t)std::max(0ll, debug_knob("queue_max_n", (long long)kQueueMaxN));
		std::vector<std::vector<long long>> elem_offs;
		for (const Group &g : m->groups) {
			std::vector<long long> v;
			for (long long sc : by_size[g.n]) v.push_back(sc / 2);
			elem_offs.push_back(std::move(v));
		}
		ssfft_status st = m->build_queue(elem_offs);
		if (st != SSFFT_SUCCESS) return st;
		// graph branches: the class launches and the long sizes' launches, largest work first, each on
		// the least loaded of up to 32 branches
		std::vector<std::pair<double, long long>> jobs;  // (work, class index or -1 - group index)
		for (size_t i = 0; i < m->classes.size(); ++i) jobs.emplace_back(m->classes[i].work, (long long)i);
		for (size_t gi : m->big) jobs.emplace_back(m->groups[gi].work, -1 - (long long)gi);
		std::stable_sort(jobs.begin(), jobs.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
		m->branches = (int)std::min<size_t>(kMaxBranches, std::max<size_t>(1, jobs.size()));
		double bload[kMaxBranches] = {};
		for (const auto &j : jobs) {
			int bb = 0;
			for (int q = 1; q < m->branches; ++q)
				if (bload[q] < bload[bb]) bb = q;
			bload[bb] += j.first;
			if (j.second >= 0) m->classes[(size_t)j.second].branch = bb;
			else m->groups[(size_t)(-1 - j.second)].branch = bb;
		}
	}
	const int nbr = m->branches;
	e = cudaStreamCreateWithFlags(&m->cap, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaEventCreateWithFlags(&m->fork, cudaEventDisableTiming);
	for (int b = 0; b < nbr && e == cudaSuccess; ++b) {
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

size_t ssfft_multi_launches(ssfft_multi_t multi) {
	if (!multi) return 0;
	const MultiPlan *m = reinterpret_cast<const MultiPlan *>(multi);
	return m->queue_mode ? m->classes.size() + m->big.size() : m->groups.size();
}

ssfft_status ssfft_multi_destroy(ssfft_multi_t multi) {
	if (!multi) return SSFFT_ERR_INVALID_VALUE;
	delete reinterpret_cast<MultiPlan *>(multi);
	return SSFFT_SUCCESS;
}

}  // extern "C"

// ---------------------------------------------------------------- diagnostics (no GPU)

namespace {

// Distinct sizes of an uneven list as ssfft_multi_create groups them: (n, count, work), sorted by
// work, largest first (the order the library keeps its groups in).
ssfft_status multi_groups(const size_t *sizes, size_t count, ssfft_dtype dtype,
                          std::vector<std::tuple<size_t, size_t, double>> &out) {
	if (!sizes || count == 0 || (dtype != SSFFT_F32 && dtype != SSFFT_F64)) return SSFFT_ERR_INVALID_VALUE;
	const size_t max_n = dtype == SSFFT_F32 ? (size_t)kMaxSubTransform : (size_t)kMaxSubTransform / 2;
	std::map<size_t, size_t> cnt;
	for (size_t i = 0; i < count; ++i) {
		if (sizes[i] == 0 || sizes[i] > max_n) return SSFFT_ERR_UNSUPPORTED;
		++cnt[sizes[i]];
	}
	out.clear();
	for (auto &kv : cnt)
		out.emplace_back(kv.first, kv.second,
		                 (double)kv.second * (double)kv.first * std::log2((double)std::max<size_t>(kv.first, 2)));
	std::stable_sort(out.begin(), out.end(), [](const auto &a, const auto &b) { return std::get<2>(a) > std::get<2>(b); });
	return SSFFT_SUCCESS;
}

}  // namespace

extern "C" ssfft_status ssfft_diag_multi_spec(const size_t *sizes, size_t count, ssfft_dtype dtype, char *json,
                                              size_t json_len, void *blob, size_t *blob_bytes) {
	std::vector<std::tuple<size_t, size_t, double>> g0, g;
	ssfft_status st = multi_groups(sizes, count, dtype, g0);
	if (st != SSFFT_SUCCESS) return st;
	// sizes above queue_max_n run as their own launches (as ssfft_multi_create does)
	const size_t qmax = (size_t)std::max(0ll, debug_knob("queue_max_n", (long long)kQueueMaxN));
	std::string own = "[";
	for (auto &x : g0) {
		if (std::get<0>(x) <= qmax) g.push_back(x);
		else own += (own.size() > 1 ? ", " : "") + std::to_string(std::get<0>(x));
	}
	own += "]";
	std::vector<QClass> classes;
	st = form_classes(dtype, g, classes);
	if (st != SSFFT_SUCCESS) return st;
	std::vector<size_t> counts;
	for (auto &x : g) counts.push_back(std::get<1>(x));
	// element offsets of every size's transforms, in list order (the caller's layout)
	std::vector<std::vector<long long>> elem_offs(g.size());
	{
		std::map<size_t, size_t> gi;
		for (size_t i = 0; i < g.size(); ++i) gi[std::get<0>(g[i])] = i;
		long long off = 0;
		for (size_t i = 0; i < count; ++i) {
			auto it = gi.find(sizes[i]);
			if (it != gi.end()) elem_offs[it->second].push_back(off);
			off += (long long)sizes[i];
		}
		if (off >= (1ll << 31)) return SSFFT_ERR_UNSUPPORTED;
	}
	// blob: FP64 tables of every member, then per class the int32 member indices and per-thread
	// offsets (8-byte aligned)
	std::vector<double> tab;
	std::string js = "{\"classes\": [";
	std::vector<std::vector<int>> kidx(classes.size()), toff(classes.size());
	for (size_t ci = 0; ci < classes.size(); ++ci) {
		const QClass &c = classes[ci];
		std::vector<QueueItem> items;
		class_items(c, counts, items);
		class_tables(c, items, elem_offs, kidx[ci], toff[ci]);
		js += ci ? ", " : "";
		js += "{\"fwd\": \"" + c.name(false) + "\", \"inv\": \"" + c.name(true) + "\", \"cta\": " + std::to_string(c.cta) +
		      ", \"smem\": " + std::to_string(c.smem) + ", \"minb\": " + std::to_string(c.minb) +
		      ", \"emax\": " + std::to_string(c.emax) + ", \"nitems\": " + std::to_string(items.size()) +
		      ", \"members\": [";
		for (size_t k = 0; k < c.sch.size(); ++k) {
			std::vector<double> tw, roots;
			schedule_twiddles(c.sch[k], tw, roots);
			js += k ? ", " : "";
			js += "{\"n\": " + std::to_string(c.sch[k].n) + ", \"per_cta\": " + std::to_string(c.sch[k].per_cta) +
			      ", \"threads\": " + std::to_string(c.sch[k].threads) + ", \"tw\": [" + std::to_string(tab.size()) +
			      ", " + std::to_string(tw.size()) + "]";
			tab.insert(tab.end(), tw.begin(), tw.end());
			js += ", \"roots\": [" + std::to_string(tab.size()) + ", " + std::to_string(roots.size()) + "]}";
			tab.insert(tab.end(), roots.begin(), roots.end());
		}
		js += "], \"items\": [";
		for (size_t i = 0; i < items.size(); ++i)
			js += (i ? ", [" : "[") + std::to_string(items[i].k) + ", " + std::to_string(items[i].count) + ", " +
			      std::to_string(items[i].first) + "]";
		js += "]}";
	}
	size_t pos = tab.size() * sizeof(double);
	std::string tjs = ", \"tables\": [";
	for (size_t ci = 0; ci < classes.size(); ++ci) {
		tjs += (ci ? ", [" : "[") + std::to_string(pos) + ", ";
		pos += kidx[ci].size() * sizeof(int);
		pos = (pos + 7) / 8 * 8;
		tjs += std::to_string(pos) + "]";
		pos += toff[ci].size() * sizeof(int);
		pos = (pos + 7) / 8 * 8;
	}
	js += "]" + tjs + "], \"own_launch\": " + own + "}";
	if (blob_bytes) {
		if (blob && *blob_bytes >= pos) {
			unsigned char *b = static_cast<unsigned char *>(blob);
			std::memset(b, 0, pos);
			std::memcpy(b, tab.data(), tab.size() * sizeof(double));
			size_t q = tab.size() * sizeof(double);
			for (size_t ci = 0; ci < classes.size(); ++ci) {
				std::memcpy(b + q, kidx[ci].data(), kidx[ci].size() * sizeof(int));
				q = (q + kidx[ci].size() * sizeof(int) + 7) / 8 * 8;
				std::memcpy(b + q, toff[ci].data(), toff[ci].size() * sizeof(int));
				q = (q + toff[ci].size() * sizeof(int) + 7) / 8 * 8;
			}
		}
		*blob_bytes = pos;
	}
	if (json && json_len) {
		if (js.size() + 1 > json_len) return SSFFT_ERR_INVALID_SIZE;
		std::memcpy(json, js.c_str(), js.size() + 1);
	}
	return SSFFT_SUCCESS;
}

extern "C" ssfft_status ssfft_diag_multi_jit_check(const size_t *sizes, size_t count, ssfft_dtype dtype,
                                                   const char *arch, size_t *image_bytes) {
	std::vector<std::tuple<size_t, size_t, double>> g0, g;
	ssfft_status st = multi_groups(sizes, count, dtype, g0);
	if (st != SSFFT_SUCCESS) return st;
	const size_t qmax = (size_t)std::max(0ll, debug_knob("queue_max_n", (long long)kQueueMaxN));
	for (auto &x : g0)
		if (std::get<0>(x) <= qmax) g.push_back(x);
	std::vector<QClass> classes;
	st = form_classes(dtype, g, classes);
	if (st != SSFFT_SUCCESS) return st;
	size_t total = 0;
	for (const QClass &c : classes) {
		size_t b = 0;
		st = jit_compile_only({c.name(false), c.name(true)}, arch ? arch : "sm_103a", &b);
		if (st != SSFFT_SUCCESS) return st;
		total += b;
	}
	if (image_bytes) *image_bytes = total;
	return SSFFT_SUCCESS;
}

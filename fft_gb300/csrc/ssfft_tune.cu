// ssfft_tune.cu -- autotuner for single-CTA plans.
//
// The planner's defaults (radix order, ~128 threads per CTA, 16 complex values per thread) were
// measured on the headline sizes; other sizes and batch counts can prefer other shapes.  When a
// plan asks for it, the tuner times candidate schedules on the plan's own batch (zero-filled
// scratch buffers, CUDA events on a private stream) by coordinate descent:
//   level 2: radix order (the planner's list, its permutations, the alternative grouping);
//   level 1 and 2: values per thread {8, 16, 32}, then CTA size {32, 64, 128, 256, 512};
//   level 2: L2 prefetch distance (1/2, 1, 2 waves of resident CTAs), then register caps
//   (launch bounds for at most 128 ... 40 registers a thread, as shared memory allows);
//   a default two-CTA cluster schedule is first timed against the one-CTA schedules.
// Every candidate runs in both directions; the stages follow the joint (forward + inverse)
// time, and the plan takes the fastest forward and the fastest inverse candidate seen.
// Candidates of one stage compile concurrently (NVRTC), and are timed one at a time under a
// process-wide lock so concurrent plan creations do not disturb each other's timings.  The
// winner is cached per (device name, kernel source, n, dtype, kind, batch range, level) in memory
// and in a text file under the kernel cache directory.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <limits>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

#include "ssfft_host.h"

namespace ssfft {

namespace {

std::mutex g_cache_mu;      // in-memory and on-disk results
std::mutex g_time_mu;       // one candidate timed at a time in the process
std::map<std::string, Knobs> g_cache;
bool g_loaded = false;

std::string cache_file() {
	char h[32];
	std::snprintf(h, sizeof h, "%016llx", (unsigned long long)codelet_hash());
	return jit_cache_dir() + "/tune-" + h + ".txt";
}

// "r=16.8.15 c=128 e=16 m=1"
std::string encode(const Knobs &k) {
	std::string r = "r=";
	for (size_t i = 0; i < k.radices.size(); ++i) r += (i ? "." : "") + std::to_string(k.radices[i]);
	r += " c=" + std::to_string(k.cta_threads) + " e=" + std::to_string(k.emax) + " m=" + std::to_string(k.minb) +
	     " p=" + std::to_string(k.precision) + " f=" + std::to_string(k.prefetch) + " s=" + std::to_string(k.pair);
	return r;
}

bool decode(const std::string &txt, Knobs &k) {
	k = Knobs();
	std::stringstream ss(txt);
	std::string tok;
	while (ss >> tok) {
		if (tok.size() < 2 || tok[1] != '=') return false;
		const std::string v = tok.substr(2);
		if (tok[0] == 'r') {
			std::stringstream rs(v);
			std::string part;
			while (std::getline(rs, part, '.'))
				if (!part.empty()) k.radices.push_back(std::atoi(part.c_str()));
		} else if (tok[0] == 'c') {
			k.cta_threads = std::atoi(v.c_str());
		} else if (tok[0] == 'e') {
			k.emax = std::atoi(v.c_str());
		} else if (tok[0] == 'm') {
			k.minb = std::atoi(v.c_str());
		} else if (tok[0] == 'p') {
			k.precision = std::atoi(v.c_str());
		} else if (tok[0] == 'f') {
			k.prefetch = std::atoi(v.c_str());
		} else if (tok[0] == 's') {
			k.pair = std::atoi(v.c_str());
		}
	}
	return true;
}

void load_locked() {
	if (g_loaded) return;
	g_loaded = true;
	std::string txt;
	if (!cache_read(cache_file(), txt)) return;
	std::stringstream ss(txt);
	std::string line;
	while (std::getline(ss, line)) {
		const size_t tab = line.find('\t');
		if (tab == std::string::npos) continue;
		Knobs k;
		if (decode(line.substr(tab + 1), k)) g_cache[line.substr(0, tab)] = k;
	}
}

void store_locked(const std::string &key, const Knobs &k) {
	g_cache[key] = k;
	std::string txt;
	for (const auto &kv : g_cache) txt += kv.first + "\t" + encode(kv.second) + "\n";
	cache_write(cache_file(), txt);
}

struct Candidate {
	Knobs knobs;
	Schedule sch, sch_inv;  // forward and inverse (RealFFT plans may differ per direction)
	std::vector<CUfunction> fns;
	ssfft_status st = SSFFT_ERR_UNSUPPORTED;
	double fwd_us = 0, inv_us = 0;
	double total() const { return fwd_us + inv_us; }
};

// Scratch of the timing runs: input and output large enough for `tb` transforms either way.
struct Scratch {
	void *in = nullptr, *out = nullptr, *tab = nullptr;
	size_t tab_bytes = 0;
	cudaStream_t stream = nullptr;
	cudaEvent_t ev[2] = {};
	~Scratch() {
		if (in) cudaFree(in);
		if (out) cudaFree(out);
		if (tab) cudaFree(tab);
		for (auto e : ev)
			if (e) cudaEventDestroy(e);
		if (stream) cudaStreamDestroy(stream);
	}
};

void compile_all(const Plan *p, size_t tb, std::vector<Candidate> &cs) {
	std::atomic<size_t> next{0};
	const int nt = (int)std::max<size_t>(1, std::min<size_t>(cs.size(), 4));
	std::vector<std::thread> th;
	const size_t limit = device_smem_limit(p->device);
	for (int t = 0; t < nt; ++t)
		th.emplace_back([&] {
			cudaSetDevice(p->device);
			for (size_t i = next++; i < cs.size(); i = next++) {
				Candidate &c = cs[i];
				if (!single_schedule(p->n, p->dtype, p->kind, tb, c.sch, &c.knobs, 0, 0) ||
				    !single_schedule(p->n, p->dtype, p->kind, tb, c.sch_inv, &c.knobs, 0, 1) ||
				    c.sch.smem_bytes > limit || c.sch_inv.smem_bytes > limit) {
					c.st = SSFFT_ERR_UNSUPPORTED;
					continue;
				}
				c.st = jit_kernels({c.sch.name(false), c.sch_inv.name(true)},
				                   std::max(c.sch.smem_bytes, c.sch_inv.smem_bytes), c.fns);
			}
		});
	for (auto &x : th) x.join();
}

ssfft_status time_dir(const Plan *p, size_t tb, Scratch &sc, Candidate &c, int inv) {
	const Schedule &sch = inv ? c.sch_inv : c.sch;
	std::vector<double> tw, roots, rtw, rot;
	single_tables(sch, p->n, tw, roots, rtw, rot);
	std::vector<float> tcb;
	if (sch.tc) tc_matrix(sch.radices[0], tcb);
	const size_t sb = p->dtype == SSFFT_F32 ? 4 : 8;
	const size_t o_roots = (tw.size() * sb + 255) & ~(size_t)255;
	const size_t o_rtw = (o_roots + roots.size() * sb + 255) & ~(size_t)255;
	const size_t o_rot = (o_rtw + rtw.size() * sb + 255) & ~(size_t)255;
	const size_t o_tcb = (o_rot + rot.size() * sb + 255) & ~(size_t)255;
	const size_t o_err = (o_tcb + tcb.size() * 4 + 255) & ~(size_t)255;
	const size_t total = o_err + 256;
	std::vector<unsigned char> blob(total, 0);
	auto put = [&](size_t off, const std::vector<double> &v) {
		for (size_t i = 0; i < v.size(); ++i) {
			if (sb == 4) {
				const float f = (float)v[i];
				std::memcpy(blob.data() + off + i * 4, &f, 4);
			} else {
				std::memcpy(blob.data() + off + i * 8, &v[i], 8);
			}
		}
	};
	put(0, tw);
	put(o_roots, roots);
	put(o_rtw, rtw);
	put(o_rot, rot);
	if (!tcb.empty()) std::memcpy(blob.data() + o_tcb, tcb.data(), tcb.size() * 4);
	if (total > sc.tab_bytes) {
		if (sc.tab) cudaFree(sc.tab);
		sc.tab = nullptr;
		sc.tab_bytes = 0;
		cudaError_t e = cudaMalloc(&sc.tab, total);
		if (e != cudaSuccess) return cuda_fail(e, "tune tables");
		sc.tab_bytes = total;
	}
	cudaError_t e = cudaMemcpy(sc.tab, blob.data(), total, cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return cuda_fail(e, "tune tables copy");
	const unsigned char *base = static_cast<const unsigned char *>(sc.tab);
	const long long grid = sch.grid((long long)tb);
	{
		ssfft_cl::Args a;
		std::memset(&a, 0, sizeof a);
		a.in = sc.in;
		a.out = sc.out;
		a.batch = (long long)tb;
		plan_dists(p, inv, a.in_dist, a.out_dist);
		a.tw = base;
		a.roots = base + o_roots;
		a.rtw = base + o_rtw;
		a.rot = base + o_rot;
		a.tcb = tcb.empty() ? nullptr : reinterpret_cast<const float *>(base + o_tcb);
		a.err = reinterpret_cast<unsigned *>(static_cast<unsigned char *>(sc.tab) + o_err);
		a.spin_limit = 1u << 22;
		CUfunction f = c.fns[inv];
		a.pf_dist = prefetch_distance(sch, c.knobs, resident_ctas(f, f, sch, p->device));
		ssfft_status st = jit_launch(f, (unsigned)grid, (unsigned)sch.cta_threads(), sch.smem_bytes, sc.stream, &a);
		if (st != SSFFT_SUCCESS) return st;
		// repeats scale with the work so that each measurement spans ~0.3 ms or more
		const double work = (double)tb * (double)p->n;
		const int reps = (int)std::min(20.0, std::max(3.0, std::ceil(3e7 / std::max(work, 1.0))));
		cudaEventRecord(sc.ev[0], sc.stream);
		for (int r = 0; r < reps && st == SSFFT_SUCCESS; ++r)
			st = jit_launch(f, (unsigned)grid, (unsigned)sch.cta_threads(), sch.smem_bytes, sc.stream, &a);
		cudaEventRecord(sc.ev[1], sc.stream);
		if (st != SSFFT_SUCCESS) return st;
		e = cudaEventSynchronize(sc.ev[1]);
		if (e != cudaSuccess) return cuda_fail(e, "tune timing");
		float ms = 0;
		cudaEventElapsedTime(&ms, sc.ev[0], sc.ev[1]);
		(inv ? c.inv_us : c.fwd_us) = 1e3 * ms / reps;
	}
	return SSFFT_SUCCESS;
}

ssfft_status time_one(const Plan *p, size_t tb, Scratch &sc, Candidate &c) {
	for (int inv = 0; inv < 2; ++inv) {
		ssfft_status st = time_dir(p, tb, sc, c, inv);
		if (st != SSFFT_SUCCESS) return st;
	}
	return SSFFT_SUCCESS;
}

}  // namespace

ssfft_status autotune_single(Plan *p, int level, Knobs &best, Knobs &best_inv, std::string &log) {
	best = Knobs();
	best.precision = p->knobs.precision;
	best_inv = best;
	log.clear();
	const bool real = p->kind != SSFFT_COMPLEX;
	const int cn = (int)(real ? p->n / 2 : p->n);
	if (cn < 8) return SSFFT_SUCCESS;  // nothing to choose
	cudaDeviceProp prop;
	cudaError_t e = cudaGetDeviceProperties(&prop, p->device);
	if (e != cudaSuccess) return cuda_fail(e, "cudaGetDeviceProperties");
	int bb = 0;
	while (bb < 40 && ((size_t)1 << (bb + 1)) <= p->batch) ++bb;
	const std::string key = std::string(prop.name) + "|" + std::to_string(p->n) + "|" +
	                        (p->dtype == SSFFT_F32 ? "f32" : "f64") + "|" + std::to_string((int)p->kind) + "|b" +
	                        std::to_string(bb) + "|L" + std::to_string(level) + "|P" +
	                        std::to_string(p->knobs.precision);
	{
		std::lock_guard<std::mutex> lock(g_cache_mu);
		load_locked();
		auto it = g_cache.find(key);
		if (it != g_cache.end()) {
			best = it->second;
			auto ii = g_cache.find(key + "|inverse");
			best_inv = ii != g_cache.end() ? ii->second : best;
			return SSFFT_SUCCESS;
		}
	}
	// timing batch: the plan's batch, capped so each scratch buffer stays within 256 MiB
	const size_t sb = p->dtype == SSFFT_F32 ? 4 : 8;
	const size_t per = (real ? 2 * (size_t)cn + 2 : 2 * (size_t)cn) * sb;
	const size_t tb = std::max<size_t>(1, std::min(p->batch, ((size_t)256 << 20) / per));
	Scratch sc;
	e = cudaMalloc(&sc.in, tb * per);
	if (e == cudaSuccess) e = cudaMalloc(&sc.out, tb * per);
	if (e == cudaSuccess) e = cudaMemset(sc.in, 0, tb * per);
	if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sc.stream, cudaStreamNonBlocking);
	if (e == cudaSuccess) e = cudaEventCreate(&sc.ev[0]);
	if (e == cudaSuccess) e = cudaEventCreate(&sc.ev[1]);
	if (e != cudaSuccess) return cuda_fail(e, "tune scratch");

	// kernel names -> forward and inverse us (identical schedules are timed once)
	std::map<std::string, std::pair<double, double>> timed;
	// every candidate is timed in both directions: besides the joint choice that steers the
	// stages, the fastest forward and the fastest inverse seen are kept (a RealFFT inverse often
	// prefers another register cap or CTA shape than its forward)
	double best_f = 1e300, best_i = 1e300;
	Knobs kf = best, ki = best;
	auto note = [&](const Candidate &c) {
		if (c.fwd_us < best_f) best_f = c.fwd_us, kf = c.knobs;
		if (c.inv_us < best_i) best_i = c.inv_us, ki = c.knobs;
	};
	auto run_stage = [&](std::vector<Candidate> &cs) -> ssfft_status {
		compile_all(p, tb, cs);
		std::lock_guard<std::mutex> lock(g_time_mu);
		for (auto &c : cs) {
			if (c.st != SSFFT_SUCCESS) continue;
			const std::string nm = c.sch.name(false) + "|" + c.sch_inv.name(true) + "|pf" + std::to_string(c.knobs.prefetch);
			auto it = timed.find(nm);
			if (it != timed.end()) {
				c.fwd_us = it->second.first;
				c.inv_us = it->second.second;
				continue;
			}
			ssfft_status st = time_one(p, tb, sc, c);
			if (st != SSFFT_SUCCESS) return st;
			timed[nm] = {c.fwd_us, c.inv_us};
			note(c);
			char line[256];
			std::snprintf(line, sizeof line, "%s threads=%dx%d fwd=%.2fus inv=%.2fus\n", c.knobs.str().c_str(),
			              c.sch.threads, c.sch.per_cta, c.fwd_us, c.inv_us);
			log += line;
		}
		const Candidate *w = nullptr;
		for (auto &c : cs)
			if (c.st == SSFFT_SUCCESS && (!w || c.total() < w->total())) w = &c;
		if (w) best = w->knobs;
		return SSFFT_SUCCESS;
	};

	{
		// a two-CTA cluster default against the single-CTA schedules; if the cluster schedule
		// wins, only its register cap (two or three CTAs per SM) is tuned further
		Schedule d0;
		if (single_schedule(p->n, p->dtype, p->kind, tb, d0, &best, 0) && d0.pair) {
			std::vector<Candidate> cs(2);
			cs[0].knobs = best;
			cs[1].knobs = best;
			cs[1].knobs.pair = 0;
			ssfft_status st = run_stage(cs);
			if (st != SSFFT_SUCCESS) return st;
			if (best.pair != 0) {
				std::vector<Candidate> cm(2);
				cm[0].knobs = best;
				cm[1].knobs = best;
				cm[1].knobs.minb = d0.minb + 1;
				st = run_stage(cm);
				if (st != SSFFT_SUCCESS) return st;
				std::lock_guard<std::mutex> lock(g_cache_mu);
				store_locked(key, kf);
				store_locked(key + "|inverse", ki);
				best = kf;
				best_inv = ki;
				return SSFFT_SUCCESS;
			}
		}
	}
	if (level >= 2) {
		std::vector<std::vector<int>> lists;
		radix_candidates(cn, lists, p->kind == SSFFT_REAL && !(p->n & 1));
		std::vector<Candidate> cs;
		for (auto &l : lists) {
			Candidate c;
			c.knobs = best;
			c.knobs.radices = l;
			cs.push_back(c);
		}
		if (cs.size() > 1) {
			ssfft_status st = run_stage(cs);
			if (st != SSFFT_SUCCESS) return st;
		}
	}
	{
		std::vector<Candidate> cs;
		for (int em : {8, 16, 32}) {
			Candidate c;
			c.knobs = best;
			c.knobs.emax = em;
			cs.push_back(c);
		}
		ssfft_status st = run_stage(cs);
		if (st != SSFFT_SUCCESS) return st;
	}
	{
		std::vector<Candidate> cs;
		for (int ct : {32, 64, 128, 256, 512}) {
			Candidate c;
			c.knobs = best;
			c.knobs.cta_threads = ct;
			cs.push_back(c);
		}
		ssfft_status st = run_stage(cs);
		if (st != SSFFT_SUCCESS) return st;
	}
	if (level >= 2) {
		// L2 prefetch distance: half, one or two waves of resident CTAs ahead
		std::vector<Candidate> cs;
		for (int q : {2, 4, 8}) {
			Candidate c;
			c.knobs = best;
			c.knobs.prefetch = q;
			cs.push_back(c);
		}
		ssfft_status st = run_stage(cs);
		if (st != SSFFT_SUCCESS) return st;
	}
	if (level >= 2) {
		// register caps: enough CTAs per SM for at most 128 ... 40 registers a thread (more CTAs
		// in flight overlap one CTA's HBM phase with another's arithmetic, if the caps do not
		// force spills), as far as shared memory and the SM's 2048 threads allow
		Schedule cur;
		if (single_schedule(p->n, p->dtype, p->kind, tb, cur, &best, 0)) {
			std::vector<Candidate> cs;
			const int by_smem = cur.smem_bytes ? (int)((227 * 1024) / cur.smem_bytes) : 32;
			const int by_threads = 2048 / cur.cta_threads();
			std::vector<int> seen{cur.minb};
			for (int regs : {128, 96, 64, 48, 40}) {
				const int m = 65536 / (cur.cta_threads() * regs);
				if (m < 2 || m > 32 || m > by_smem || m > by_threads) continue;
				if (std::find(seen.begin(), seen.end(), m) != seen.end()) continue;
				seen.push_back(m);
				Candidate c;
				c.knobs = best;
				c.knobs.minb = m;
				cs.push_back(c);
			}
			if (!cs.empty()) {
				Candidate keep;
				keep.knobs = best;
				cs.insert(cs.begin(), keep);
				ssfft_status st = run_stage(cs);
				if (st != SSFFT_SUCCESS) return st;
			}
		}
	}
	std::lock_guard<std::mutex> lock(g_cache_mu);
	store_locked(key, kf);
	store_locked(key + "|inverse", ki);
	best = kf;
	best_inv = ki;
	return SSFFT_SUCCESS;
}

}  // namespace ssfft

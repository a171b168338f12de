// ssfft_serve.cu -- request serving with continuous batching (include/ssfft.h, "serving").
//
// The reference transforms one buffer per call on the caller's thread.  A server instead takes
// requests (size, kind, direction, frames, host buffers) from any thread and runs them in waves:
//   * admission: a request's device buffers come from one arena allocated at start-up (the HBM
//     budget); requests wait in FIFO order until their group's buffers fit;
//   * a wave takes up to max_requests_per_wave admitted requests, groups them by
//     (n, dtype, kind, direction), and on its own stream copies each request's input into its
//     group's contiguous device block, runs one batched launch per group, and copies outputs back;
//   * up to max_waves_in_flight waves run at once, so requests arriving while earlier ones are on
//     the GPU are admitted as soon as buffers and a wave slot free up;
//   * a host callback at the end of each wave's stream work marks its requests complete (the
//     latency of a request is completion time minus submit time) and releases its buffers.
// With coalesce = 0 the server runs the plain baseline instead: each request alone, one
// synchronous copy-in / launch / copy-out at a time, which is what a caller looping over
// ssfft_exec_host does.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <random>
#include <thread>
#include <tuple>
#include <vector>

#include "ssfft_host.h"

namespace ssfft {
namespace {

using Clock = std::chrono::steady_clock;

// First-fit allocator over one device allocation (offsets, 256-byte aligned).
class Arena {
	std::map<size_t, size_t> free_;  // offset -> size
public:
	size_t capacity = 0;
	void reset(size_t cap) {
		capacity = cap;
		free_.clear();
		free_[0] = cap;
	}
	bool alloc(size_t bytes, size_t &off) {
		bytes = (bytes + 255) & ~(size_t)255;
		for (auto it = free_.begin(); it != free_.end(); ++it) {
			if (it->second >= bytes) {
				off = it->first;
				const size_t rest = it->second - bytes;
				free_.erase(it);
				if (rest) free_[off + bytes] = rest;
				return true;
			}
		}
		return false;
	}
	void release(size_t off, size_t bytes) {
		bytes = (bytes + 255) & ~(size_t)255;
		auto it = free_.emplace(off, bytes).first;
		auto nx = std::next(it);
		if (nx != free_.end() && it->first + it->second == nx->first) {
			it->second += nx->second;
			free_.erase(nx);
		}
		if (it != free_.begin()) {
			auto pv = std::prev(it);
			if (pv->first + pv->second == it->first) {
				pv->second += it->second;
				free_.erase(it);
			}
		}
	}
};

struct Req {
	ssfft_request r;
	uint64_t id = 0;
	Clock::time_point submitted;
	int state = 0;  // 0 queued, 1 running, 2 done, 3 failed
	size_t in_bytes = 0, out_bytes = 0;
};

struct ShapeKey {
	size_t n;
	int dtype, kind, slot;  // slot: wave slot for multi-pass shapes (they own scratch), else -1
	bool operator<(const ShapeKey &o) const {
		return std::tie(n, dtype, kind, slot) < std::tie(o.n, o.dtype, o.kind, o.slot);
	}
};

// Shapes longer than one CTA holds run multi-pass plans with plan-owned scratch.
// Shapes whose plans hold scratch (multi-pass or Bluestein): one plan per wave slot.  The
// planner's answer is cached per shape (the serving loop asks for every wave).
bool multi_pass(const ssfft_request &r) {
	static std::mutex mu;
	static std::map<std::tuple<size_t, int, int>, bool> memo;
	const auto key = std::make_tuple(r.n, (int)r.dtype, (int)r.kind);
	std::lock_guard<std::mutex> lock(mu);
	auto it = memo.find(key);
	if (it != memo.end()) return it->second;
	const bool mp = !plan_single_cta(r.n, r.dtype, r.kind);
	memo.emplace(key, mp);
	return mp;
}

size_t scalar_bytes(ssfft_dtype dt) { return dt == SSFFT_F32 ? 4 : 8; }

void req_bytes(const ssfft_request &r, size_t &in, size_t &out) {
	const size_t sb = scalar_bytes(r.dtype);
	const size_t c = 2 * r.n, h = 2 * (r.n / 2);
	if (r.kind == SSFFT_COMPLEX) in = out = c * sb * r.frames;
	else if (!r.inverse) in = r.n * sb * r.frames, out = h * sb * r.frames;
	else in = h * sb * r.frames, out = r.n * sb * r.frames;
}

double req_flops(const ssfft_request &r) {
	const double n = (double)r.n;
	return (r.kind == SSFFT_COMPLEX ? 5.0 : 2.5) * n * std::log2(std::max(n, 2.0)) * (double)r.frames;
}

}  // namespace

struct ServerImpl;

struct Wave {
	ServerImpl *srv = nullptr;
	int slot = 0;
	std::vector<Req *> reqs;
	std::vector<std::pair<size_t, size_t>> blocks;  // arena (offset, bytes) to release
	bool failed = false;
};

struct ServerImpl {
	ssfft_server_config cfg{};
	int device = 0;
	unsigned char *arena_base = nullptr;
	Arena arena;
	std::vector<cudaStream_t> streams;
	std::vector<bool> slot_busy;
	std::mutex mu;
	std::condition_variable cv;       // scheduler: new work / resources freed
	std::condition_variable done_cv;  // waiters: completions
	std::deque<Req *> pending;
	std::deque<std::unique_ptr<Req>> all;  // owns requests; ids are indices + base
	uint64_t id_base = 0;
	std::vector<double> lat_us;
	uint64_t n_submitted = 0, n_completed = 0, n_failed = 0, n_waves = 0, n_launches = 0;
	double frames_done = 0, flops_done = 0;
	Clock::time_point first_submit, last_done;
	bool have_first = false;
	bool stop = false;
	int running_waves = 0;
	std::mutex plan_mu;
	std::map<ShapeKey, ssfft_plan_t> plans;
	std::thread worker;

	// Plan of a request shape; multi-pass shapes get one plan per wave slot so that concurrent
	// waves never share scratch.  Compiles outside the lock so shapes build concurrently.
	ssfft_status get_plan(const ssfft_request &r, int slot, ssfft_plan_t &p) {
		const bool mp = multi_pass(r);
		ShapeKey k{r.n, (int)r.dtype, (int)r.kind, mp ? slot : -1};
		{
			std::lock_guard<std::mutex> lock(plan_mu);
			auto it = plans.find(k);
			if (it != plans.end()) {
				p = it->second;
				return SSFFT_SUCCESS;
			}
		}
		// batch capacity: single-CTA plans hold no per-batch memory; multi-pass plans keep their
		// scratch near 32 MiB
		size_t cap = 4096;
		if (mp) {
			const size_t per = (r.kind == SSFFT_COMPLEX ? r.n : r.n / 2) * 2 * scalar_bytes(r.dtype);
			cap = std::max<size_t>(1, std::min<size_t>(cap, (size_t(32) << 20) / per));
		}
		cudaSetDevice(device);
		ssfft_plan_t np = nullptr;
		ssfft_status st = ssfft_plan_create(&np, r.n, r.dtype, r.kind, cap);
		if (st != SSFFT_SUCCESS) return st;
		std::lock_guard<std::mutex> lock(plan_mu);
		auto it = plans.find(k);
		if (it != plans.end()) {
			ssfft_plan_destroy(np);  // another thread built it meanwhile
			p = it->second;
		} else {
			plans[k] = np;
			p = np;
		}
		return SSFFT_SUCCESS;
	}

	void finish_request(Req *q, bool ok, Clock::time_point now) {
		q->state = ok ? 2 : 3;
		if (ok) {
			++n_completed;
			lat_us.push_back(std::chrono::duration<double, std::micro>(now - q->submitted).count());
			frames_done += (double)q->r.frames;
			flops_done += req_flops(q->r);
		} else {
			++n_failed;
		}
		last_done = now;
	}

	static void CUDART_CB on_wave_done(void *p) {
		Wave *w = static_cast<Wave *>(p);
		ServerImpl *s = w->srv;
		const auto now = Clock::now();
		{
			std::lock_guard<std::mutex> lock(s->mu);
			for (Req *q : w->reqs) s->finish_request(q, !w->failed, now);
			for (auto &b : w->blocks) s->arena.release(b.first, b.second);
			s->slot_busy[w->slot] = false;
			--s->running_waves;
		}
		s->cv.notify_all();
		s->done_cv.notify_all();
		delete w;
	}

	// Run one wave on stream slot `slot`.  Called by the scheduler without the lock held.
	void launch_wave(Wave *w) {
		cudaStream_t s = streams[w->slot];
		std::map<std::tuple<size_t, int, int, int>, std::vector<size_t>> groups;  // shape+dir -> req idx
		for (size_t i = 0; i < w->reqs.size(); ++i) {
			const ssfft_request &r = w->reqs[i]->r;
			groups[std::make_tuple(r.n, (int)r.dtype, (int)r.kind, r.inverse)].push_back(i);
		}
		size_t bi = 0;
		for (auto &g : groups) {
			const auto &idx = g.second;
			const size_t in_off = w->blocks[bi].first, out_off = w->blocks[bi + 1].first;
			bi += 2;
			size_t pos_in = 0, pos_out = 0, frames = 0;
			for (size_t i : idx) {
				Req *q = w->reqs[i];
				if (cudaMemcpyAsync(arena_base + in_off + pos_in, q->r.h_in, q->in_bytes, cudaMemcpyHostToDevice, s) !=
				    cudaSuccess)
					w->failed = true;
				pos_in += q->in_bytes;
				frames += q->r.frames;
			}
			const ssfft_request &r0 = w->reqs[idx[0]]->r;
			ssfft_plan_t plan = nullptr;
			if (get_plan(r0, w->slot, plan) != SSFFT_SUCCESS) {
				w->failed = true;
			} else {
				const size_t cap = ssfft_plan_batch(plan);
				const size_t fin = w->reqs[idx[0]]->in_bytes / r0.frames, fout = w->reqs[idx[0]]->out_bytes / r0.frames;
				for (size_t f0 = 0; f0 < frames; f0 += cap) {
					const size_t nb = std::min(cap, frames - f0);
					if (ssfft_exec_batch(plan, r0.inverse, arena_base + in_off + f0 * fin, arena_base + out_off + f0 * fout,
					                     nb, s) != SSFFT_SUCCESS)
						w->failed = true;
					std::lock_guard<std::mutex> lock(mu);
					++n_launches;
				}
			}
			for (size_t i : idx) {
				Req *q = w->reqs[i];
				if (cudaMemcpyAsync(q->r.h_out, arena_base + out_off + pos_out, q->out_bytes, cudaMemcpyDeviceToHost, s) !=
				    cudaSuccess)
					w->failed = true;
				pos_out += q->out_bytes;
			}
		}
		if (cudaLaunchHostFunc(s, on_wave_done, w) != cudaSuccess) {
			// no callback will come: complete synchronously
			cudaStreamSynchronize(s);
			w->failed = true;
			on_wave_done(w);
		}
	}

	// Take admitted requests for one wave (lock held); returns nullptr if nothing fits now.
	Wave *form_wave(int slot) {
		Wave *w = new Wave();
		w->srv = this;
		w->slot = slot;
		const size_t maxr = cfg.coalesce ? (size_t)cfg.max_requests_per_wave : 1;
		// group in arrival order; each group needs one contiguous in and out block
		std::map<std::tuple<size_t, int, int, int>, std::vector<Req *>> groups;
		std::vector<std::tuple<size_t, int, int, int>> order;
		size_t taken = 0;
		while (!pending.empty() && taken < maxr) {
			Req *q = pending.front();
			auto key = std::make_tuple(q->r.n, (int)q->r.dtype, (int)q->r.kind, q->r.inverse);
			if (!groups.count(key)) order.push_back(key);
			groups[key].push_back(q);
			pending.pop_front();
			++taken;
		}
		// allocate per group; groups that do not fit go back to the front, in order
		std::vector<Req *> back;
		for (auto &key : order) {
			auto &v = groups[key];
			size_t bin = 0, bout = 0;
			for (Req *q : v) bin += q->in_bytes, bout += q->out_bytes;
			size_t oi = 0, oo = 0;
			bool ok = arena.alloc(bin, oi);
			if (ok && !arena.alloc(bout, oo)) {
				arena.release(oi, bin);
				ok = false;
			}
			if (!ok) {
				back.insert(back.end(), v.begin(), v.end());
				continue;
			}
			w->blocks.push_back({oi, bin});
			w->blocks.push_back({oo, bout});
			for (Req *q : v) {
				q->state = 1;
				w->reqs.push_back(q);
			}
		}
		// keep FIFO order for the ones sent back
		std::sort(back.begin(), back.end(), [](Req *a, Req *b) { return a->id < b->id; });
		for (auto it = back.rbegin(); it != back.rend(); ++it) pending.push_front(*it);
		if (w->reqs.empty()) {
			delete w;
			return nullptr;
		}
		// launch_wave walks groups in key order; lay blocks out to match
		std::map<std::tuple<size_t, int, int, int>, std::pair<std::pair<size_t, size_t>, std::pair<size_t, size_t>>> blk;
		std::vector<Req *> ordered;
		size_t bi = 0;
		std::map<std::tuple<size_t, int, int, int>, std::vector<Req *>> placed;
		for (Req *q : w->reqs) placed[std::make_tuple(q->r.n, (int)q->r.dtype, (int)q->r.kind, q->r.inverse)].push_back(q);
		for (auto &key : order) {
			if (!placed.count(key)) continue;
			blk[key] = {w->blocks[bi], w->blocks[bi + 1]};
			bi += 2;
		}
		w->blocks.clear();
		w->reqs.clear();
		for (auto &kv : placed) {
			w->blocks.push_back(blk[kv.first].first);
			w->blocks.push_back(blk[kv.first].second);
			for (Req *q : kv.second) w->reqs.push_back(q);
		}
		return w;
	}

	void run_plain(Req *q) {
		// the baseline: one request, synchronously, on one stream
		cudaStream_t s = streams[0];
		size_t oi = 0, oo = 0;
		bool ok;
		{
			std::lock_guard<std::mutex> lock(mu);
			ok = arena.alloc(q->in_bytes, oi) && arena.alloc(q->out_bytes, oo);
		}
		ssfft_plan_t plan = nullptr;
		ok = ok && get_plan(q->r, 0, plan) == SSFFT_SUCCESS;
		ok = ok && cudaMemcpyAsync(arena_base + oi, q->r.h_in, q->in_bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
		for (size_t f0 = 0; ok && f0 < q->r.frames; f0 += ssfft_plan_batch(plan)) {
			const size_t nb = std::min(ssfft_plan_batch(plan), q->r.frames - f0);
			ok = ssfft_exec_batch(plan, q->r.inverse, arena_base + oi + f0 * (q->in_bytes / q->r.frames),
			                      arena_base + oo + f0 * (q->out_bytes / q->r.frames), nb, s) == SSFFT_SUCCESS;
			++n_launches;
		}
		ok = ok && cudaMemcpyAsync(q->r.h_out, arena_base + oo, q->out_bytes, cudaMemcpyDeviceToHost, s) == cudaSuccess;
		ok = cudaStreamSynchronize(s) == cudaSuccess && ok;
		const auto now = Clock::now();
		std::lock_guard<std::mutex> lock(mu);
		arena.release(oi, q->in_bytes);
		arena.release(oo, q->out_bytes);
		++n_waves;
		finish_request(q, ok, now);
	}

	void loop() {
		cudaSetDevice(device);
		for (;;) {
			Req *plain = nullptr;
			Wave *w = nullptr;
			{
				std::unique_lock<std::mutex> lock(mu);
				for (;;) {
					if (stop && pending.empty()) return;
					if (!pending.empty()) {
						if (!cfg.coalesce) {
							plain = pending.front();
							pending.pop_front();
							plain->state = 1;
							break;
						}
						int slot = -1;
						for (int i = 0; i < (int)slot_busy.size(); ++i)
							if (!slot_busy[i]) {
								slot = i;
								break;
							}
						if (slot >= 0) {
							w = form_wave(slot);
							if (w) {
								slot_busy[slot] = true;
								++running_waves;
								++n_waves;
								break;
							}
						}
					}
					cv.wait_for(lock, std::chrono::milliseconds(50));
				}
			}
			if (plain) {
				run_plain(plain);
				done_cv.notify_all();
			} else if (w) {
				launch_wave(w);
			}
		}
	}
};

}  // namespace ssfft

using namespace ssfft;

extern "C" {

ssfft_status ssfft_server_create(ssfft_server_t *out, const ssfft_server_config *cfg) {
	if (!out) return SSFFT_ERR_INVALID_VALUE;
	*out = nullptr;
	std::unique_ptr<ServerImpl> s(new ServerImpl());
	if (cfg) s->cfg = *cfg;
	if (!s->cfg.hbm_budget_bytes) s->cfg.hbm_budget_bytes = (size_t)1 << 30;
	if (s->cfg.max_waves_in_flight <= 0) s->cfg.max_waves_in_flight = 4;
	if (s->cfg.max_requests_per_wave <= 0) s->cfg.max_requests_per_wave = 256;
	cudaError_t e = cudaGetDevice(&s->device);
	if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
	void *base = nullptr;
	e = cudaMalloc(&base, s->cfg.hbm_budget_bytes);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(server arena)");
	s->arena_base = static_cast<unsigned char *>(base);
	s->arena.reset(s->cfg.hbm_budget_bytes);
	const int nstreams = s->cfg.coalesce ? s->cfg.max_waves_in_flight : 1;
	for (int i = 0; i < nstreams; ++i) {
		cudaStream_t st;
		e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
		if (e != cudaSuccess) {
			for (auto x : s->streams) cudaStreamDestroy(x);
			cudaFree(base);
			return cuda_fail(e, "cudaStreamCreate(server)");
		}
		s->streams.push_back(st);
	}
	s->slot_busy.assign(nstreams, false);
	ServerImpl *raw = s.get();
	s->worker = std::thread([raw] { raw->loop(); });
	*out = reinterpret_cast<ssfft_server_t>(s.release());
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_server_prepare(ssfft_server_t srv, size_t n, ssfft_dtype dtype, ssfft_kind kind) {
	if (!srv) return SSFFT_ERR_INVALID_VALUE;
	ServerImpl *s = reinterpret_cast<ServerImpl *>(srv);
	ssfft_request r{};
	r.n = n;
	r.dtype = dtype;
	r.kind = kind;
	r.frames = 1;
	ssfft_plan_t p = nullptr;
	const int slots = multi_pass(r) ? (int)s->streams.size() : 1;
	for (int i = 0; i < slots; ++i) {
		ssfft_status st = s->get_plan(r, i, p);
		if (st != SSFFT_SUCCESS) return st;
	}
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_server_submit(ssfft_server_t srv, const ssfft_request *req, uint64_t *ticket) {
	if (!srv || !req || !req->h_in || !req->h_out || req->frames == 0 || req->n == 0) return SSFFT_ERR_INVALID_VALUE;
	if (req->kind != SSFFT_COMPLEX && req->n < 2) return SSFFT_ERR_INVALID_SIZE;
	ServerImpl *s = reinterpret_cast<ServerImpl *>(srv);
	std::unique_ptr<Req> q(new Req());
	q->r = *req;
	req_bytes(q->r, q->in_bytes, q->out_bytes);
	if (q->in_bytes + q->out_bytes + 512 > s->cfg.hbm_budget_bytes) return SSFFT_ERR_BUDGET;
	q->submitted = Clock::now();
	{
		std::lock_guard<std::mutex> lock(s->mu);
		if (s->stop) return SSFFT_ERR_SHUTDOWN;
		q->id = s->id_base + s->all.size();
		if (ticket) *ticket = q->id;
		if (!s->have_first) {
			s->first_submit = q->submitted;
			s->have_first = true;
		}
		++s->n_submitted;
		s->pending.push_back(q.get());
		s->all.push_back(std::move(q));
		// forget finished requests once a million newer ones exist (their tickets expire)
		while (s->all.size() > (size_t(1) << 20) && s->all.front()->state >= 2) {
			s->all.pop_front();
			++s->id_base;
		}
	}
	s->cv.notify_all();
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_server_wait(ssfft_server_t srv, uint64_t ticket, double timeout_seconds) {
	if (!srv) return SSFFT_ERR_INVALID_VALUE;
	ServerImpl *s = reinterpret_cast<ServerImpl *>(srv);
	std::unique_lock<std::mutex> lock(s->mu);
	if (ticket < s->id_base || ticket >= s->id_base + s->all.size()) return SSFFT_ERR_INVALID_VALUE;
	Req *q = s->all[ticket - s->id_base].get();
	const bool ok = s->done_cv.wait_for(lock, std::chrono::duration<double>(timeout_seconds),
	                                    [q] { return q->state >= 2; });
	if (!ok) return SSFFT_ERR_TIMEOUT;
	return q->state == 2 ? SSFFT_SUCCESS : SSFFT_ERR_CUDA;
}

ssfft_status ssfft_server_drain(ssfft_server_t srv, double timeout_seconds) {
	if (!srv) return SSFFT_ERR_INVALID_VALUE;
	ServerImpl *s = reinterpret_cast<ServerImpl *>(srv);
	std::unique_lock<std::mutex> lock(s->mu);
	const bool ok = s->done_cv.wait_for(lock, std::chrono::duration<double>(timeout_seconds), [s] {
		return s->n_completed + s->n_failed == s->n_submitted;
	});
	return ok ? (s->n_failed ? SSFFT_ERR_CUDA : SSFFT_SUCCESS) : SSFFT_ERR_TIMEOUT;
}

ssfft_status ssfft_server_get_stats(ssfft_server_t srv, ssfft_server_stats *st, int reset) {
	if (!srv || !st) return SSFFT_ERR_INVALID_VALUE;
	ServerImpl *s = reinterpret_cast<ServerImpl *>(srv);
	std::lock_guard<std::mutex> lock(s->mu);
	std::memset(st, 0, sizeof *st);
	st->submitted = s->n_submitted;
	st->completed = s->n_completed;
	st->failed = s->n_failed;
	st->waves = s->n_waves;
	st->launches = s->n_launches;
	st->frames = s->frames_done;
	st->flops = s->flops_done;
	if (s->have_first && s->n_completed)
		st->span_seconds = std::chrono::duration<double>(s->last_done - s->first_submit).count();
	if (!s->lat_us.empty()) {
		std::vector<double> v = s->lat_us;
		auto pct = [&v](double p) {
			const size_t k = std::min(v.size() - 1, (size_t)std::floor(p * (double)(v.size() - 1) + 0.5));
			std::nth_element(v.begin(), v.begin() + k, v.end());
			return v[k];
		};
		st->p50_latency_us = pct(0.50);
		st->p99_latency_us = pct(0.99);
		double sum = 0, mx = 0;
		for (double x : s->lat_us) sum += x, mx = std::max(mx, x);
		st->mean_latency_us = sum / (double)s->lat_us.size();
		st->max_latency_us = mx;
	}
	if (reset) {
		// keep request records of anything still in flight; forget the statistics
		s->lat_us.clear();
		s->n_submitted -= s->n_completed + s->n_failed;
		s->n_completed = s->n_failed = s->n_waves = s->n_launches = 0;
		s->frames_done = s->flops_done = 0;
		s->have_first = false;
	}
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_server_destroy(ssfft_server_t srv) {
	if (!srv) return SSFFT_ERR_INVALID_VALUE;
	ServerImpl *s = reinterpret_cast<ServerImpl *>(srv);
	{
		std::lock_guard<std::mutex> lock(s->mu);
		s->stop = true;
	}
	s->cv.notify_all();
	if (s->worker.joinable()) s->worker.join();
	// wait (bounded) for waves still on the GPU; their callbacks touch the server
	for (int i = 0; i < 6000; ++i) {
		{
			std::lock_guard<std::mutex> lock(s->mu);
			if (s->running_waves == 0) break;
		}
		std::this_thread::sleep_for(std::chrono::milliseconds(10));
	}
	for (auto st : s->streams) {
		cudaStreamSynchronize(st);
		cudaStreamDestroy(st);
	}
	for (auto &kv : s->plans) ssfft_plan_destroy(kv.second);
	if (s->arena_base) cudaFree(s->arena_base);
	delete s;
	return SSFFT_SUCCESS;
}

// ---------------------------------------------------------------- synthetic load

ssfft_status ssfft_server_loadgen(ssfft_server_t srv, const ssfft_loadgen_config *cfg, ssfft_server_stats *stats) {
	if (!srv || !cfg || cfg->offered_rate <= 0 || cfg->duration_s <= 0) return SSFFT_ERR_INVALID_VALUE;
	ServerImpl *s = reinterpret_cast<ServerImpl *>(srv);
	const size_t nmin = std::max<size_t>(2, cfg->n_min), nmax = std::max(nmin, cfg->n_max);
	const int maxf = cfg->max_frames > 0 ? cfg->max_frames : 64;
	// the 2^a 3^b 5^c sizes in [nmin, nmax]
	std::vector<size_t> sizes;
	for (size_t a = 1; a <= nmax; a *= 2)
		for (size_t b = a; b <= nmax; b *= 3)
			for (size_t c = b; c <= nmax; c *= 5)
				if (c >= nmin) sizes.push_back(c);
	std::sort(sizes.begin(), sizes.end());
	std::mt19937_64 rng(cfg->seed);
	std::uniform_real_distribution<double> u01(0.0, 1.0);
	const double mean_frames = (1.0 + maxf) / 2.0;
	std::exponential_distribution<double> gap(cfg->offered_rate / mean_frames);
	struct Planned {
		double t;
		ssfft_request r;
	};
	std::vector<Planned> plan;
	for (double t = gap(rng); t < cfg->duration_s; t += gap(rng)) {
		Planned p{};
		p.t = t;
		const double lx = std::log((double)sizes.front()) + u01(rng) * (std::log((double)sizes.back()) - std::log((double)sizes.front()));
		size_t n = *std::lower_bound(sizes.begin(), sizes.end(), (size_t)std::ceil(std::exp(lx) - 1e-9));
		const bool real = u01(rng) < cfg->real_fraction;
		// real transforms take even lengths (as the reference's RealFFT requires): the next even size
		if (real && (n & 1)) {
			auto it = std::upper_bound(sizes.begin(), sizes.end(), n);
			while (it != sizes.end() && (*it & 1)) ++it;
			n = it != sizes.end() ? *it : sizes.back() - (sizes.back() & 1);
		}
		p.r.kind = real ? SSFFT_REAL : SSFFT_COMPLEX;
		p.r.dtype = SSFFT_F32;
		p.r.inverse = u01(rng) < 0.5 ? 1 : 0;
		p.r.n = n;
		p.r.frames = 1 + (size_t)(u01(rng) * maxf) % (size_t)maxf;
		plan.push_back(p);
	}
	// pinned host buffers: one input pool of N(0,1) values, one output pool (results unused)
	size_t maxbytes = 0;
	for (auto &p : plan) {
		size_t bi, bo;
		req_bytes(p.r, bi, bo);
		maxbytes = std::max(maxbytes, std::max(bi, bo));
	}
	void *hin = nullptr, *hout = nullptr;
	cudaError_t e = cudaHostAlloc(&hin, std::max<size_t>(maxbytes, 16), cudaHostAllocDefault);
	if (e != cudaSuccess) return cuda_fail(e, "cudaHostAlloc(loadgen in)");
	e = cudaHostAlloc(&hout, std::max<size_t>(maxbytes, 16), cudaHostAllocDefault);
	if (e != cudaSuccess) {
		cudaFreeHost(hin);
		return cuda_fail(e, "cudaHostAlloc(loadgen out)");
	}
	{
		std::normal_distribution<float> nd(0.f, 1.f);
		float *f = static_cast<float *>(hin);
		for (size_t i = 0; i < maxbytes / 4; ++i) f[i] = nd(rng);
	}
	// plans first (distinct shapes, compiled on several threads), so compilation is not measured
	{
		std::map<std::tuple<size_t, int, int>, ssfft_request> shapes;
		for (auto &p : plan) shapes[std::make_tuple(p.r.n, (int)p.r.dtype, (int)p.r.kind)] = p.r;
		std::vector<ssfft_request> todo;
		for (auto &kv : shapes) todo.push_back(kv.second);
		std::atomic<size_t> next{0};
		std::atomic<int> bad{0};
		const int nt = (int)std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
		std::vector<std::thread> th;
		for (int t = 0; t < nt; ++t)
			th.emplace_back([&] {
				for (size_t i = next++; i < todo.size(); i = next++)
					if (ssfft_server_prepare(srv, todo[i].n, todo[i].dtype, todo[i].kind) != SSFFT_SUCCESS) bad = 1;
			});
		for (auto &x : th) x.join();
		if (bad) {
			cudaFreeHost(hin);
			cudaFreeHost(hout);
			return SSFFT_ERR_UNSUPPORTED;
		}
	}
	ssfft_server_drain(srv, 600);
	ssfft_server_stats dummy;
	ssfft_server_get_stats(srv, &dummy, 1);
	const auto t0 = Clock::now();
	ssfft_status st = SSFFT_SUCCESS;
	for (auto &p : plan) {
		const auto due = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(p.t));
		while (Clock::now() < due) {
			const auto left = due - Clock::now();
			if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
		}
		p.r.h_in = hin;
		p.r.h_out = hout;
		uint64_t tk;
		st = ssfft_server_submit(srv, &p.r, &tk);
		if (st != SSFFT_SUCCESS) break;
	}
	ssfft_status dr = ssfft_server_drain(srv, 600);
	if (stats) ssfft_server_get_stats(srv, stats, 0);
	cudaFreeHost(hin);
	cudaFreeHost(hout);
	return st != SSFFT_SUCCESS ? st : dr;
}

}  // extern "C"

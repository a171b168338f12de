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
//   * an event recorded after each wave's stream work is polled by a completion thread, which
//     marks the wave's requests complete (the latency of a request is completion time minus
//     submit time) and releases its buffers.
// Requests whose host buffers are page-locked and mapped (cudaHostAlloc / cudaHostRegister; the
// GPU reaches them over the host link) and whose shape runs in one CTA are served in place: the
// wave uploads one table of every transform's input and output offsets, and one launch per
// group reads the inputs from and writes the outputs to the callers' buffers directly, so a
// request costs no copy call and no arena space.  Other requests take the copy path above.
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
	bool zc = false;  // served in place from mapped host buffers (no copies, no arena)
};

// Whether [p, p + bytes) is page-locked host memory mapped into the device's address space at the
// same address (the GPU can load and store it directly).
bool host_mapped(const void *p, size_t bytes) {
	if (!p || !bytes) return false;
	cudaPointerAttributes a, b;
	const unsigned char *last = static_cast<const unsigned char *>(p) + bytes - 1;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess || cudaPointerGetAttributes(&b, last) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return a.type == cudaMemoryTypeHost && b.type == cudaMemoryTypeHost && a.devicePointer == p &&
	       b.devicePointer == static_cast<const void *>(last);
}

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

// Requests of one wave with the same (n, dtype, kind, direction, in place): one batched launch.
using GroupKey = std::tuple<size_t, int, int, int, int>;
GroupKey group_key(const Req *q) {
	return GroupKey(q->r.n, (int)q->r.dtype, (int)q->r.kind, q->r.inverse, q->zc ? 1 : 0);
}

struct WaveGroup {
	std::vector<Req *> reqs;
	bool zc = false;
	size_t in_off = 0, out_off = 0, in_bytes = 0, out_bytes = 0;  // copy groups: arena blocks
	size_t frames = 0;
};

struct Wave {
	ServerImpl *srv = nullptr;
	int slot = 0;
	std::vector<WaveGroup> groups;
	bool failed = false;
};

struct ServerImpl {
	ssfft_server_config cfg{};
	int device = 0;
	unsigned char *arena_base = nullptr;
	Arena arena;
	std::vector<cudaStream_t> streams;
	std::vector<bool> slot_busy;
	// per wave slot: pinned host and device tables of the in-place transforms' offsets
	static constexpr size_t kTableBytes = size_t(1) << 20;
	std::vector<long long *> h_tab, d_tab;
	std::mutex mu;
	std::condition_variable cv;       // scheduler: new work / resources freed
	std::condition_variable done_cv;  // waiters: completions
	std::deque<Req *> pending;
	std::deque<std::unique_ptr<Req>> all;  // owns requests; ids are indices + base
	uint64_t id_base = 0;
	std::vector<double> lat_us;
	uint64_t n_submitted = 0, n_completed = 0, n_failed = 0, n_waves = 0, n_launches = 0, n_in_place = 0;
	double frames_done = 0, flops_done = 0;
	Clock::time_point first_submit, last_done;
	bool have_first = false;
	bool stop = false;
	int running_waves = 0;
	std::mutex plan_mu;
	std::map<ShapeKey, ssfft_plan_t> plans;
	std::thread worker;
	// completion: an event per wave slot, polled by the completion thread while waves are in flight
	// (lower latency than a host-function callback; debug switch serve_hostfunc=1 uses callbacks)
	bool hostfunc = false;
	std::vector<cudaEvent_t> slot_event;
	std::mutex fly_mu;
	std::condition_variable fly_cv;
	std::deque<Wave *> in_flight;
	bool fly_stop = false;
	std::thread completer;

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
			if (q->zc) ++n_in_place;
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
			for (WaveGroup &g : w->groups) {
				for (Req *q : g.reqs) s->finish_request(q, !w->failed, now);
				if (!g.zc) {
					s->arena.release(g.in_off, g.in_bytes);
					s->arena.release(g.out_off, g.out_bytes);
				}
			}
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
		// in-place groups: every transform's input and output offset (scalars from the group's first
		// request buffer) in one table, uploaded with one copy
		long long *ht = h_tab[w->slot];
		std::vector<size_t> tab_at(w->groups.size(), 0);
		size_t tpos = 0;
		for (size_t gi = 0; gi < w->groups.size(); ++gi) {
			WaveGroup &g = w->groups[gi];
			if (!g.zc) continue;
			const ssfft_request &r0 = g.reqs[0]->r;
			const size_t sb = scalar_bytes(r0.dtype);
			const long long fin = (long long)(g.reqs[0]->in_bytes / r0.frames / sb);
			const long long fout = (long long)(g.reqs[0]->out_bytes / r0.frames / sb);
			const unsigned char *in0 = static_cast<const unsigned char *>(r0.h_in);
			const unsigned char *out0 = static_cast<const unsigned char *>(r0.h_out);
			tab_at[gi] = tpos;
			size_t k = 0;
			for (Req *q : g.reqs) {
				const long long di = (static_cast<const unsigned char *>(q->r.h_in) - in0) / (long long)sb;
				for (size_t f = 0; f < q->r.frames; ++f) ht[tpos + k++] = di + (long long)f * fin;
			}
			k = 0;
			for (Req *q : g.reqs) {
				const long long dout = (static_cast<unsigned char *>(q->r.h_out) - out0) / (long long)sb;
				for (size_t f = 0; f < q->r.frames; ++f) ht[tpos + g.frames + k++] = dout + (long long)f * fout;
			}
			tpos += 2 * g.frames;
		}
		if (tpos && cudaMemcpyAsync(d_tab[w->slot], ht, tpos * sizeof(long long), cudaMemcpyHostToDevice, s) !=
		                cudaSuccess)
			w->failed = true;
		for (size_t gi = 0; gi < w->groups.size(); ++gi) {
			WaveGroup &g = w->groups[gi];
			const ssfft_request &r0 = g.reqs[0]->r;
			ssfft_plan_t plan = nullptr;
			const bool have_plan = get_plan(r0, w->slot, plan) == SSFFT_SUCCESS;
			if (!have_plan) w->failed = true;
			const size_t cap = have_plan ? ssfft_plan_batch(plan) : 1;
			if (g.zc) {
				const long long *d_in_offs = d_tab[w->slot] + tab_at[gi];
				for (size_t f0 = 0; have_plan && f0 < g.frames; f0 += cap) {
					const size_t nb = std::min(cap, g.frames - f0);
					if (launch_batch_offs(reinterpret_cast<const Plan *>(plan), r0.inverse, r0.h_in, r0.h_out, nb,
					                      d_in_offs + f0, s, d_in_offs + g.frames + f0) != SSFFT_SUCCESS)
						w->failed = true;
					std::lock_guard<std::mutex> lock(mu);
					++n_launches;
				}
				continue;
			}
			size_t pos_in = 0, pos_out = 0;
			for (Req *q : g.reqs) {
				if (cudaMemcpyAsync(arena_base + g.in_off + pos_in, q->r.h_in, q->in_bytes, cudaMemcpyHostToDevice, s) !=
				    cudaSuccess)
					w->failed = true;
				pos_in += q->in_bytes;
			}
			const size_t fin = g.reqs[0]->in_bytes / r0.frames, fout = g.reqs[0]->out_bytes / r0.frames;
			for (size_t f0 = 0; have_plan && f0 < g.frames; f0 += cap) {
				const size_t nb = std::min(cap, g.frames - f0);
				if (ssfft_exec_batch(plan, r0.inverse, arena_base + g.in_off + f0 * fin, arena_base + g.out_off + f0 * fout,
				                     nb, s) != SSFFT_SUCCESS)
					w->failed = true;
				std::lock_guard<std::mutex> lock(mu);
				++n_launches;
			}
			for (Req *q : g.reqs) {
				if (cudaMemcpyAsync(q->r.h_out, arena_base + g.out_off + pos_out, q->out_bytes, cudaMemcpyDeviceToHost, s) !=
				    cudaSuccess)
					w->failed = true;
				pos_out += q->out_bytes;
			}
		}
		if (!hostfunc) {
			if (cudaEventRecord(slot_event[w->slot], s) != cudaSuccess) {
				cudaStreamSynchronize(s);
				w->failed = true;
				on_wave_done(w);
				return;
			}
			{
				std::lock_guard<std::mutex> lock(fly_mu);
				in_flight.push_back(w);
			}
			fly_cv.notify_one();
			return;
		}
		if (cudaLaunchHostFunc(s, on_wave_done, w) != cudaSuccess) {
			// no callback will come: complete synchronously
			cudaStreamSynchronize(s);
			w->failed = true;
			on_wave_done(w);
		}
	}

	// Completion thread: polls the events of the waves in flight (in any order; a slot's event was
	// recorded after its wave's last copy or launch) and completes each wave whose work is done;
	// sleeps when nothing is in flight.
	void complete_loop() {
		cudaSetDevice(device);
		std::vector<Wave *> mine;
		for (;;) {
			{
				std::unique_lock<std::mutex> lock(fly_mu);
				if (mine.empty()) fly_cv.wait(lock, [this] { return fly_stop || !in_flight.empty(); });
				while (!in_flight.empty()) {
					mine.push_back(in_flight.front());
					in_flight.pop_front();
				}
				if (fly_stop && mine.empty()) return;
			}
			bool progress = false;
			for (size_t i = 0; i < mine.size();) {
				const cudaError_t e = cudaEventQuery(slot_event[mine[i]->slot]);
				if (e == cudaErrorNotReady) {
					++i;
					continue;
				}
				Wave *w = mine[i];
				if (e != cudaSuccess) w->failed = true;
				mine.erase(mine.begin() + (long)i);
				on_wave_done(w);
				progress = true;
			}
			if (!progress) std::this_thread::yield();
		}
	}

	// Take admitted requests for one wave (lock held); returns nullptr if nothing fits now.
	Wave *form_wave(int slot) {
		const size_t maxr = cfg.coalesce ? (size_t)cfg.max_requests_per_wave : 1;
		// group in arrival order
		std::map<GroupKey, size_t> index;
		std::vector<WaveGroup> groups;
		std::vector<Req *> back;
		size_t taken = 0, table = 0;
		const size_t table_cap = kTableBytes / sizeof(long long);
		while (!pending.empty() && taken < maxr) {
			Req *q = pending.front();
			pending.pop_front();
			++taken;
			if (q->zc && table + 2 * q->r.frames > table_cap) {
				back.push_back(q);  // the offset table is full: next wave
				continue;
			}
			if (q->zc) table += 2 * q->r.frames;
			auto it = index.find(group_key(q));
			if (it == index.end()) {
				it = index.emplace(group_key(q), groups.size()).first;
				groups.emplace_back();
				groups.back().zc = q->zc;
			}
			WaveGroup &g = groups[it->second];
			g.reqs.push_back(q);
			g.frames += q->r.frames;
			g.in_bytes += q->in_bytes;
			g.out_bytes += q->out_bytes;
		}
		// arena blocks for the copy groups; groups that do not fit go back to the queue
		Wave *w = new Wave();
		w->srv = this;
		w->slot = slot;
		for (WaveGroup &g : groups) {
			if (!g.zc) {
				bool ok = arena.alloc(g.in_bytes, g.in_off);
				if (ok && !arena.alloc(g.out_bytes, g.out_off)) {
					arena.release(g.in_off, g.in_bytes);
					ok = false;
				}
				if (!ok) {
					back.insert(back.end(), g.reqs.begin(), g.reqs.end());
					continue;
				}
			}
			for (Req *q : g.reqs) q->state = 1;
			w->groups.push_back(std::move(g));
		}
		// keep FIFO order for the ones sent back
		std::sort(back.begin(), back.end(), [](Req *a, Req *b) { return a->id < b->id; });
		for (auto it = back.rbegin(); it != back.rend(); ++it) pending.push_front(*it);
		if (w->groups.empty()) {
			delete w;
			return nullptr;
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
	// default 8 waves in flight: measured on GB300 (the bench's Poisson mix), p99 at 1.5 M
	// transforms/s offered 2.4 -> 1.6 ms and at 1.75 M/s 10.5 -> 3.8 ms against 4 waves
	if (s->cfg.max_waves_in_flight <= 0) s->cfg.max_waves_in_flight = 8;
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
	// per-slot offset tables of the in-place groups (batched servers only)
	if (s->cfg.coalesce) {
		for (int i = 0; i < nstreams; ++i) {
			void *h = nullptr, *d = nullptr;
			e = cudaHostAlloc(&h, ServerImpl::kTableBytes, cudaHostAllocDefault);
			if (e == cudaSuccess) e = cudaMalloc(&d, ServerImpl::kTableBytes);
			if (e != cudaSuccess) {
				if (h) cudaFreeHost(h);
				for (size_t k = 0; k < s->h_tab.size(); ++k) {
					cudaFreeHost(s->h_tab[k]);
					cudaFree(s->d_tab[k]);
				}
				for (auto x : s->streams) cudaStreamDestroy(x);
				cudaFree(base);
				return cuda_fail(e, "server offset tables");
			}
			s->h_tab.push_back(static_cast<long long *>(h));
			s->d_tab.push_back(static_cast<long long *>(d));
		}
	}
	s->hostfunc = debug_knob("serve_hostfunc", 0) == 1;
	for (int i = 0; i < nstreams; ++i) {
		cudaEvent_t ev = nullptr;
		e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
		if (e != cudaSuccess) {
			for (auto x : s->slot_event) cudaEventDestroy(x);
			for (size_t k = 0; k < s->h_tab.size(); ++k) {
				cudaFreeHost(s->h_tab[k]);
				cudaFree(s->d_tab[k]);
			}
			for (auto x : s->streams) cudaStreamDestroy(x);
			cudaFree(base);
			return cuda_fail(e, "server events");
		}
		s->slot_event.push_back(ev);
	}
	ServerImpl *raw = s.get();
	s->completer = std::thread([raw] { raw->complete_loop(); });
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
	// in place: batched server, a shape that runs in one CTA, mapped host buffers aligned for the
	// kernel's paired loads and stores, and a table share that fits one wave
	const size_t align = 2 * scalar_bytes(q->r.dtype);
	q->zc = s->cfg.coalesce && debug_knob("serve_inplace", 1) != 0 && !multi_pass(q->r) &&
	        2 * q->r.frames <= ServerImpl::kTableBytes / sizeof(long long) &&
	        (uintptr_t)q->r.h_in % align == 0 && (uintptr_t)q->r.h_out % align == 0 &&
	        host_mapped(q->r.h_in, q->in_bytes) && host_mapped(q->r.h_out, q->out_bytes);
	if (!q->zc && q->in_bytes + q->out_bytes + 512 > s->cfg.hbm_budget_bytes) return SSFFT_ERR_BUDGET;
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
	st->in_place = s->n_in_place;
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
		s->n_completed = s->n_failed = s->n_waves = s->n_launches = s->n_in_place = 0;
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
	{
		std::lock_guard<std::mutex> lock(s->fly_mu);
		s->fly_stop = true;
	}
	s->fly_cv.notify_all();
	if (s->completer.joinable()) s->completer.join();
	for (auto st : s->streams) {
		cudaStreamSynchronize(st);
		cudaStreamDestroy(st);
	}
	for (auto ev : s->slot_event) cudaEventDestroy(ev);
	for (auto &kv : s->plans) ssfft_plan_destroy(kv.second);
	for (size_t k = 0; k < s->h_tab.size(); ++k) {
		cudaFreeHost(s->h_tab[k]);
		cudaFree(s->d_tab[k]);
	}
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

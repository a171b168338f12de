// ssfft_stage.cu -- host-memory execution (ssfft_exec_host) and plan teardown.
//
// ssfft_exec_host is the GB300 form of the reference's host-iterator fft/ifft
// (signalsmith-fft.h:374-386): the caller's host buffers stream through the device in chunks,
// each chunk's host->device copy, transform and device->host copy issued on one of three
// streams so that the two copy directions and the kernels of neighbouring chunks overlap.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdlib>
#include <cstring>

#include "ssfft_host.h"

namespace ssfft {

void plan_release(Plan *p) {
	if (!p) return;
	int prev = -1;
	cudaGetDevice(&prev);
	cudaSetDevice(p->device);
	if (p->stage) {
		HostStage *st = p->stage;
		for (int i = 0; i < HostStage::kStreams; ++i) {
			if (st->stream[i]) cudaStreamSynchronize(st->stream[i]);
			if (st->d_in[i]) cudaFree(st->d_in[i]);
			if (st->d_out[i]) cudaFree(st->d_out[i]);
			if (st->stream[i]) cudaStreamDestroy(st->stream[i]);
		}
		if (st->bounce_in) cudaFreeHost(st->bounce_in);
		if (st->bounce_out) cudaFreeHost(st->bounce_out);
		delete st;
		p->stage = nullptr;
	}
	if (p->large) {
		large_release(p->large);
		p->large = nullptr;
	}
	if (p->d_tables) cudaFree(p->d_tables);
	p->d_tables = nullptr;
	if (prev >= 0) cudaSetDevice(prev);
}

// Chunk of ~32 MiB of input per stream (at least one transform), three streams (measured on
// GB300 with the RealFFT headline frames: 16 MiB 1027-1037, 32-96 MiB 1050-1074 GFLOP/s end to
// end, 4-8 MiB 861-968; a fourth stream no better).  Debug switches, read when a plan first runs
// on host buffers: stage_mb (chunk MiB), stage_streams (1..4).
static ssfft_status stage_init(Plan *p) {
	if (p->stage) return SSFFT_SUCCESS;
	HostStage *st = new HostStage();
	const size_t per_in = std::max(plan_in_bytes(p, 0, 1), plan_in_bytes(p, 1, 1));
	const size_t per_out = std::max(plan_out_bytes(p, 0, 1), plan_out_bytes(p, 1, 1));
	const long long mb_dbg = debug_knob("stage_mb", 32);
	const size_t mb = mb_dbg > 0 ? (size_t)mb_dbg : 32;
	size_t chunk = std::max<size_t>(1, (mb << 20) / std::max<size_t>(per_in, 1));
	chunk = std::min(chunk, p->batch);
	st->chunk = chunk;
	const long long ns_dbg = debug_knob("stage_streams", 3);
	const int ns = ns_dbg > 0 ? (int)std::min<long long>(HostStage::kStreams, ns_dbg) : 3;
	// multi-pass plans share one scratch buffer, so their chunks run on a single stream
	st->streams = p->large ? 1 : ns;
	for (int i = 0; i < st->streams; ++i) {
		cudaError_t e = cudaStreamCreateWithFlags(&st->stream[i], cudaStreamNonBlocking);
		if (e == cudaSuccess) e = cudaMalloc(&st->d_in[i], per_in * chunk);
		if (e == cudaSuccess) e = cudaMalloc(&st->d_out[i], per_out * chunk);
		if (e != cudaSuccess) {
			p->stage = st;  // released with the plan
			return cuda_fail(e, "exec_host staging");
		}
	}
	p->stage_bytes = (size_t)st->streams * (per_in + per_out) * chunk;
	p->stage = st;
	return SSFFT_SUCCESS;
}

}  // namespace ssfft

using namespace ssfft;

// The device address of `bytes` of pinned, device-mapped host memory at `p` (cudaHostAlloc,
// cudaHostRegister), or null if any part of the range is not such memory.
static void *mapped_host(const void *p, size_t bytes) {
	if (!bytes) return nullptr;
	cudaPointerAttributes a, b;
	const unsigned char *last = static_cast<const unsigned char *>(p) + bytes - 1;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess || cudaPointerGetAttributes(&b, last) != cudaSuccess) {
		cudaGetLastError();  // clear the error of a pointer the runtime does not know
		return nullptr;
	}
	if (a.type != cudaMemoryTypeHost || b.type != cudaMemoryTypeHost || !a.devicePointer || !b.devicePointer)
		return nullptr;
	if (static_cast<unsigned char *>(b.devicePointer) - static_cast<unsigned char *>(a.devicePointer) !=
	    (std::ptrdiff_t)(bytes - 1))
		return nullptr;
	return a.devicePointer;
}

// Whether [p, p + bytes) is page-locked host memory the runtime knows (a DMA from it needs no
// staging by the driver).
static bool pinned_host(const void *p, size_t bytes) {
	if (!bytes) return false;
	cudaPointerAttributes a;
	if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	if (a.type != cudaMemoryTypeHost) return false;
	cudaPointerAttributes b;
	const unsigned char *last = static_cast<const unsigned char *>(p) + bytes - 1;
	if (cudaPointerGetAttributes(&b, last) != cudaSuccess) {
		cudaGetLastError();
		return false;
	}
	return b.type == cudaMemoryTypeHost;
}

// Small calls (the whole batch in one chunk, at most kBounceMax bytes each way; e.g. one
// transform per call, the reference's usage pattern): one stream, and pageable buffers go through
// the plan's pinned bounce buffers (a host memcpy, then true asynchronous DMA) instead of the
// driver's synchronous staging of pageable copies.  Debug switch small_host=0 turns it off.
static constexpr size_t kBounceMax = size_t(4) << 20;

static ssfft_status exec_host_small(Plan *p, int inverse, const void *h_in, void *h_out, size_t in_b, size_t out_b) {
	HostStage *sg = p->stage;
	if (!sg->bounce_in) {
		cudaError_t e = cudaHostAlloc(&sg->bounce_in, kBounceMax, cudaHostAllocMapped);
		if (e == cudaSuccess) e = cudaHostAlloc(&sg->bounce_out, kBounceMax, cudaHostAllocMapped);
		if (e != cudaSuccess) return cuda_fail(e, "exec_host bounce buffers");
		sg->bounce_bytes = kBounceMax;
	}
	// one-CTA plans with plain loads and stores (not the bulk-copy staged, tensor-core or cluster
	// kernels) run the kernel on the mapped bounce buffers themselves, over the host link: no copy
	// calls, one launch (debug switch small_zc=0 copies through device buffers instead)
	const Schedule &sch = inverse ? p->main.sch_inv : p->main.sch;
	if (!p->large && !sch.staged && !sch.tc && !sch.pair && debug_knob("small_zc", 1) != 0) {
		void *d_bin = nullptr, *d_bout = nullptr;
		cudaError_t e = cudaHostGetDevicePointer(&d_bin, sg->bounce_in, 0);
		if (e == cudaSuccess) e = cudaHostGetDevicePointer(&d_bout, sg->bounce_out, 0);
		if (e != cudaSuccess) return cuda_fail(e, "exec_host mapped bounce buffers");
		std::memcpy(sg->bounce_in, h_in, in_b);
		cudaStream_t s = sg->stream[0];
		ssfft_status st = launch_batch(p, inverse, d_bin, d_bout, p->batch, s);
		if (st != SSFFT_SUCCESS) return st;
		e = cudaStreamSynchronize(s);
		if (e != cudaSuccess) return cuda_fail(e, "exec_host sync");
		std::memcpy(h_out, sg->bounce_out, out_b);
		return SSFFT_SUCCESS;
	}
	const bool pin_in = pinned_host(h_in, in_b), pin_out = pinned_host(h_out, out_b);
	const void *src = h_in;
	if (!pin_in) {
		std::memcpy(sg->bounce_in, h_in, in_b);
		src = sg->bounce_in;
	}
	void *dst = pin_out ? h_out : sg->bounce_out;
	cudaStream_t s = sg->stream[0];
	cudaError_t e = cudaMemcpyAsync(sg->d_in[0], src, in_b, cudaMemcpyHostToDevice, s);
	if (e != cudaSuccess) return cuda_fail(e, "exec_host H2D");
	ssfft_status st = p->large ? launch_large(p, inverse, sg->d_in[0], sg->d_out[0], p->batch, s)
	                           : launch_batch(p, inverse, sg->d_in[0], sg->d_out[0], p->batch, s);
	if (st != SSFFT_SUCCESS) return st;
	e = cudaMemcpyAsync(dst, sg->d_out[0], out_b, cudaMemcpyDeviceToHost, s);
	if (e != cudaSuccess) return cuda_fail(e, "exec_host D2H");
	e = cudaStreamSynchronize(s);
	if (e != cudaSuccess) return cuda_fail(e, "exec_host sync");
	if (!pin_out) std::memcpy(h_out, sg->bounce_out, out_b);
	return SSFFT_SUCCESS;
}

extern "C" ssfft_status ssfft_exec_host(ssfft_plan_t plan, int inverse, const void *h_in, void *h_out) {
	Plan *p = reinterpret_cast<Plan *>(plan);
	if (!p || !h_in || !h_out) return SSFFT_ERR_INVALID_VALUE;
	std::lock_guard<std::mutex> lock(p->stage_mutex);
	int prev = -1;
	cudaGetDevice(&prev);
	if (prev != p->device) cudaSetDevice(p->device);
	// zero copy (debug switch zero_copy=1): when both buffers are pinned and mapped, the kernel
	// reads and writes them over the host link directly; no staging copies
	if (debug_knob("zero_copy", 0) == 1 && !p->large) {
		const void *d_in = mapped_host(h_in, plan_in_bytes(p, inverse, p->batch));
		void *d_out = mapped_host(h_out, plan_out_bytes(p, inverse, p->batch));
		if (d_in && d_out) {
			ssfft_status st = stage_init(p);
			if (st == SSFFT_SUCCESS) st = launch_batch(p, inverse, d_in, d_out, p->batch, p->stage->stream[0]);
			if (st == SSFFT_SUCCESS) {
				cudaError_t e = cudaStreamSynchronize(p->stage->stream[0]);
				if (e != cudaSuccess) st = cuda_fail(e, "exec_host zero-copy sync");
			}
			if (prev >= 0 && prev != p->device) cudaSetDevice(prev);
			return st;
		}
	}
	ssfft_status st = stage_init(p);
	if (st != SSFFT_SUCCESS) return st;
	HostStage *sg = p->stage;
	const size_t per_in = plan_in_bytes(p, inverse, 1), per_out = plan_out_bytes(p, inverse, 1);
	if (p->batch <= sg->chunk && p->batch * std::max(per_in, per_out) <= kBounceMax &&
	    debug_knob("small_host", 1) != 0) {
		st = exec_host_small(p, inverse, h_in, h_out, p->batch * per_in, p->batch * per_out);
		if (prev >= 0 && prev != p->device) cudaSetDevice(prev);
		return st;
	}
	const unsigned char *src = static_cast<const unsigned char *>(h_in);
	unsigned char *dst = static_cast<unsigned char *>(h_out);
	size_t done = 0;
	int k = 0;
	while (done < p->batch && st == SSFFT_SUCCESS) {
		const size_t b = std::min(sg->chunk, p->batch - done);
		const int i = k % sg->streams;
		cudaStream_t s = sg->stream[i];
		cudaError_t e = cudaMemcpyAsync(sg->d_in[i], src + done * per_in, b * per_in, cudaMemcpyHostToDevice, s);
		if (e != cudaSuccess) {
			st = cuda_fail(e, "exec_host H2D");
			break;
		}
		st = p->large ? launch_large(p, inverse, sg->d_in[i], sg->d_out[i], b, s)
		              : launch_batch(p, inverse, sg->d_in[i], sg->d_out[i], b, s);
		if (st != SSFFT_SUCCESS) break;
		e = cudaMemcpyAsync(dst + done * per_out, sg->d_out[i], b * per_out, cudaMemcpyDeviceToHost, s);
		if (e != cudaSuccess) {
			st = cuda_fail(e, "exec_host D2H");
			break;
		}
		done += b;
		++k;
	}
	for (int i = 0; i < sg->streams; ++i) {
		cudaError_t e = cudaStreamSynchronize(sg->stream[i]);
		if (e != cudaSuccess && st == SSFFT_SUCCESS) st = cuda_fail(e, "exec_host sync");
	}
	if (prev >= 0 && prev != p->device) cudaSetDevice(prev);
	return st;
}

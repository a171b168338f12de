// tests/emu/cuda_emu.h -- host emulation of the CUDA built-ins the codelet kernels use, so that
// fft_gb300/csrc/ssfft_codelets.cuh compiles with g++ and runs on the CPU: one std::thread per
// CUDA thread, std::barrier for __syncthreads, a static array for dynamic shared memory.
// Test infrastructure only (tests/test_emulated_kernels.py); it checks the kernels' index
// arithmetic, butterflies and real split/merge without a GPU.
#pragma once
#include <barrier>
#include <cstddef>
#include <cstdint>
#include <cstring>

#define SSFFT_EMULATION 1
#define __device__
#define __host__
#define __global__
#define __forceinline__ inline
#define __launch_bounds__(...)
#define __cluster_dims__(...)
#define __shared__
#define __align__(x)

struct float2 {
	float x, y;
};
struct double2 {
	double x, y;
};
struct alignas(16) float4 {
	float x, y, z, w;
};
inline float4 make_float4(float x, float y, float z, float w) { return float4{x, y, z, w}; }
inline float2 make_float2(float x, float y) { return float2{x, y}; }
inline double2 make_double2(double x, double y) { return double2{x, y}; }

template <class T>
inline T __ldcs(const T *p) { return *p; }
template <class T>
inline T __ldg(const T *p) { return *p; }
template <class T>
inline void __stcs(T *p, T v) { *p = v; }

struct EmuIdx {
	unsigned x = 0, y = 0, z = 0;
};
extern thread_local EmuIdx threadIdx, blockIdx, gridDim;
extern thread_local std::barrier<> *emu_barrier;
inline void __syncthreads() { emu_barrier->arrive_and_wait(); }

namespace ssfft_cl {
extern unsigned char smem_raw[];
}

// __syncthreads_or / atomicOr for the staged kernels
#include <atomic>
extern std::atomic<int> emu_or_acc;
inline int __syncthreads_or(int pred) {
	if (pred) emu_or_acc.fetch_or(1);
	__syncthreads();
	const int r = emu_or_acc.load();
	__syncthreads();
	if (threadIdx.x == 0) emu_or_acc.store(0);
	__syncthreads();
	return r;
}
inline unsigned atomicOr(unsigned *p, unsigned v) {
	unsigned old = *p;
	*p |= v;
	return old;
}

// ssfft_noalloc.cu -- a complex FP32 transform that allocates no memory when called.
//
// Some callers cannot allocate device memory at the moment they need a transform: a real-time
// audio thread that must not block in the driver's allocator, code running inside a framework
// that owns every device allocation, or a process that has pre-reserved all of HBM.  For them
// ssfft_fft_noalloc_f32 runs a multi-pass transform whose only working memory beyond the
// caller's input and output is the file-scope array below, which the library holds on every GPU
// that loads it until the process exits.
//
// The transform is the multi-pass idea (sub-transforms chained through HBM) in its simplest
// form: one kernel launch per radix-2/3/4/5 Stockham pass, ping-ponging between the caller's
// output and the scratch array, twiddles computed in-kernel with sincospif after an exact
// integer reduction of the angle to the first quadrant.  The kernels are compiled into the
// library (no plan, no run-time compilation, no table upload).
#include <cuda_runtime.h>

#include <mutex>

#include "ssfft_host.h"

namespace ssfft {
namespace {

// Largest transform the scratch array holds: 2^20 complex FP32 points (8 MiB per GPU).
constexpr size_t kNoAllocMaxN = size_t(1) << 20;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) float2 g_noalloc_scratch[kNoAllocMaxN];

std::mutex g_noalloc_mutex;
float2 *g_noalloc_ptr[kNoAllocMaxDevices] = {};

// e^{-2 pi i k / L}, 0 <= k < L: quadrant by integer arithmetic, then sincospif on [0, 1/2).
__device__ __forceinline__ float2 root_f32(unsigned k, unsigned L) {
	const unsigned long long k4 = 4ull * k;
	const unsigned q = (unsigned)(k4 / L);
	const unsigned r = (unsigned)(k4 - (unsigned long long)q * L);
	float s, c;
	sincospif((float)r / (float)(2ull * L), &s, &c);  // angle (pi/2) r / L
	float x, y;                                       // e^{+i theta}, theta = q pi/2 + angle
	switch (q & 3) {
	case 0: x = c; y = s; break;
	case 1: x = -s; y = c; break;
	case 2: x = -c; y = -s; break;
	default: x = s; y = -c; break;
	}
	return make_float2(x, -y);
}

// One radix-R Stockham pass over HBM: butterfly j reads src[j + r n/R], applies
// W_{ns R}^{(j mod ns) r}, runs the R-point DFT and writes dst[(j - j mod ns) R + j mod ns + r ns].
template <int R>
__global__ void __launch_bounds__(256) noalloc_pass(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                                    unsigned n, unsigned ns, int conj_in, int conj_out) {
	const unsigned nb = n / R;
	const unsigned j = blockIdx.x * blockDim.x + threadIdx.x;
	if (j >= nb) return;
	const unsigned m = j % ns;
	float2 v[R];
#pragma unroll
	for (int r = 0; r < R; ++r) {
		float2 x = src[j + r * nb];
		if (conj_in) x.y = -x.y;
		v[r] = x;
	}
	if (ns > 1) {
#pragma unroll
		for (int r = 1; r < R; ++r) v[r] = ssfft_cl::mul(v[r], root_f32(m * r, ns * R));
	}
	ssfft_cl::dft<R>(v);
	const unsigned base = (j - m) * R + m;
#pragma unroll
	for (int r = 0; r < R; ++r) {
		float2 x = v[r];
		if (conj_out) x.y = -x.y;
		dst[base + r * ns] = x;
	}
}

// n == 1: the transform is the identity in both directions.
__global__ void noalloc_copy(const float2 *__restrict__ src, float2 *__restrict__ dst) { dst[0] = src[0]; }

// Radices 4, 2, 3, 5 covering n (their count), or -1 if n has another prime factor.
int noalloc_radices(size_t n, int *rad) {
	int k = 0;
	while (n % 4 == 0) {
		rad[k++] = 4;
		n /= 4;
	}
	while (n % 2 == 0) {
		rad[k++] = 2;
		n /= 2;
	}
	while (n % 3 == 0) {
		rad[k++] = 3;
		n /= 3;
	}
	while (n % 5 == 0) {
		rad[k++] = 5;
		n /= 5;
	}
	return n == 1 ? k : -1;
}

// Device address of the scratch array on the current device (set-up on the first call).
ssfft_status noalloc_scratch(float2 **ptr) {
	int dev = 0;
	cudaError_t e = cudaGetDevice(&dev);
	if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
	if (dev < 0 || dev >= kNoAllocMaxDevices) return SSFFT_ERR_UNSUPPORTED;
	std::lock_guard<std::mutex> lock(g_noalloc_mutex);
	if (!g_noalloc_ptr[dev]) {
		void *p = nullptr;
		e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
		if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(noalloc scratch)");
		// Load every kernel of this entry point now: under CUDA's lazy module loading each one
		// would otherwise be loaded by the first call whose size needs it, which may come later
		// on a time-critical thread or inside a stream capture.
		const void *kernels[] = {(const void *)noalloc_pass<2>, (const void *)noalloc_pass<3>,
		                         (const void *)noalloc_pass<4>, (const void *)noalloc_pass<5>,
		                         (const void *)noalloc_copy};
		for (const void *k : kernels) {
			cudaFuncAttributes fa;
			e = cudaFuncGetAttributes(&fa, k);
			if (e != cudaSuccess) return cuda_fail(e, "cudaFuncGetAttributes(noalloc kernels)");
		}
		g_noalloc_ptr[dev] = static_cast<float2 *>(p);
	}
	*ptr = g_noalloc_ptr[dev];
	return SSFFT_SUCCESS;
}

}  // namespace
}  // namespace ssfft

using namespace ssfft;

extern "C" size_t ssfft_fft_noalloc_max_size(void) { return kNoAllocMaxN; }

extern "C" ssfft_status ssfft_fft_noalloc_f32(const void *d_in, void *d_out, size_t n, int inverse, void *stream) {
	if (!d_in || !d_out) return SSFFT_ERR_INVALID_VALUE;
	if ((uintptr_t)d_in % 8 || (uintptr_t)d_out % 8) return SSFFT_ERR_INVALID_VALUE;
	if (n == 0 || n > kNoAllocMaxN) return SSFFT_ERR_INVALID_SIZE;
	// the buffers must not overlap at all: with an odd number of passes the first pass reads
	// `in` while it writes `out`
	const uintptr_t a0 = (uintptr_t)d_in, b0 = (uintptr_t)d_out, bytes = (uintptr_t)n * sizeof(float2);
	if (a0 < b0 + bytes && b0 < a0 + bytes) return SSFFT_ERR_INVALID_VALUE;
	int rad[64];
	const int P = noalloc_radices(n, rad);
	if (P < 0) return SSFFT_ERR_UNSUPPORTED;
	float2 *scratch = nullptr;
	ssfft_status st = noalloc_scratch(&scratch);
	if (st != SSFFT_SUCCESS) return st;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	const float2 *in = static_cast<const float2 *>(d_in);
	float2 *out = static_cast<float2 *>(d_out);
	if (P == 0) {
		noalloc_copy<<<1, 1, 0, s>>>(in, out);
	} else {
		// ping-pong so that the last pass writes `out`
		const float2 *src = in;
		unsigned ns = 1;
		for (int p = 0; p < P; ++p) {
			float2 *dst = ((P - 1 - p) % 2 == 0) ? out : scratch;
			const int R = rad[p];
			const unsigned nb = (unsigned)(n / R);
			const unsigned grid = (nb + 255) / 256;
			const int ci = inverse && p == 0, co = inverse && p == P - 1;
			switch (R) {
			case 2: noalloc_pass<2><<<grid, 256, 0, s>>>(src, dst, (unsigned)n, ns, ci, co); break;
			case 3: noalloc_pass<3><<<grid, 256, 0, s>>>(src, dst, (unsigned)n, ns, ci, co); break;
			case 4: noalloc_pass<4><<<grid, 256, 0, s>>>(src, dst, (unsigned)n, ns, ci, co); break;
			default: noalloc_pass<5><<<grid, 256, 0, s>>>(src, dst, (unsigned)n, ns, ci, co); break;
			}
			src = dst;
			ns *= (unsigned)R;
		}
	}
	cudaError_t e = cudaGetLastError();
	if (e != cudaSuccess) return cuda_fail(e, "noalloc launch");
	return SSFFT_SUCCESS;
}

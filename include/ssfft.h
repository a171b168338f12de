/*
 * ssfft.h -- C ABI of the GB300 (sm_103a) Signalsmith-FFT transform library, libssfft.so.
 *
 * The reference (Signalsmith FFT, signalsmith-fft.h) is a header-only C++ template library with
 * no FFI of its own.  This header is the drop-in boundary a foreign caller binds instead: every
 * entry point below names the reference interface it replaces (file:line in signalsmith-fft.h).
 * The C++ drop-in front end (include/signalsmith-fft.h in this repository) is written on top of
 * these functions.
 *
 * Conventions (as the reference):
 *   - complex data are interleaved {re, im} pairs of float (SSFFT_F32) or double (SSFFT_F64);
 *   - forward uses e^{-2 pi i nk/N}; the inverse is UNNORMALISED: ifft(fft(x)) == N*x
 *     (signalsmith-fft.h:374-386);
 *   - real transforms (kind SSFFT_REAL / SSFFT_REAL_HALFSHIFT) map n reals to n/2 complex bins;
 *     for SSFFT_REAL bin 0 holds {DC, Nyquist} (signalsmith-fft.h:459-462); the inverse maps n/2
 *     bins back to 2*(n/2) reals scaled by n; only out[0 .. n/2) complex (forward) or
 *     out[0 .. 2*(n/2)) reals (inverse) are written.
 * Differences (documented extensions): errors are reported as status codes (the reference has
 * none); device pointers are accepted; `in` may equal `out` for single-pass sizes.
 *
 * Every function is thread-safe for distinct plans.  One plan must not be executed concurrently
 * from two host threads on two streams that overlap (its device tables are read-only, so this
 * is safe on the device side, but the host-staging entry point ssfft_exec_host shares buffers).
 */
#ifndef SSFFT_H
#define SSFFT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
	SSFFT_SUCCESS = 0,
	SSFFT_ERR_INVALID_SIZE = 1,   /* n == 0, real n < 2, or beyond the supported maximum */
	SSFFT_ERR_INVALID_VALUE = 2,  /* bad enum, NULL pointer, misaligned pointer */
	SSFFT_ERR_CUDA = 3,           /* a CUDA runtime call failed (see ssfft_last_cuda_error) */
	SSFFT_ERR_ALLOC = 4,          /* device or pinned host allocation failed */
	SSFFT_ERR_UNSUPPORTED = 5,    /* combination not implemented on this device */
	SSFFT_ERR_BUDGET = 6,         /* request does not fit the server's HBM budget */
	SSFFT_ERR_TIMEOUT = 7,        /* a bounded wait gave up */
	SSFFT_ERR_NOT_READY = 8,      /* asynchronous result not yet available */
	SSFFT_ERR_SHUTDOWN = 9        /* server is stopping */
} ssfft_status;

typedef enum { SSFFT_F32 = 0, SSFFT_F64 = 1 } ssfft_dtype;

typedef enum {
	SSFFT_COMPLEX = 0,        /* FFT<V>            signalsmith-fft.h:69-387  */
	SSFFT_REAL = 1,           /* RealFFT<V>        signalsmith-fft.h:393-503 */
	SSFFT_REAL_HALFSHIFT = 2  /* ModifiedRealFFT<V> signalsmith-fft.h:505-508 (FFTOptions::halfFreqShift :389-391) */
} ssfft_kind;

typedef struct ssfft_plan_s *ssfft_plan_t;

/* Human-readable name of a status code. */
const char *ssfft_status_string(ssfft_status s);
/* Text of the last CUDA error seen by the calling thread ("" if none). */
const char *ssfft_last_cuda_error(void);

/* ---------------------------------------------------------------- fast-size helpers
 * Bit-exact with the reference, including RealFFT's quirks (sizeMaximum may exceed n, and
 * sizeMinimum may return a non-fast even size). */
size_t ssfft_size_minimum(size_t n);       /* FFT<V>::sizeMinimum      signalsmith-fft.h:327-337 */
size_t ssfft_size_maximum(size_t n);       /* FFT<V>::sizeMaximum      signalsmith-fft.h:338-348 */
size_t ssfft_real_size_minimum(size_t n);  /* RealFFT<V>::sizeMinimum  signalsmith-fft.h:403-405 */
size_t ssfft_real_size_maximum(size_t n);  /* RealFFT<V>::sizeMaximum  signalsmith-fft.h:406-408 */

/* ---------------------------------------------------------------- plans
 * Replaces FFT<V>(size) / setSize (signalsmith-fft.h:350-363, setPlan :139-185) and
 * RealFFT<V>(size) / setSize (signalsmith-fft.h:410-435): factorises n into Stockham radix
 * passes, builds FP64 twiddle tables and uploads them (rounded once to the plan's dtype) to the
 * current CUDA device.  `batch` is the number of transforms one ssfft_exec call processes,
 * stored contiguously (distance n complex for SSFFT_COMPLEX; n reals in / n/2 complex out for
 * real kinds).  Plans are bound to the device that was current at creation. */
ssfft_status ssfft_plan_create(ssfft_plan_t *plan, size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch);
ssfft_status ssfft_plan_destroy(ssfft_plan_t plan);
/* Transform size the plan was created for (FFT::size :370-372 / RealFFT::size :442-444). */
size_t ssfft_plan_size(ssfft_plan_t plan);
/* Plan's batch, and the device bytes its tables and scratch hold. */
size_t ssfft_plan_batch(ssfft_plan_t plan);
size_t ssfft_plan_device_bytes(ssfft_plan_t plan);
/* Describe the schedule: number of device passes, radices of the in-CTA pass list, threads per
 * transform and transforms per CTA.  radices may be NULL; cap is its length. */
ssfft_status ssfft_plan_describe(ssfft_plan_t plan, int *npasses, int *radices, int cap, int *threads_per_transform,
                                 int *transforms_per_cta, int *kernel_launches);

/* ---------------------------------------------------------------- execution
 * Replaces FFT<V>::fft / ifft (signalsmith-fft.h:374-386, run :295-315) and RealFFT<V>::fft /
 * ifft (:446-502) for `batch` transforms at once, with device pointers, asynchronously on
 * `stream` (a cudaStream_t; NULL = legacy default stream).  inverse != 0 selects ifft. */
ssfft_status ssfft_exec(ssfft_plan_t plan, int inverse, const void *d_in, void *d_out, void *stream);
/* As ssfft_exec for the first `batch` (<= plan batch) transforms only. */
ssfft_status ssfft_exec_batch(ssfft_plan_t plan, int inverse, const void *d_in, void *d_out, size_t batch,
                              void *stream);
/* Device-side failure report: the staged kernels bound every wait on their bulk copies; a wait
 * that runs out sets a per-plan flag instead of hanging.  Reads and clears it (synchronises the
 * device); returns SSFFT_ERR_TIMEOUT and *flags != 0 if a launch gave up.  No reference
 * counterpart (the reference reports no errors). */
ssfft_status ssfft_plan_error(ssfft_plan_t plan, unsigned *flags);
/* Host-memory variant of FFT<V>::fft / ifft: `h_in` / `h_out` are host buffers (pinned or
 * pageable).  The batch is cut into chunks whose host->device copy, transform and device->host
 * copy overlap on internal streams; returns when h_out is complete. */
ssfft_status ssfft_exec_host(ssfft_plan_t plan, int inverse, const void *h_in, void *h_out);

/* ---------------------------------------------------------------- allocation-free transform
 * No counterpart in the reference.  For callers that cannot allocate device memory at the moment
 * they need a transform -- a real-time audio callback that must never block inside the CUDA
 * allocator, or an application whose own memory manager owns every byte of device memory -- this
 * computes one complex FP32 transform using only the caller's input and output and a scratch
 * array of 2^20 complex values (8 MiB) that the library keeps on every GPU that loads it, until
 * the process exits.  It creates no plan and calls no allocator.
 *   - n must be 2^a 3^b 5^c and at most ssfft_fft_noalloc_max_size() (= 1048576); larger sizes
 *     return SSFFT_ERR_INVALID_SIZE, other prime factors SSFFT_ERR_UNSUPPORTED;
 *   - d_in and d_out are distinct, 8-byte aligned device buffers of n complex floats; inverse != 0
 *     computes the unnormalised inverse, as ssfft_exec does;
 *   - the first call on each device looks up the scratch array's device address; make that first
 *     call before any stream capture;
 *   - every call uses the same array: calls that can overlap on the GPU (other streams, other
 *     host threads) race, so the caller must serialise them.  Nothing needs clearing between
 *     calls: a call reads only scratch values it wrote itself. */
size_t ssfft_fft_noalloc_max_size(void);
ssfft_status ssfft_fft_noalloc_f32(const void *d_in, void *d_out, size_t n, int inverse, void *stream);

/* ---------------------------------------------------------------- diagnostics
 * Host-only helpers (no GPU needed) that expose the planner's choices; they have no counterpart
 * in the reference.  ssfft_jit_check compiles the kernels of a single-CTA plan for `arch`
 * (e.g. "sm_103a") and returns the image size; ssfft_schedule_name returns the kernel template
 * the plan runs; ssfft_schedule_tables returns its FP64 tables (pass with NULL arrays first to
 * get the counts). */
ssfft_status ssfft_jit_check(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, const char *arch,
                             size_t *image_bytes);
ssfft_status ssfft_schedule_info(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, int *radices, int cap,
                                 int *npasses, int *threads, int *per_cta, size_t *smem_bytes);
ssfft_status ssfft_schedule_name(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, int inverse, char *buf,
                                 size_t cap);
ssfft_status ssfft_schedule_tables(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, double *tw,
                                   size_t *ntw, double *roots, size_t *nroots, double *rtw, size_t *nrtw, double *rot,
                                   size_t *nrot);

#ifdef __cplusplus
}
#endif

#endif /* SSFFT_H */

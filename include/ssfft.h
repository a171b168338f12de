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
/* Opt-in 5-smooth variants.  The reference's helpers above never pick a factor of 5 (their fast
 * remainders are 2^a 3^b with b <= 2, signalsmith-fft.h:317-348); these return the nearest
 * 2^a 3^b 5^c instead, which this library runs as fast (radix-5 butterflies in registers):
 *   ssfft_size_minimum_smooth(n): smallest 2^a 3^b 5^c >= n (0 -> 0; 0 if none fits in size_t);
 *   ssfft_size_maximum_smooth(n): largest 2^a 3^b 5^c <= n (0 -> 0);
 *   ssfft_real_size_minimum_smooth(n): smallest even m >= n with m/2 5-smooth (0 -> 0);
 *   ssfft_real_size_maximum_smooth(n): largest even m <= n with m/2 5-smooth (0 if n < 2). */
size_t ssfft_size_minimum_smooth(size_t n);
size_t ssfft_size_maximum_smooth(size_t n);
size_t ssfft_real_size_minimum_smooth(size_t n);
size_t ssfft_real_size_maximum_smooth(size_t n);

/* ---------------------------------------------------------------- plans
 * Replaces FFT<V>(size) / setSize (signalsmith-fft.h:350-363, setPlan :139-185) and
 * RealFFT<V>(size) / setSize (signalsmith-fft.h:410-435): factorises n into Stockham radix
 * passes, builds FP64 twiddle tables and uploads them (rounded once to the plan's dtype) to the
 * current CUDA device.  `batch` is the number of transforms one ssfft_exec call processes,
 * stored contiguously (distance n complex for SSFFT_COMPLEX; n reals in / n/2 complex out for
 * real kinds).  Plans are bound to the device that was current at creation. */
ssfft_status ssfft_plan_create(ssfft_plan_t *plan, size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch);
ssfft_status ssfft_plan_destroy(ssfft_plan_t plan);
/* Plans created successfully by this process so far (a monotonic count; diagnostics, e.g. to
 * check that a front end reuses its plans).  No reference counterpart. */
size_t ssfft_plans_created(void);

/* Schedule options for ssfft_plan_create_ex (zero-initialise; 0 = planner default).  No reference
 * counterpart: the reference's plan is fixed by its factorisation (setPlan :139-185). */
typedef struct ssfft_plan_options {
    int autotune;          /* 0 off; 1 time candidate CTA shapes and values per thread; 2 also radix
                            * orders.  Results are cached per (device, n, dtype, kind, batch range) in
                            * memory and under $SSFFT_CACHE_DIR.  SSFFT_AUTOTUNE=1|2 sets a default. */
    int cta_threads;       /* target threads per CTA */
    int values_per_thread; /* complex values a thread holds in one pass (<= 32) */
    int min_ctas_per_sm;   /* launch bound (register cap) */
    int radices[24];       /* explicit pass order, 0-terminated; product must equal the complex
                            * length (n, or n/2 for real kinds) */
    int precision;         /* SSFFT_PRECISION_FP32 or SSFFT_PRECISION_SPLIT_BF16 */
    int prefetch_quarter_waves; /* L2 prefetch distance of the batch kernel in quarter waves of
                                 * resident CTAs: 0 = planner default (4: one wave), -1 = off */
    int fuse_split;        /* RealFFT split fused into the last forward / first inverse pass:
                            * 0 planner default (from 256 reals), 1 wherever possible, -1 never */
    int cluster_split;     /* complex FP32 transforms run by a cluster of two CTAs (four-step inside
                            * the cluster, half a transform per CTA): 0 planner default (off),
                            * -1 never, k > 0 with `radices` given: its first k radices are the
                            * first phase (their product n1 and n / n1 both even) */
    int staging;           /* input staged in shared memory by bulk (TMA) copies, persistent CTAs:
                            * 0 planner default (long complex FP32 transforms whose plain kernel
                            * runs one CTA per SM), -1 never, 1 wherever the input fits */
} ssfft_plan_options;
/* SSFFT_PRECISION_SPLIT_BF16 (complex FP32 plans that run in one CTA): the first radix pass
 * (radix <= 16) runs as tensor-core matrix products (tcgen05) on FP32 values split into three
 * BF16 parts, accumulated in FP32; later passes are FP32.  Other plans ignore it. */
enum { SSFFT_PRECISION_FP32 = 0, SSFFT_PRECISION_SPLIT_BF16 = 1 };
/* ssfft_plan_create with options (options may be NULL).  Options apply to transforms that run in
 * one CTA; longer ones use the multi-pass schedule regardless. */
ssfft_status ssfft_plan_create_ex(ssfft_plan_t *plan, size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch,
                                  const ssfft_plan_options *options);
/* The schedule options in force ("radices=16.8.15 cta=128 emax=16 minb=1", 0 = default) and the
 * autotuner's timings of the candidates it measured for this plan (one line each; empty when
 * the choice came from the cache).  Text is truncated to len-1 bytes. */
ssfft_status ssfft_plan_tuning(ssfft_plan_t plan, char *choice, size_t choice_len, char *log, size_t log_len);
/* Transform size the plan was created for (FFT::size :370-372 / RealFFT::size :442-444). */
size_t ssfft_plan_size(ssfft_plan_t plan);
/* Plan's batch, and the device bytes its tables and scratch hold. */
size_t ssfft_plan_batch(ssfft_plan_t plan);
size_t ssfft_plan_device_bytes(ssfft_plan_t plan);
/* Describe the schedule: number of device passes, radices of the in-CTA pass list, threads per
 * transform and transforms per CTA.  radices may be NULL; cap is its length. */
ssfft_status ssfft_plan_describe(ssfft_plan_t plan, int *npasses, int *radices, int cap, int *threads_per_transform,
                                 int *transforms_per_cta, int *kernel_launches);
/* The kernel template a single-CTA plan launches in direction `inverse` (text truncated to
 * len-1 bytes; "multi-pass" for plans beyond one CTA).  No reference counterpart. */
ssfft_status ssfft_plan_kernel(ssfft_plan_t plan, int inverse, char *name, size_t len);

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

/* ---------------------------------------------------------------- uneven-size batches
 * No single reference counterpart (the reference's FFT object has one size; a caller with many
 * sizes loops over objects).  `count` independent complex transforms of sizes sizes[i] (each at
 * most 16384 points FP32 / 8192 FP64), stored back to back: transform i starts at the sum of the
 * sizes before it (complex elements).  ssfft_multi_exec runs them all as one CUDA graph launch
 * (captured once per input/output/direction) of work-item queue kernels and per-size launches:
 * sizes up to 1024 points whose size-specialised schedules share a CTA shape form classes of up
 * to four, one kernel per class holds their passes, and its CTAs take work items (as many
 * transforms as one CTA runs) from a queue ordered longest transforms first; longer sizes keep
 * one offset-table launch each (fully unrolled passes of many sizes in one kernel thrash the
 * instruction cache); all launches run on parallel branches.
 * ssfft_multi_exec_plain runs one plain launch per distinct size, one after another, on
 * `stream`, for comparison. */
typedef struct ssfft_multi_s *ssfft_multi_t;
ssfft_status ssfft_multi_create(ssfft_multi_t *multi, const size_t *sizes, size_t count, ssfft_dtype dtype);
/* ssfft_multi_create with plan options for every size (e.g. autotune; radices must be empty). */
ssfft_status ssfft_multi_create_ex(ssfft_multi_t *multi, const size_t *sizes, size_t count, ssfft_dtype dtype,
                                   const ssfft_plan_options *options);
ssfft_status ssfft_multi_exec(ssfft_multi_t multi, int inverse, const void *d_in, void *d_out, void *stream);
ssfft_status ssfft_multi_exec_plain(ssfft_multi_t multi, int inverse, const void *d_in, void *d_out, void *stream);
ssfft_status ssfft_multi_info(ssfft_multi_t multi, size_t *distinct_sizes, size_t *total_elements);
/* Launches one ssfft_multi_exec makes (queue classes; one per size with the per-size design). */
size_t ssfft_multi_launches(ssfft_multi_t multi);
ssfft_status ssfft_multi_destroy(ssfft_multi_t multi);

/* ---------------------------------------------------------------- serving (continuous batching)
 * No reference counterpart: the reference transforms one buffer per call.  A server takes
 * fft/ifft requests of mixed sizes and kinds from many callers (e.g. audio blocks from many
 * streams), admits each against an HBM budget for its device buffers, and executes admitted
 * requests in waves: a wave groups its requests by (n, dtype, kind, direction), copies inputs in,
 * runs one batched launch per group, copies outputs back, on its own stream; several waves are
 * in flight at once, so requests arriving while others run are admitted as buffers and wave
 * slots free up.  A request's result does not depend on what it was batched with (the kernel of
 * a given shape computes every transform identically). */
typedef struct ssfft_server_s *ssfft_server_t;

typedef struct {
	size_t hbm_budget_bytes;   /* device arena for in-flight request buffers (0: 1 GiB) */
	int max_waves_in_flight;   /* concurrent waves, one stream each (0: 8) */
	int max_requests_per_wave; /* (0: 256) */
	int coalesce;              /* 1: batched waves; 0: plain, one request at a time, synchronously */
} ssfft_server_config;

typedef struct {
	ssfft_kind kind;
	ssfft_dtype dtype;
	int inverse;
	size_t n;          /* transform size (real length for real kinds) */
	size_t frames;     /* transforms in this request, stored back to back */
	const void *h_in;  /* host input; valid until completion */
	void *h_out;       /* host output; valid until completion */
} ssfft_request;
/* Requests whose h_in and h_out are page-locked and mapped (cudaHostAlloc, cudaHostRegister),
 * aligned to two scalars, and whose shape runs in one CTA are served in place by a batched server:
 * its kernels read the input from and write the output to those buffers over the host link, and
 * the request takes no arena space.  Other requests are copied through the HBM arena. */

typedef struct {
	uint64_t submitted, completed, failed, waves, launches;
	double p50_latency_us, p99_latency_us, mean_latency_us, max_latency_us;
	double span_seconds;   /* first submit to last completion */
	double frames;         /* transforms completed */
	double flops;          /* 5 n log2 n per complex, 2.5 n log2 n per real transform completed */
	uint64_t in_place;     /* requests served in place from mapped host buffers (no copies) */
} ssfft_server_stats;

ssfft_status ssfft_server_create(ssfft_server_t *srv, const ssfft_server_config *cfg);
/* Build (compile) the plan of one request shape ahead of traffic. */
ssfft_status ssfft_server_prepare(ssfft_server_t srv, size_t n, ssfft_dtype dtype, ssfft_kind kind);
/* Queue a request (non-blocking); SSFFT_ERR_BUDGET if it alone exceeds the HBM budget. */
ssfft_status ssfft_server_submit(ssfft_server_t srv, const ssfft_request *req, uint64_t *ticket);
/* Wait for one request (SSFFT_ERR_TIMEOUT after timeout_seconds; its result status otherwise).
 * Tickets stay valid until a million newer requests have been submitted. */
ssfft_status ssfft_server_wait(ssfft_server_t srv, uint64_t ticket, double timeout_seconds);
/* Wait until every submitted request has completed. */
ssfft_status ssfft_server_drain(ssfft_server_t srv, double timeout_seconds);
ssfft_status ssfft_server_get_stats(ssfft_server_t srv, ssfft_server_stats *stats, int reset);
ssfft_status ssfft_server_destroy(ssfft_server_t srv);

/* Synthetic open-loop load for measurement: Poisson arrivals at `offered_rate` transforms/s for
 * `duration_s`, each request 1..max_frames frames of one size drawn log-uniformly from the
 * 2^a 3^b 5^c sizes in [n_min, n_max], real with probability real_fraction, inverse with
 * probability 1/2, FP32, N(0,1) inputs from pinned host memory.  Fills *stats over the run. */
typedef struct {
	double offered_rate;
	double duration_s;
	uint64_t seed;
	size_t n_min, n_max;
	int max_frames;
	double real_fraction;
} ssfft_loadgen_config;
ssfft_status ssfft_server_loadgen(ssfft_server_t srv, const ssfft_loadgen_config *cfg, ssfft_server_stats *stats);

/* ---------------------------------------------------------------- allocation-free transform
 * No counterpart in the reference.  For callers that cannot allocate device memory at the moment
 * they need a transform -- a real-time audio callback that must never block inside the CUDA
 * allocator, or an application whose own memory manager owns every byte of device memory -- this
 * computes one complex FP32 transform using only the caller's input and output and a scratch
 * array of 2^20 complex values (8 MiB) that the library keeps on every GPU that loads it, until
 * the process exits.  It creates no plan and calls no allocator.
 *   - n must be 2^a 3^b 5^c and at most ssfft_fft_noalloc_max_size() (= 1048576); larger sizes
 *     return SSFFT_ERR_INVALID_SIZE, other prime factors SSFFT_ERR_UNSUPPORTED;
 *   - d_in and d_out are 8-byte aligned device buffers of n complex floats that do not overlap
 *     (SSFFT_ERR_INVALID_VALUE otherwise); inverse != 0 computes the unnormalised inverse, as
 *     ssfft_exec does;
 *   - the first call on each device looks up the scratch array's device address and loads all of
 *     this entry point's kernels; make that first call before any stream capture;
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
/* Options the diagnostics below apply in the calling thread (NULL: planner defaults). */
ssfft_status ssfft_schedule_options(const ssfft_plan_options *options);
/* Direction (0 forward, 1 inverse) whose schedule ssfft_schedule_info / _tables report in the
 * calling thread: a RealFFT plan may run its radix list in a different order per direction. */
ssfft_status ssfft_schedule_direction(int inverse);
/* Tensor-core tile check (GPU): D = A B for one 128 x 32 x 32 FP32 tile through the split-BF16
 * tcgen05 path (A row-major 128 x 32, bt = B transposed, 32 x 32 row-major, D row-major
 * 128 x 32, all host memory); *flags receives the kernel's error flag.  No reference
 * counterpart. */
ssfft_status ssfft_diag_tc_tile(const float *a, const float *bt, float *d, unsigned *flags);
/* The plan of n points beyond one CTA as launch records: `json` receives the multi-pass
 * kernel names, CTA shapes, shared memory, groups, strides and table offsets (or, for lengths
 * that run Bluestein's algorithm, its element-wise kernels, M and the offsets of the chirp and
 * of b); `blob` the table bytes (NULL: only *blob_bytes is set).  Host only; lengths that run in
 * one CTA return SSFFT_ERR_UNSUPPORTED.  No reference counterpart. */
ssfft_status ssfft_diag_large_spec(size_t n, ssfft_dtype dtype, ssfft_kind kind, char *json, size_t json_len,
                                   void *blob, size_t *blob_bytes);
/* The work-item queue an uneven list runs as (host only, no GPU): `json` receives its classes
 * (kernel names, CTA threads, shared memory, member sizes with their transforms per item and
 * the offsets of their FP64 tables in `blob`, the items [member, count, first] in queue order,
 * and per class the byte offsets in `blob` of its int32 tables: the member of each item and, per
 * item and thread, the element offset of the transform that thread works on, -1 for none);
 * `blob` the FP64 pass twiddles and roots, then those tables (NULL: only *blob_bytes is set).
 * Sizes above 1024 points keep a launch of their own ("own_launch" in `json`).
 * ssfft_diag_multi_jit_check compiles the class kernels for `arch`.  No reference counterpart. */
ssfft_status ssfft_diag_multi_spec(const size_t *sizes, size_t count, ssfft_dtype dtype, char *json, size_t json_len,
                                   void *blob, size_t *blob_bytes);
ssfft_status ssfft_diag_multi_jit_check(const size_t *sizes, size_t count, ssfft_dtype dtype, const char *arch,
                                        size_t *image_bytes);
ssfft_status ssfft_jit_check(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, const char *arch,
                             size_t *image_bytes);
ssfft_status ssfft_schedule_info(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, int *radices, int cap,
                                 int *npasses, int *threads, int *per_cta, size_t *smem_bytes);
ssfft_status ssfft_schedule_name(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, int inverse, char *buf,
                                 size_t cap);
/* Failure-detection check (GPU): one staged launch of four n-point complex FP32 transforms
 * (16 <= n <= 16384; lengths whose input does not fit beside the work buffer stage the first
 * pass's leading rows and copy the rest into the work buffer, with a second barrier) whose
 * barriers wait for copies that are never issued, bounded by spin_limit attempts; the kernel must
 * set the error flag (returned in *flags) and return.  No reference counterpart. */
ssfft_status ssfft_diag_staged_timeout(size_t n, unsigned spin_limit, unsigned *flags);
ssfft_status ssfft_schedule_tables(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, double *tw,
                                   size_t *ntw, double *roots, size_t *nroots, double *rtw, size_t *nrtw, double *rot,
                                   size_t *nrot);

#ifdef __cplusplus
}
#endif

#endif /* SSFFT_H */

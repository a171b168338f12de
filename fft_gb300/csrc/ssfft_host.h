// ssfft_host.h -- host-side plan objects shared by the translation units of libssfft.so.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/ssfft.h"
#include "ssfft_codelets.cuh"

namespace ssfft {

constexpr int kElemsPerThread = 16;     // complex values a thread holds in one pass
constexpr int kMaxCtaThreads = 1024;
constexpr int kMaxSubTransform = 16384; // longest transform one CTA runs (FP32)
// Staged (bulk-copy) kernels: dynamic shared memory at most 227 KiB less the kernel's static
// barriers; long complex FP32 transforms (>= kLongStagedMin points) stage at <= kLongStagedThreads
// threads per transform
constexpr size_t kStagedSmemMax = 227 * 1024 - 256;
constexpr int kLongStagedMin = 8192;
constexpr int kLongStagedThreads = 384;
constexpr int kLongStagedMinThreads = 224;
constexpr int kLongStagedLocalMax = 64;  // spill bytes per thread a default long staged kernel may have

// A size-specialised kernel schedule: the compile-time parameters of one ssfft_cl::batch (or
// ssfft_cl::strided) instantiation.
struct Schedule {
	ssfft_dtype dtype = SSFFT_F32;
	int n = 0;                // complex points per transform
	std::vector<int> radices; // pass order
	int threads = 0;          // threads per transform
	int per_cta = 0;          // transforms per CTA
	int smem_stride = 0;      // padded complex slots per transform
	int kind = 0;             // ssfft_cl::kComplex / kReal / kRealHalfShift
	bool odd = false;         // real length is odd (scalar loads/stores)
	bool staged = false;      // ssfft_cl::batch_staged (bulk-copy input staging, persistent CTAs)
	bool tc = false;          // ssfft_cl::batch_tc (first pass as split-BF16 tensor-core products)
	int fuse = 0;             // RealFFT split fused into a pass: 1 forward (last pass), 2 inverse (first)
	int minb = 1;             // launch-bound CTAs per SM (register cap)
	int emax = 16;            // complex values a thread holds in one pass
	unsigned in_bytes = 0;    // staged: input bytes of one transform
	int stage_rows = 0;       // staged, > 0: only the first pass's rows r < stage_rows are staged
	size_t smem_bytes = 0;
	int pair = 0;             // ssfft_cl::pair (two-CTA cluster): the first `pair` radices are phase A
	int n1 = 0;               // pair: phase A length (product of its radices)
	int cta_threads() const { return threads * per_cta; }
	long long grid(long long batch) const { return pair ? 2 * batch : (batch + per_cta - 1) / per_cta; }
	std::string name(bool inverse) const;
};

// Schedule choices that override the planner's defaults (0 / empty = default); set by the
// caller (ssfft_plan_options) or by the autotuner.
struct Knobs {
	std::vector<int> radices;  // pass order, product = complex points
	int cta_threads = 0;       // target threads per CTA
	int emax = 0;              // complex values a thread holds in one pass
	int minb = 0;              // launch-bound CTAs per SM
	int precision = 0;         // SSFFT_PRECISION_*: 1 = first pass on the tensor cores (split BF16)
	int prefetch = -1;         // L2 prefetch distance in quarter waves of resident CTAs (-1 default)
	int fuse = -1;             // RealFFT split fused into a pass: -1 planner default, 0 never (an
	                           // explicit radix order from the caller is kept as given), 1 always
	int pair = -1;             // two-CTA cluster schedule: -1 planner default, 0 never, k > 0 with the
	                           // first k of `radices` as phase A
	int staging = 0;           // bulk-copy input staging: 0 planner default, -1 never, 1 wherever it fits
	// no shape choice made (precision is not a shape choice)
	bool empty() const { return radices.empty() && !cta_threads && !emax && !minb && prefetch < 0 && pair < 0; }
	std::string str() const;
};

// Device tables of one schedule (all inside the plan's single table allocation).
struct Tables {
	const void *tw = nullptr, *roots = nullptr, *rtw = nullptr, *rot = nullptr;
	const float *tcb = nullptr;  // tensor-core schedules: the first pass's DFT, 32 x 32 FP32
};

// Forward and inverse may differ (a RealFFT with the split fused runs the radix list rotated
// differently per direction); otherwise sch_inv / tab_inv equal sch / tab.
struct SubPlan {
	Schedule sch, sch_inv;
	Tables tab, tab_inv;
	CUfunction fwd = nullptr, inv = nullptr;
	int grid_cap = 0, grid_cap_inv = 0;  // staged (per direction): resident CTAs (persistent grid)
	long long pf_dist = 0, pf_dist_inv = 0;  // batch kernel: L2 prefetch distance in CTAs
	unsigned *err = nullptr; // staged: device error word
};

// Multi-pass (four-step) schedule for transforms longer than one CTA holds; see ssfft_large.cu.
struct LargePlan;

// Buffers and streams for ssfft_exec_host's copy/compute pipeline.
struct HostStage {
	static constexpr int kStreams = 4;  // at most; three by default
	cudaStream_t stream[kStreams] = {};
	void *d_in[kStreams] = {};
	void *d_out[kStreams] = {};
	size_t chunk = 0;   // transforms per chunk
	int streams = kStreams;
	// small calls: pinned host bounce buffers (in and out, bounce_bytes each), allocated on first use
	void *bounce_in = nullptr, *bounce_out = nullptr;
	size_t bounce_bytes = 0;
};

struct Plan {
	size_t n = 0;
	ssfft_dtype dtype = SSFFT_F32;
	ssfft_kind kind = SSFFT_COMPLEX;
	size_t batch = 1;
	int device = 0;
	SubPlan main;
	void *d_tables = nullptr;
	size_t table_bytes = 0;
	size_t scratch_bytes = 0;
	size_t stage_bytes = 0;
	int launches_per_exec = 1;
	LargePlan *large = nullptr;
	HostStage *stage = nullptr;
	Knobs knobs;              // schedule choices in force (explicit or tuned)
	Knobs knobs_inv;          // the inverse's (equal to knobs unless the autotuner chose apart)
	std::string tune_log;     // candidates the autotuner timed when this plan was made
	int autotune = 0;         // 0 off, 1 quick (threads / CTA shape), 2 full (also radix order)
	std::mutex stage_mutex;
};

// errors
ssfft_status cuda_fail(cudaError_t e, const char *what);

// Developer switches.  Every schedule experiment the library supports is read from ONE
// environment variable, SSFFT_DEBUG, a comma-separated list of key=value pairs (e.g.
// "staged=1,prefetch=0"); no other environment variable changes what the library computes or
// how.  Read each time a plan (or host-buffer call) asks, so a process can change it between
// plans.  Returns `dflt` when the key is absent or its value is not an integer.
long long debug_knob(const char *key, long long dflt);

// roots of unity, schedules and tables
void unit_root(unsigned long long k, unsigned long long L, double *re, double *im);
bool choose_radices(int n, std::vector<int> &radices, bool large_composites = true, bool real_split = false);
// allow_staged: 0 never, 1 when the debug switch staged=1 is set, 2 always (where the size allows it)
bool make_schedule(ssfft_dtype dtype, int n, int kind, bool odd, size_t batch, Schedule &s, int allow_staged = 1,
                   const Knobs *knobs = nullptr, int fuse = 0);
// dir: -1 the direction-independent base schedule, 0 forward, 1 inverse (RealFFT plans may fuse
// the split into a pass, with the radix list rotated per direction)
bool single_schedule(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, Schedule &s,
                     const Knobs *knobs = nullptr, int allow_staged = 1, int dir = -1);
void single_tables(const Schedule &s, size_t n_real, std::vector<double> &tw, std::vector<double> &roots,
                   std::vector<double> &rtw, std::vector<double> &rot);
void radix_candidates(int n, std::vector<std::vector<int>> &out, bool real_split = false);
// two-CTA cluster schedule of an n-point complex FP32 transform (ssfft_cl::pair)
bool pair_schedule(int n, Schedule &s, const Knobs *knobs);
void tc_matrix(int r0, std::vector<float> &bt);
// autotuner (ssfft_tune.cu): picks knobs for a single-CTA plan, cached per device and shape
ssfft_status autotune_single(Plan *p, int level, Knobs &best, Knobs &best_inv, std::string &log);
// prefetch distance in CTAs for a schedule with `resident` CTAs on the GPU at once
long long prefetch_distance(const Schedule &s, const Knobs &k, long long resident);
long long resident_ctas(CUfunction fwd, CUfunction inv, const Schedule &s, int device);
void schedule_twiddles(const Schedule &s, std::vector<double> &tw, std::vector<double> &roots);
size_t device_smem_limit(int dev);

// JIT (ssfft_jit.cu)
std::string device_arch(int device);
ssfft_status jit_kernels(const std::vector<std::string> &names, size_t smem_bytes, std::vector<CUfunction> &fns);
ssfft_status jit_compile_only(const std::vector<std::string> &names, const std::string &arch, size_t *image_bytes);
ssfft_status jit_launch(CUfunction f, unsigned grid, unsigned block, size_t smem, cudaStream_t stream, void *args);
ssfft_status jit_launch_grid(CUfunction f, unsigned grid_x, unsigned grid_y, unsigned block, size_t smem,
                             cudaStream_t stream, void *args);
int jit_occupancy(CUfunction f, int block, size_t smem);
// local (spill and stack) bytes per thread of a loaded kernel
int jit_local_bytes(CUfunction f);
const char *jit_last_log();
std::string jit_cache_dir();
uint64_t codelet_hash();
bool cache_read(const std::string &path, std::string &out);
void cache_write(const std::string &path, const std::string &data);

// plans
void plan_dists(const Plan *p, int inverse, long long &in_dist, long long &out_dist);
size_t plan_in_bytes(const Plan *p, int inverse, size_t batch);
size_t plan_out_bytes(const Plan *p, int inverse, size_t batch);
size_t size_minimum(size_t n);
size_t size_maximum(size_t n);
ssfft_status plan_build_large(Plan *p);
bool plan_single_cta(size_t n, ssfft_dtype dtype, ssfft_kind kind);
void plan_release(Plan *p);
ssfft_status launch_batch(const Plan *p, int inverse, const void *in, void *out, size_t batch, cudaStream_t s);
ssfft_status launch_batch_offs(const Plan *p, int inverse, const void *in, void *out, size_t batch,
                               const long long *d_offs, cudaStream_t s, const long long *d_offs_out = nullptr);
ssfft_status launch_large(Plan *p, int inverse, const void *in, void *out, size_t batch, cudaStream_t s);
void large_release(LargePlan *lp);
ssfft_status large_jit_check(size_t n, ssfft_dtype dtype, ssfft_kind kind, const char *arch, size_t *image_bytes);
bool large_describe(size_t n, ssfft_dtype dtype, ssfft_kind kind, std::vector<long long> &F);
ssfft_status large_spec(size_t n, ssfft_dtype dtype, ssfft_kind kind, std::string &json,
                        std::vector<unsigned char> &blob);

}  // namespace ssfft

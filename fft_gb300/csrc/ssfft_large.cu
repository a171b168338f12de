// ssfft_large.cu -- multi-pass (four-step) transforms for sizes beyond one CTA.
//
// The reference runs large sizes depth-first with the same radix steps (cache blocking when a
// sub-block exceeds 64 KiB, signalsmith-fft.h:130-136).  Here a transform of N complex points
// (N = F1 * F2 [* F3], each factor <= 1024) runs as 2 or 3 kernel passes over HBM:
//
//   n = n1 F2 F3 + n2 F3 + n3,  k = k1 + F1 k2 + F1 F2 k3
//   pass 1: Y1[k1][n2][n3] = DFT_F1 over n1, times W_N^{(n2 F3 + n3) k1}        (in -> scratch)
//   pass 2: Y2[k1][k2][n3] = DFT_F2 over n2, times W_{F2 F3}^{n3 k2}            (scratch, in place)
//   pass 3: X[k1 + F1 k2 + F1 F2 k3] = DFT_F3 over n3                          (scratch -> out)
//
// Each pass is one launch of ssfft_cl::strided: a CTA takes G sub-transforms that are adjacent
// in memory, so strided loads and stores move G-element contiguous segments through shared
// memory, and the inter-pass twiddle is applied in the pass's store.  Real transforms of
// h = n/2 > 16384 points add the even/odd split (forward) or pre-twiddle (inverse) as one
// element-wise kernel (ssfft_cl::real_split).
//
// Lengths with a prime factor above 1024 (which no pass can take) run Bluestein's algorithm
// instead: a chirp product, an M-point forward transform (M >= 2N - 1, 2^a 3^b 5^c), a product
// with the precomputed spectrum of the conjugate chirp, an M-point inverse transform and a final
// chirp product (ssfft_cl::blue_*); the M-point transforms are ordinary plans of this library.
// The reference handles such primes with its O(p^2) generic step (signalsmith-fft.h:187-215).
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "ssfft_host.h"

namespace ssfft {

constexpr long long kMaxFactor = 1024;
constexpr int kGroup = 16;  // sub-transforms per CTA in the strided passes

struct LargePass {
	Schedule sub;              // N-point sub-transform (sub.per_cta = G)
	bool sload = false, sstore = false;
	long long twn = 1;
	int lb = 0;
	long long U0 = 1, U1 = 1;
	long long is0 = 0, is1 = 0, in_es = 1, os0 = 0, os1 = 0, out_es = 1;
	size_t off_tw = 0, off_roots = 0, off_twlo = 0, off_twhi = 0;
	CUfunction fwd = nullptr, inv = nullptr;
	long long pf_dist = 0;     // L2 prefetch distance in CTAs (one wave of resident CTAs)
	std::string name(bool inverse, bool first, bool last, int rot) const;
};

struct LargePlan {
	long long N = 0;            // complex points
	std::vector<long long> F;   // pass factors
	std::vector<LargePass> pass;
	bool real = false, modified = false;
	size_t off_rtw = 0, off_rot = 0;
	CUfunction split_fwd = nullptr, split_inv = nullptr;
	void *d_tables = nullptr;
	void *d_scratch = nullptr;
	size_t scratch_batch = 0;
	// Bluestein (M > 0): inner M-point plan, chirp w_k and spectrum of conj(w) in d_tables
	long long M = 0;
	ssfft_plan_t inner = nullptr;
	size_t off_chirp = 0, off_bhat = 0, off_brot = 0;
	CUfunction blue_pre[2] = {}, blue_mul = nullptr, blue_post[2] = {};
	// odd real lengths: rows of n reals packed into (unpacked from) rows of N complex in d_pack
	bool odd = false;
	CUfunction pack = nullptr, unpack = nullptr;
	void *d_pack = nullptr;
};

// Smallest 2^a 3^b 5^c >= v.
static long long smooth_at_least(long long v) {
	long long best = -1;
	for (long long p5 = 1; p5 < 2 * v + 1; p5 *= 5)
		for (long long p3 = p5; p3 < 2 * v + 1; p3 *= 3) {
			long long x = p3;
			while (x < v) x *= 2;
			if (best < 0 || x < best) best = x;
		}
	return best;
}

static std::string blue_name(const char *k, ssfft_dtype dt, int conj) {
	std::string r = std::string("ssfft_cl::") + k + "<" + (dt == SSFFT_F32 ? "float" : "double");
	if (conj >= 0) r += conj ? ", true" : ", false";
	return r + ">";
}

std::string LargePass::name(bool inverse, bool first, bool last, int rot) const {
	const bool cin = inverse && first, cout = inverse && last;
	std::string r = "ssfft_cl::strided<";
	r += sub.dtype == SSFFT_F32 ? "float" : "double";
	r += ", " + std::to_string(sub.n) + ", " + std::to_string(sub.threads) + ", " + std::to_string(sub.per_cta) + ", " +
	     std::to_string(sub.smem_stride) + ", " + (cin ? "true" : "false") + ", " + (cout ? "true" : "false") + ", " +
	     std::to_string(sub.emax) + ", " + (sload ? "true" : "false") + ", " + (sstore ? "true" : "false") +
	     ", " + std::to_string(twn) + "LL, " + std::to_string(lb) + ", " + std::to_string(rot);
	for (int x : sub.radices) r += ", " + std::to_string(x);
	r += ">";
	return r;
}

static std::string split_name(ssfft_dtype dt, long long h, bool mod, bool inverse) {
	return std::string("ssfft_cl::real_split<") + (dt == SSFFT_F32 ? "float" : "double") + ", " + std::to_string(h) +
	       "LL, " + (mod ? "true" : "false") + ", " + (inverse ? "true" : "false") + ">";
}

static std::string pack_name(ssfft_dtype dt, bool unpack) {
	return std::string("ssfft_cl::real_pack<") + (dt == SSFFT_F32 ? "float" : "double") + ", " +
	       (unpack ? "true" : "false") + ">";
}

// Split N into 2 (N <= kMaxFactor^2) or 3 balanced factors, each <= kMaxFactor.
static bool large_factors(long long N, std::vector<long long> &F) {
	std::vector<long long> primes;
	long long m = N;
	for (long long p = 2; p * p <= m; ++p)
		while (m % p == 0) {
			primes.push_back(p);
			m /= p;
		}
	if (m > 1) primes.push_back(m);
	for (long long p : primes)
		if (p > kMaxFactor) return false;
	const int P = N <= kMaxFactor * kMaxFactor ? 2 : 3;
	if (N > kMaxFactor * kMaxFactor * kMaxFactor) return false;
	std::sort(primes.begin(), primes.end(), [](long long a, long long b) { return a > b; });
	F.assign(P, 1);
	for (long long p : primes) {
		// give p to the smallest group that can take it
		int best = -1;
		for (int i = 0; i < P; ++i)
			if (F[i] * p <= kMaxFactor && (best < 0 || F[i] < F[best])) best = i;
		if (best < 0) return false;
		F[best] *= p;
	}
	for (long long f : F)
		if (f < 2) return false;
	return true;
}

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

template <typename T>
static void put(std::vector<unsigned char> &blob, size_t off, const std::vector<double> &src) {
	T *dst = reinterpret_cast<T *>(blob.data() + off);
	for (size_t i = 0; i < src.size(); ++i) dst[i] = (T)src[i];
}

void large_release(LargePlan *lp) {
	if (!lp) return;
	if (lp->inner) ssfft_plan_destroy(lp->inner);
	if (lp->d_pack) cudaFree(lp->d_pack);
	if (lp->d_scratch) cudaFree(lp->d_scratch);
	if (lp->d_tables) cudaFree(lp->d_tables);
	delete lp;
}

// Schedule, strides and FP64 tables of a multi-pass plan (no GPU needed).
struct LargeTables {
	std::vector<std::vector<double>> tw, roots, twlo, twhi;
};

static ssfft_status large_schedule(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t smem_limit, LargePlan *lp,
                                   LargeTables &t) {
	const bool real = kind != SSFFT_COMPLEX;
	const long long N = (long long)(real ? n / 2 : n);
	lp->odd = real && (n & 1);  // packed around the passes (the pairs of odd rows are misaligned)
	std::vector<long long> F;
	if (!large_factors(N, F)) {
		// Bluestein (every kind; the half-shift rotations ride on its chirp kernels)
		if (N > (1ll << 29)) return SSFFT_ERR_UNSUPPORTED;
		lp->N = N;
		lp->F.clear();
		lp->real = real;
		lp->modified = kind == SSFFT_REAL_HALFSHIFT;
		lp->pass.clear();
		lp->M = smooth_at_least(2 * N - 1);
		return SSFFT_SUCCESS;
	}
	lp->N = N;
	lp->F = F;
	lp->real = real;
	lp->modified = kind == SSFFT_REAL_HALFSHIFT;
	const int P = (int)F.size();
	const size_t eb = dtype == SSFFT_F32 ? 8 : 16;
	t.tw.assign(P, {});
	t.roots.assign(P, {});
	t.twlo.assign(P, {});
	t.twhi.assign(P, {});
	auto &tw = t.tw, &roots = t.roots, &twlo = t.twlo, &twhi = t.twhi;
	lp->pass.clear();
	lp->pass.reserve(P);
	long long L = N;  // length of the dimensions not yet transformed
	for (int i = 0; i < P; ++i) {
		LargePass &ps = *lp->pass.emplace(lp->pass.end());
		const long long Fi = F[i], R = L / Fi, Q = N / L;
		const bool last = i == P - 1;
		Schedule s;
		// (fewest-pass sub-transform lists, e.g. 243 = 27 * 9, measured no faster on GB300)
		if (!make_schedule(dtype, (int)Fi, 0, false, 1, s, false)) return SSFFT_ERR_UNSUPPORTED;
		// G sub-transforms per CTA: 128-256 B segments, <= 1024 threads, <= ~100 KiB smem
		const long long U0 = last ? F[0] : R;
		// the debug switch large_group overrides the group size (experiments; read when the plan is made)
		const long long ge = debug_knob("large_group", 0);
		const int group = ge > 0 ? (int)std::min(64ll, ge) : kGroup;
		int G = (int)std::min<long long>(group, U0);
		while (G > 1 && (G * s.threads > kMaxCtaThreads || (size_t)G * s.smem_stride * eb > 100 * 1024)) --G;
		s.per_cta = G;
		// + the CTA's inter-pass twiddles (G x (KH + KL) values, KL = 16) for passes that have them
		const size_t twk = (i < P - 1) ? (size_t)G * (((Fi + 15) / 16 + 16) | 1) * eb : 0;
		s.smem_bytes = (size_t)G * s.smem_stride * eb + twk;
		if (s.smem_bytes > smem_limit) return SSFFT_ERR_UNSUPPORTED;
		ps.sub = s;
		if (!last) {
			ps.sload = ps.sstore = true;
			ps.U0 = R;
			ps.U1 = Q;
			ps.is0 = ps.os0 = 1;
			ps.is1 = ps.os1 = L;
			ps.in_es = ps.out_es = R;
			ps.twn = L;
		} else {
			// rows of F_P contiguous; output index k1 + F1 k2 (+ F1 F2 k3)
			ps.sload = false;
			ps.sstore = true;
			ps.U0 = F[0];
			ps.U1 = P == 2 ? 1 : Q / F[0];
			ps.is0 = N / F[0];
			ps.os0 = 1;
			ps.is1 = Fi;           // P == 3: u1 = k2, row offset k2 F3
			ps.os1 = F[0];         // P == 3: output offset F1 k2
			ps.in_es = 1;
			ps.out_es = N / Fi;    // F1 F2 (or F1 for P == 2)
			ps.twn = 1;
		}
		schedule_twiddles(s, tw[i], roots[i]);
		if (ps.twn > 1) {
			int lb = 0;
			while ((1ll << (2 * lb)) < ps.twn) ++lb;  // 2^lb >= sqrt(twn)
			ps.lb = lb;
			const long long lo = 1ll << lb, hi = (ps.twn + lo - 1) / lo;
			for (long long k = 0; k < lo; ++k) {
				double re, im;
				unit_root((unsigned long long)k, (unsigned long long)ps.twn, &re, &im);
				twlo[i].push_back(re);
				twlo[i].push_back(im);
			}
			for (long long k = 0; k < hi; ++k) {
				double re, im;
				unit_root((unsigned long long)(k * lo), (unsigned long long)ps.twn, &re, &im);
				twhi[i].push_back(re);
				twhi[i].push_back(im);
			}
		}
		L = R;
	}
	return SSFFT_SUCCESS;
}

// Kernel names of a multi-pass plan: per pass forward then inverse, then the real split/merge.
static std::vector<std::string> large_kernel_names(const LargePlan *lp, ssfft_dtype dtype) {
	std::vector<std::string> names;
	if (lp->M) {
		names = {blue_name("blue_pre", dtype, 0), blue_name("blue_pre", dtype, 1), blue_name("blue_mul", dtype, -1),
		         blue_name("blue_post", dtype, 0), blue_name("blue_post", dtype, 1)};
		if (lp->real) {
			names.push_back(split_name(dtype, lp->N, lp->modified, false));
			names.push_back(split_name(dtype, lp->N, lp->modified, true));
		}
		if (lp->odd) {
			names.push_back(pack_name(dtype, false));
			names.push_back(pack_name(dtype, true));
		}
		return names;
	}
	const int P = (int)lp->pass.size();
	for (int i = 0; i < P; ++i) {
		const LargePass &ps = lp->pass[i];
		const bool first = i == 0, last = i == P - 1;
		const int rot_f = lp->modified && first ? 1 : 0, rot_i = lp->modified && last ? 2 : 0;
		names.push_back(ps.name(false, first, last, rot_f));
		// a real inverse arrives pre-twiddled and conjugated, so its first pass does not conjugate
		names.push_back(lp->real ? ps.name(true, false, last, rot_i) : ps.name(true, first, last, 0));
	}
	if (lp->real) {
		names.push_back(split_name(dtype, lp->N, lp->modified, false));
		names.push_back(split_name(dtype, lp->N, lp->modified, true));
	}
	if (lp->odd) {
		names.push_back(pack_name(dtype, false));
		names.push_back(pack_name(dtype, true));
	}
	return names;
}

ssfft_status large_jit_check(size_t n, ssfft_dtype dtype, ssfft_kind kind, const char *arch, size_t *image_bytes) {
	LargePlan lp;
	LargeTables t;
	ssfft_status st = large_schedule(n, dtype, kind, 227 * 1024, &lp, t);
	if (st != SSFFT_SUCCESS) return st;
	st = jit_compile_only(large_kernel_names(&lp, dtype), arch, image_bytes);
	if (st == SSFFT_SUCCESS && lp.M) {
		size_t inner = 0;  // the M-point transforms
		st = ssfft_jit_check((size_t)lp.M, dtype, SSFFT_COMPLEX, 1, arch, &inner);
		if (image_bytes) *image_bytes += inner;
	}
	return st;
}

// Bluestein plan: chirp w_k = e^{-i pi k^2 / N} (k^2 reduced mod 2N exactly), the M-point
// spectrum of b (b_m = conj(w_|m|) for |m| < N, m taken mod M) computed once with the inner
// plan, and scratch for a chunk of transforms.
// Bluestein tables: the split twiddles (RealFFT), the chirp w_k = e^{-i pi k^2 / N} (k^2 reduced
// modulo 2N exactly) and b (b_m = conj(w_|m|), |m| < N, zero elsewhere; its M-point spectrum is
// taken on the device) in the plan's dtype; sets the offsets in *lp.  blob holds everything
// before the spectrum, bb the values of b.
static size_t blue_tables(LargePlan *lp, size_t n, ssfft_dtype dtype, std::vector<unsigned char> &blob,
                          std::vector<unsigned char> &bb) {
	const long long N = lp->N, M = lp->M;
	const size_t eb = dtype == SSFFT_F32 ? 8 : 16, sb = eb / 2;
	std::vector<double> chirp, rtw, b((size_t)M * 2, 0.0);
	chirp.reserve((size_t)N * 2);
	for (long long k = 0; k < N; ++k) {
		const unsigned long long k2 =
		    (unsigned long long)(((unsigned __int128)k * (unsigned __int128)k) % (unsigned __int128)(2 * N));
		double re, im;
		unit_root(k2, 2 * (unsigned long long)N, &re, &im);
		chirp.push_back(re);
		chirp.push_back(im);
		b[2 * k] = re;  // conj(w_k)
		b[2 * k + 1] = -im;
		if (k) {
			b[2 * (M - k)] = re;
			b[2 * (M - k) + 1] = -im;
		}
	}
	std::vector<double> rot;
	if (lp->real)
		for (long long i = 0; i <= N / 2; ++i) {
			double re, im;
			// -i e^{-2 pi i (k or k + 1/2) / n} (signalsmith-fft.h:420-425)
			if (lp->modified) unit_root(2 * (unsigned long long)i + 1, 2 * (unsigned long long)n, &re, &im);
			else unit_root((unsigned long long)i, n, &re, &im);
			rtw.push_back(im);
			rtw.push_back(-re);
		}
	if (lp->modified)
		for (long long i = 0; i < N; ++i) {  // e^{-2 pi i k / n} (:426-432)
			double re, im;
			unit_root((unsigned long long)i, n, &re, &im);
			rot.push_back(re);
			rot.push_back(im);
		}
	lp->off_rtw = 0;
	lp->off_brot = align_up(rtw.size() * sb, 256);
	lp->off_chirp = align_up(lp->off_brot + rot.size() * sb, 256);
	lp->off_bhat = align_up(lp->off_chirp + chirp.size() * sb, 256);
	const size_t total = align_up(lp->off_bhat + (size_t)M * eb, 256);
	blob.assign(lp->off_bhat, 0);
	if (sb == 4) {
		put<float>(blob, lp->off_rtw, rtw);
		put<float>(blob, lp->off_brot, rot);
		put<float>(blob, lp->off_chirp, chirp);
	} else {
		put<double>(blob, lp->off_rtw, rtw);
		put<double>(blob, lp->off_brot, rot);
		put<double>(blob, lp->off_chirp, chirp);
	}
	bb.assign((size_t)M * eb, 0);
	if (sb == 4) put<float>(bb, 0, b);
	else put<double>(bb, 0, b);
	return total;
}

static ssfft_status plan_build_bluestein(Plan *p, LargePlan *lp) {
	const long long M = lp->M;
	const size_t eb = p->dtype == SSFFT_F32 ? 8 : 16;
	std::vector<unsigned char> blob, bb;
	const size_t total = blue_tables(lp, p->n, p->dtype, blob, bb);
	cudaError_t e = cudaMalloc(&lp->d_tables, total);
	if (e == cudaSuccess) e = cudaMemcpy(lp->d_tables, blob.data(), blob.size(), cudaMemcpyHostToDevice);
	unsigned char *bhat = static_cast<unsigned char *>(lp->d_tables) + lp->off_bhat;
	if (e == cudaSuccess) e = cudaMemcpy(bhat, bb.data(), bb.size(), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return cuda_fail(e, "bluestein tables");
	p->table_bytes = total;
	// scratch: M complex per transform in flight, up to ~256 MiB
	const size_t per = (size_t)M * eb;
	lp->scratch_batch = std::max<size_t>(1, std::min<size_t>(std::min<size_t>(p->batch, 65535), (256u << 20) / per));
	e = cudaMalloc(&lp->d_scratch, per * lp->scratch_batch);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(bluestein scratch)");
	p->scratch_bytes = per * lp->scratch_batch;
	ssfft_status st = ssfft_plan_create(&lp->inner, (size_t)M, p->dtype, SSFFT_COMPLEX, lp->scratch_batch);
	if (st != SSFFT_SUCCESS) return st;
	// spectrum of b, in place, once
	st = ssfft_exec_batch(lp->inner, 0, bhat, bhat, 1, nullptr);
	if (st == SSFFT_SUCCESS) {
		e = cudaDeviceSynchronize();
		if (e != cudaSuccess) st = cuda_fail(e, "bluestein spectrum");
	}
	if (st != SSFFT_SUCCESS) return st;
	std::vector<CUfunction> fns;
	st = jit_kernels(large_kernel_names(lp, p->dtype), 0, fns);
	if (st != SSFFT_SUCCESS) return st;
	lp->blue_pre[0] = fns[0];
	lp->blue_pre[1] = fns[1];
	lp->blue_mul = fns[2];
	lp->blue_post[0] = fns[3];
	lp->blue_post[1] = fns[4];
	if (lp->real) {
		lp->split_fwd = fns[5];
		lp->split_inv = fns[6];
	}
	if (lp->odd) {
		lp->pack = fns[7];
		lp->unpack = fns[8];
		e = cudaMalloc(&lp->d_pack, (size_t)lp->N * eb * lp->scratch_batch);
		if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(odd-length pack buffer)");
		p->scratch_bytes += (size_t)lp->N * eb * lp->scratch_batch;
	}
	p->launches_per_exec = 3 + 2 * reinterpret_cast<const Plan *>(lp->inner)->launches_per_exec + (lp->real ? 1 : 0) +
	                       (lp->odd ? 1 : 0);
	return SSFFT_SUCCESS;
}

// The complex N-point transform of nb transforms (dist N) through Bluestein, src -> dst; cin /
// cout conjugate the input / output.
static ssfft_status launch_bluestein(LargePlan *lp, ssfft_dtype dtype, const void *src, void *dst, long long nb,
                                     bool cin, bool cout, cudaStream_t s, const void *rot_in = nullptr,
                                     const void *rot_out = nullptr) {
	const unsigned char *tab = static_cast<const unsigned char *>(lp->d_tables);
	ssfft_cl::BlueArgs a;
	a.in = src;
	a.out = dst;
	a.work = lp->d_scratch;
	a.chirp = tab + lp->off_chirp;
	a.bhat = tab + lp->off_bhat;
	a.n = lp->N;
	a.m = lp->M;
	a.batch = nb;
	a.dist = lp->N;
	a.rot_in = rot_in;
	a.rot_out = rot_out;
	const unsigned gm = (unsigned)((lp->M + 255) / 256), gn = (unsigned)((lp->N + 255) / 256);
	ssfft_status st = jit_launch_grid(lp->blue_pre[cin ? 1 : 0], gm, (unsigned)nb, 256, 0, s, &a);
	if (st == SSFFT_SUCCESS) st = ssfft_exec_batch(lp->inner, 0, lp->d_scratch, lp->d_scratch, (size_t)nb, s);
	if (st == SSFFT_SUCCESS) st = jit_launch_grid(lp->blue_mul, gm, (unsigned)nb, 256, 0, s, &a);
	if (st == SSFFT_SUCCESS) st = ssfft_exec_batch(lp->inner, 1, lp->d_scratch, lp->d_scratch, (size_t)nb, s);
	if (st == SSFFT_SUCCESS) st = jit_launch_grid(lp->blue_post[cout ? 1 : 0], gn, (unsigned)nb, 256, 0, s, &a);
	(void)dtype;
	return st;
}

// The pass tables of a multi-pass plan in one blob (pass twiddles, roots and the two-level
// inter-pass twiddles of every pass, then the real split twiddles and half-shift rotations), in
// the plan's dtype; sets the offsets in *lp.
static void large_blob(LargePlan *lp, LargeTables &tabs, size_t n, ssfft_dtype dtype, std::vector<unsigned char> &blob) {
	const bool real = lp->real;
	const long long N = lp->N;
	const int P = (int)lp->pass.size();
	const size_t eb = dtype == SSFFT_F32 ? 8 : 16, sb = eb / 2;
	auto &tw = tabs.tw, &roots = tabs.roots, &twlo = tabs.twlo, &twhi = tabs.twhi;
	std::vector<double> rtw, rot;
	if (real) {
		for (long long i = 0; i <= N / 2; ++i) {
			double re, im;
			if (lp->modified) unit_root(2 * i + 1, 2 * (unsigned long long)n, &re, &im);
			else unit_root(i, n, &re, &im);
			rtw.push_back(im);
			rtw.push_back(-re);
		}
		if (lp->modified)
			for (long long i = 0; i < N; ++i) {
				double re, im;
				unit_root(i, n, &re, &im);
				rot.push_back(re);
				rot.push_back(im);
			}
	}
	// one table allocation
	size_t off = 0;
	for (int i = 0; i < P; ++i) {
		LargePass &ps = lp->pass[i];
		ps.off_tw = off;
		off = align_up(off + tw[i].size() * sb, 256);
		ps.off_roots = off;
		off = align_up(off + roots[i].size() * sb, 256);
		ps.off_twlo = off;
		off = align_up(off + twlo[i].size() * sb, 256);
		ps.off_twhi = off;
		off = align_up(off + twhi[i].size() * sb, 256);
	}
	lp->off_rtw = off;
	off = align_up(off + rtw.size() * sb, 256);
	lp->off_rot = off;
	off = align_up(off + rot.size() * sb, 256);
	blob.assign(std::max<size_t>(off, 256), 0);
	for (int i = 0; i < P; ++i) {
		const LargePass &ps = lp->pass[i];
		if (sb == 4) {
			put<float>(blob, ps.off_tw, tw[i]);
			put<float>(blob, ps.off_roots, roots[i]);
			put<float>(blob, ps.off_twlo, twlo[i]);
			put<float>(blob, ps.off_twhi, twhi[i]);
		} else {
			put<double>(blob, ps.off_tw, tw[i]);
			put<double>(blob, ps.off_roots, roots[i]);
			put<double>(blob, ps.off_twlo, twlo[i]);
			put<double>(blob, ps.off_twhi, twhi[i]);
		}
	}
	if (sb == 4) {
		put<float>(blob, lp->off_rtw, rtw);
		put<float>(blob, lp->off_rot, rot);
	} else {
		put<double>(blob, lp->off_rtw, rtw);
		put<double>(blob, lp->off_rot, rot);
	}
}

ssfft_status plan_build_large(Plan *p) {
	LargePlan *lp = new LargePlan();
	p->large = lp;
	LargeTables tabs;
	ssfft_status st0 = large_schedule(p->n, p->dtype, p->kind, device_smem_limit(p->device), lp, tabs);
	if (st0 != SSFFT_SUCCESS) return st0;
	if (lp->M) return plan_build_bluestein(p, lp);
	const bool real = lp->real;
	const long long N = lp->N;
	const int P = (int)lp->pass.size();
	const size_t eb = p->dtype == SSFFT_F32 ? 8 : 16;
	std::vector<unsigned char> blob;
	large_blob(lp, tabs, p->n, p->dtype, blob);
	cudaError_t e = cudaMalloc(&lp->d_tables, blob.size());
	if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(large tables)");
	e = cudaMemcpy(lp->d_tables, blob.data(), blob.size(), cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(large tables)");
	p->table_bytes = blob.size();

	// scratch: N complex per transform, for up to ~512 MiB of transforms at once
	const size_t per = (size_t)N * eb;
	lp->scratch_batch = std::max<size_t>(1, std::min<size_t>(p->batch, (512u << 20) / per));
	e = cudaMalloc(&lp->d_scratch, per * lp->scratch_batch);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(scratch)");
	p->scratch_bytes = per * lp->scratch_batch;

	// kernels: every pass in both directions, plus the real split / merge
	const std::vector<std::string> names = large_kernel_names(lp, p->dtype);
	size_t smem_max = 0;
	for (const LargePass &ps : lp->pass) smem_max = std::max(smem_max, ps.sub.smem_bytes);
	std::vector<CUfunction> fns;
	ssfft_status st = jit_kernels(names, smem_max, fns);
	if (st != SSFFT_SUCCESS) return st;
	const bool prefetch = debug_knob("prefetch", 1) != 0;
	for (int i = 0; i < P; ++i) {
		LargePass &ps = lp->pass[i];
		ps.fwd = fns[2 * i];
		ps.inv = fns[2 * i + 1];
		// prefetch one wave of resident CTAs ahead (as the batch kernel does)
		if (prefetch) ps.pf_dist = resident_ctas(ps.fwd, ps.inv, ps.sub, p->device);
	}
	if (real) {
		lp->split_fwd = fns[2 * P];
		lp->split_inv = fns[2 * P + 1];
	}
	if (lp->odd) {
		lp->pack = fns[2 * P + 2];
		lp->unpack = fns[2 * P + 3];
		e = cudaMalloc(&lp->d_pack, per * lp->scratch_batch);
		if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(odd-length pack buffer)");
		p->scratch_bytes += per * lp->scratch_batch;
	}
	p->launches_per_exec = P + (real ? 1 : 0) + (lp->odd ? 1 : 0);
	return SSFFT_SUCCESS;
}

ssfft_status launch_large(Plan *p, int inverse, const void *in, void *out, size_t batch, cudaStream_t s) {
	LargePlan *lp = p->large;
	const size_t eb = p->dtype == SSFFT_F32 ? 8 : 16, sb = eb / 2;
	const unsigned char *tab = static_cast<const unsigned char *>(lp->d_tables);
	const long long N = lp->N;
	const int P = (int)lp->pass.size();
	long long in_dist, out_dist;  // scalars between consecutive transforms of the caller's buffers
	plan_dists(p, inverse, in_dist, out_dist);
	// odd real rows: the pass input (forward) or output (inverse) is the packed buffer
	auto pack_launch = [&](CUfunction f, const void *src, void *dst, long long nb) {
		ssfft_cl::PackArgs a;
		a.src = src;
		a.dst = dst;
		a.batch = nb;
		a.n = (long long)p->n;
		a.h = N;
		return jit_launch_grid(f, (unsigned)((N + 255) / 256), (unsigned)nb, 256, 0, s, &a);
	};
	for (size_t b0 = 0; b0 < batch; b0 += lp->scratch_batch) {
		const long long nb = (long long)std::min(lp->scratch_batch, batch - b0);
		const unsigned char *src = static_cast<const unsigned char *>(in) + b0 * (size_t)in_dist * sb;
		unsigned char *dst = static_cast<unsigned char *>(out) + b0 * (size_t)out_dist * sb;
		const void *first_in = src;
		// where the complex result of the passes goes: the caller's output, or (odd real
		// inverse) the packed buffer that is unpacked into it at the end
		void *pass_out = lp->odd && inverse ? lp->d_pack : static_cast<void *>(dst);
		if (lp->odd && !inverse) {
			// rows of n reals -> rows of N complex, into the caller's output (N complex a row)
			ssfft_status st = pack_launch(lp->pack, src, dst, nb);
			if (st != SSFFT_SUCCESS) return st;
			first_in = dst;
		}
		if (lp->real && inverse) {
			// pre-twiddle the bins into the pass buffer (the caller's input is left alone)
			ssfft_cl::SplitArgs a;
			a.buf = pass_out;
			a.src = src;
			a.batch = nb;
			a.dist = N;
			a.rtw = tab + lp->off_rtw;
			const long long pairs = N / 2 + 1;
			ssfft_status st = jit_launch_grid(lp->split_inv, (unsigned)((pairs + 255) / 256), (unsigned)nb, 256, 0, s, &a);
			if (st != SSFFT_SUCCESS) return st;
			first_in = pass_out;
		}
		if (lp->M) {
			// complex engine: Bluestein (a RealFFT inverse arrives pre-twiddled and conjugated)
			const bool cin = inverse && !lp->real, cout = inverse;
			const void *rot_in = lp->modified && !inverse ? tab + lp->off_brot : nullptr;
			const void *rot_out = lp->modified && inverse ? tab + lp->off_brot : nullptr;
			ssfft_status st = launch_bluestein(lp, p->dtype, first_in, pass_out, nb, cin, cout, s, rot_in, rot_out);
			if (st != SSFFT_SUCCESS) return st;
		}
		for (int i = 0; i < P; ++i) {
			const LargePass &ps = lp->pass[i];
			ssfft_cl::StridedArgs a;
			a.in = i == 0 ? first_in : lp->d_scratch;
			a.out = i == P - 1 ? pass_out : lp->d_scratch;
			a.U0 = ps.U0;
			a.U1 = ps.U1;
			a.U2 = nb;
			a.is0 = ps.is0;
			a.is1 = ps.is1;
			a.is2 = N;
			a.in_es = ps.in_es;
			a.os0 = ps.os0;
			a.os1 = ps.os1;
			a.os2 = N;
			a.out_es = ps.out_es;
			a.tw = tab + ps.off_tw;
			a.roots = tab + ps.off_roots;
			a.twlo = tab + ps.off_twlo;
			a.twhi = tab + ps.off_twhi;
			a.rot = tab + lp->off_rot;
			a.rot_in_stride2 = N;
			a.rot_out_stride2 = N;
			a.pf_dist = ps.pf_dist;
			const long long G = ps.sub.per_cta;
			const long long grid = nb * ps.U1 * ((ps.U0 + G - 1) / G);
			if (grid > 0x7fffffffLL) return SSFFT_ERR_INVALID_SIZE;
			ssfft_status st = jit_launch(inverse ? ps.inv : ps.fwd, (unsigned)grid, (unsigned)ps.sub.cta_threads(),
			                             ps.sub.smem_bytes, s, &a);
			if (st != SSFFT_SUCCESS) return st;
		}
		if (lp->real && !inverse) {
			ssfft_cl::SplitArgs a;
			a.buf = dst;
			a.src = dst;
			a.batch = nb;
			a.dist = N;
			a.rtw = tab + lp->off_rtw;
			const long long pairs = N / 2 + 1;
			ssfft_status st = jit_launch_grid(lp->split_fwd, (unsigned)((pairs + 255) / 256), (unsigned)nb, 256, 0, s, &a);
			if (st != SSFFT_SUCCESS) return st;
		}
		if (lp->odd && inverse) {
			// rows of N complex -> rows of n reals (2N of them; the last real is not written)
			ssfft_status st = pack_launch(lp->unpack, lp->d_pack, dst, nb);
			if (st != SSFFT_SUCCESS) return st;
		}
	}
	return SSFFT_SUCCESS;
}

// The multi-pass plan of n points as launch records (no GPU needed): a JSON object with the
// passes' kernel names (forward, inverse), CTA shape, shared memory, groups and StridedArgs
// strides and table offsets, and the table blob the passes read; for Bluestein lengths the
// element-wise kernels, M and the table offsets instead.
ssfft_status large_spec(size_t n, ssfft_dtype dtype, ssfft_kind kind, std::string &json,
                        std::vector<unsigned char> &blob) {
	LargePlan lp;
	LargeTables t;
	ssfft_status st = large_schedule(n, dtype, kind, 227 * 1024, &lp, t);
	if (st != SSFFT_SUCCESS) return st;
	const std::vector<std::string> names = large_kernel_names(&lp, dtype);
	auto num = [](long long v) { return std::to_string(v); };
	if (lp.M) {
		// Bluestein: the element-wise kernels, the tables with b (not its spectrum: the device
		// takes that with the M-point plan when the plan is made) at off_bhat
		std::vector<unsigned char> bb;
		blob.clear();
		const size_t total = blue_tables(&lp, n, dtype, blob, bb);
		blob.resize(total, 0);
		std::memcpy(blob.data() + lp.off_bhat, bb.data(), bb.size());
		json = "{\"N\": " + num(lp.N) + ", \"M\": " + num(lp.M) + ", \"real\": " + num(lp.real) +
		       ", \"modified\": " + num(lp.modified) + ", \"odd\": " + num(lp.odd) + ", \"off_rtw\": " +
		       num((long long)lp.off_rtw) + ", \"off_brot\": " + num((long long)lp.off_brot) + ", \"off_chirp\": " +
		       num((long long)lp.off_chirp) + ", \"off_bhat\": " + num((long long)lp.off_bhat) + ", \"blue\": [";
		for (int i = 0; i < 5; ++i) json += std::string(i ? ", " : "") + "\"" + names[i] + "\"";
		json += "], \"passes\": []";
		if (lp.real) json += ", \"split_fwd\": \"" + names[5] + "\", \"split_inv\": \"" + names[6] + "\"";
		if (lp.odd) json += ", \"pack\": \"" + names[7] + "\", \"unpack\": \"" + names[8] + "\"";
		json += "}";
		return SSFFT_SUCCESS;
	}
	large_blob(&lp, t, n, dtype, blob);
	json = "{\"N\": " + num(lp.N) + ", \"real\": " + num(lp.real) + ", \"modified\": " + num(lp.modified) +
	       ", \"odd\": " + num(lp.odd) + ", \"off_rtw\": " + num((long long)lp.off_rtw) + ", \"off_rot\": " +
	       num((long long)lp.off_rot) + ", \"passes\": [";
	for (size_t i = 0; i < lp.pass.size(); ++i) {
		const LargePass &ps = lp.pass[i];
		json += std::string(i ? ", " : "") + "{\"fwd\": \"" + names[2 * i] + "\", \"inv\": \"" + names[2 * i + 1] +
		        "\", \"cta\": " + num(ps.sub.cta_threads()) + ", \"smem\": " + num((long long)ps.sub.smem_bytes) +
		        ", \"G\": " + num(ps.sub.per_cta) + ", \"U0\": " + num(ps.U0) + ", \"U1\": " + num(ps.U1) +
		        ", \"is0\": " + num(ps.is0) + ", \"is1\": " + num(ps.is1) + ", \"in_es\": " + num(ps.in_es) +
		        ", \"os0\": " + num(ps.os0) + ", \"os1\": " + num(ps.os1) + ", \"out_es\": " + num(ps.out_es) +
		        ", \"off_tw\": " + num((long long)ps.off_tw) + ", \"off_roots\": " + num((long long)ps.off_roots) +
		        ", \"off_twlo\": " + num((long long)ps.off_twlo) + ", \"off_twhi\": " + num((long long)ps.off_twhi) +
		        "}";
	}
	json += "]";
	if (lp.real) json += ", \"split_fwd\": \"" + names[2 * lp.pass.size()] + "\", \"split_inv\": \"" +
		                  names[2 * lp.pass.size() + 1] + "\"";
	if (lp.odd) json += ", \"pack\": \"" + names[2 * lp.pass.size() + 2] + "\", \"unpack\": \"" +
		                 names[2 * lp.pass.size() + 3] + "\"";
	json += "}";
	return SSFFT_SUCCESS;
}

// Pass factors of the multi-pass plan of n points (no GPU needed).
bool large_describe(size_t n, ssfft_dtype dtype, ssfft_kind kind, std::vector<long long> &F) {
	LargePlan lp;
	LargeTables t;
	if (large_schedule(n, dtype, kind, 227 * 1024, &lp, t) != SSFFT_SUCCESS) return false;
	F = lp.F;
	return true;
}

}  // namespace ssfft

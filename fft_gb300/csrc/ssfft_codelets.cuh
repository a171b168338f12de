// ssfft_codelets.cuh -- size-specialised Stockham transform kernels for sm_103a.
//
// This header is compiled at plan time (NVRTC) for each (dtype, n, kind, schedule) the host
// planner picks, so every radix, stride, twiddle offset and thread mapping is a compile-time
// constant.  It includes no host headers (NVRTC provides the vector types and intrinsics).
//
// One CTA runs PER_CTA independent transforms of N complex points, THREADS threads each.  A
// transform is the compile-time pass list Rs...; the pass of radix R after passes whose radices
// multiply to NS reads element j + r*(N/R) (j < N/R, r < R), applies the twiddle
// W_{NS*R}^{(j mod NS) r}, runs an R-point DFT in registers and writes element
// (j - j mod NS)*R + (j mod NS) + r*NS.  Reads are at unit stride in j and the last pass writes
// at unit stride, so the first pass loads straight from HBM and the last pass stores straight
// to HBM (coalesced); only the passes in between go through shared memory.  The reference's
// digit-reversal permutation (signalsmith-fft.h:157-184, 288-293) thereby costs nothing.  The
// inverse runs the forward passes on conjugated data (ifft(x) = conj(fft(conj(x)))).
//
// Real transforms (RealFFT, signalsmith-fft.h:446-502) run the h = n_real/2 point complex
// transform with the even/odd split fused: the forward's split reads the last pass's output
// from shared memory and writes the h bins to HBM; the inverse's pre-twiddle reads the bins
// from HBM and writes the first pass's input to shared memory.
#pragma once

namespace ssfft_cl {

// Kernel arguments (identical layout on the host side, ssfft_jit.cu).
struct Args {
	const void *in;
	void *out;
	long long batch;     // transforms in this launch
	long long in_dist;   // distance between consecutive transforms, in scalars
	long long out_dist;
	const void *tw;      // per-pass twiddles, [pass][r-1][m] (complex, dtype)
	const void *rtw;     // real split twiddles -i e^{-2 pi i (k or k+1/2)/n_real}, k <= h/2
	const void *rot;     // half-shift rotations e^{-2 pi i k / n_real}, k < h
	const void *roots;   // W_R^k for the direct-DFT passes, concatenated
	unsigned int *err;   // staged kernels: set non-zero when a bounded wait gave up
	unsigned int spin_limit;  // staged kernels: mbarrier try_wait attempts before giving up
	unsigned int in_bytes;    // staged kernels: input bytes of one transform (multiple of 16)
	const long long *offs;    // batch kernel: if set, transform g starts offs[g] scalars into in and out
	unsigned int drop_copy;   // staged kernels, failure-detection check only: the barrier expects each
	                          // group's bytes but no copy is issued, so every wait runs out (0 normally)
};

enum : int { kComplex = 0, kReal = 1, kRealHalfShift = 2 };
// element sources / destinations of a pass: padded shared memory, HBM, or the unpadded staging
// buffer a bulk copy filled
enum : int { kSmem = 0, kGlobal = 1, kStage = 2 };

template <typename T>
struct Cx;
template <>
struct Cx<float> {
	using C = float2;
	static constexpr int kPadShift = 4;  // one pad slot per 16 float2 (128 B)
};
template <>
struct Cx<double> {
	using C = double2;
	static constexpr int kPadShift = 3;  // one pad slot per 8 double2 (128 B)
};

__device__ __forceinline__ float2 mkc(float x, float y) { return make_float2(x, y); }
__device__ __forceinline__ double2 mkc(double x, double y) { return make_double2(x, y); }

template <class C>
__device__ __forceinline__ C add(C a, C b) { return mkc(a.x + b.x, a.y + b.y); }
template <class C>
__device__ __forceinline__ C sub(C a, C b) { return mkc(a.x - b.x, a.y - b.y); }
template <class C>
__device__ __forceinline__ C mul(C a, C b) { return mkc(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
// a * conj(b)
template <class C>
__device__ __forceinline__ C mulc(C a, C b) { return mkc(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
template <class C>
__device__ __forceinline__ C conj(C a) { return mkc(a.x, -a.y); }
// -i * a
template <class C>
__device__ __forceinline__ C mul_ni(C a) { return mkc(a.y, -a.x); }
template <class C, typename S>
__device__ __forceinline__ C scale(C a, S s) { return mkc(a.x * s, a.y * s); }

template <int kShift>
__device__ __forceinline__ int pidx(int i) { return i + (i >> kShift); }

// ------------------------------------------------------------------ R-point forward DFTs
// In place, natural order in and out: v[k] <- sum_r v[r] e^{-2 pi i r k / R}.

template <class C>
__device__ __forceinline__ void dft2(C &a, C &b) {
	C t = a;
	a = add(t, b);
	b = sub(t, b);
}

template <class C>
__device__ __forceinline__ void dft4(C &a, C &b, C &c, C &d) {
	C s02 = add(a, c), d02 = sub(a, c), s13 = add(b, d), d13 = mul_ni(sub(b, d));
	a = add(s02, s13);
	c = sub(s02, s13);
	b = add(d02, d13);
	d = sub(d02, d13);
}

template <class C>
__device__ __forceinline__ void dft3(C &a, C &b, C &c) {
	using S = decltype(a.x);
	const S h = S(0.86602540378443864676);  // sin(2 pi / 3)
	C s = add(b, c), d = sub(b, c);
	C m = mkc(a.x - S(0.5) * s.x, a.y - S(0.5) * s.y);
	a = add(a, s);
	b = mkc(m.x + h * d.y, m.y - h * d.x);
	c = mkc(m.x - h * d.y, m.y + h * d.x);
}

template <class C>
__device__ __forceinline__ void dft5(C &a, C &b, C &c, C &d, C &e) {
	using S = decltype(a.x);
	const S c1 = S(0.30901699437494742410);   // cos(2 pi / 5)
	const S c2 = S(-0.80901699437494742410);  // cos(4 pi / 5)
	const S s1 = S(0.95105651629515357212);   // sin(2 pi / 5)
	const S s2 = S(0.58778525229247312917);   // sin(4 pi / 5)
	C p1 = add(b, e), m1 = sub(b, e), p2 = add(c, d), m2 = sub(c, d);
	C r1 = mkc(a.x + c1 * p1.x + c2 * p2.x, a.y + c1 * p1.y + c2 * p2.y);
	C r2 = mkc(a.x + c2 * p1.x + c1 * p2.x, a.y + c2 * p1.y + c1 * p2.y);
	C i1 = mkc(s1 * m1.x + s2 * m2.x, s1 * m1.y + s2 * m2.y);  // X1 = r1 - i*i1, X4 = r1 + i*i1
	C i2 = mkc(s2 * m1.x - s1 * m2.x, s2 * m1.y - s1 * m2.y);  // X2 = r2 - i*i2, X3 = r2 + i*i2
	a = add(a, add(p1, p2));
	b = mkc(r1.x + i1.y, r1.y - i1.x);
	e = mkc(r1.x - i1.y, r1.y + i1.x);
	c = mkc(r2.x + i2.y, r2.y - i2.x);
	d = mkc(r2.x - i2.y, r2.y + i2.x);
}

template <class C>
__device__ __forceinline__ void dft8(C *v) {
	using S = decltype(v[0].x);
	const S a = S(0.70710678118654752440);
	dft4(v[0], v[2], v[4], v[6]);
	dft4(v[1], v[3], v[5], v[7]);
	const C o1 = mkc(a * (v[3].x + v[3].y), a * (v[3].y - v[3].x));   // * W8^1
	const C o2 = mul_ni(v[5]);                                          // * W8^2
	const C o3 = mkc(a * (v[7].y - v[7].x), -a * (v[7].x + v[7].y));  // * W8^3
	const C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6], o0 = v[1];
	v[0] = add(e0, o0);
	v[4] = sub(e0, o0);
	v[1] = add(e1, o1);
	v[5] = sub(e1, o1);
	v[2] = add(e2, o2);
	v[6] = sub(e2, o2);
	v[3] = add(e3, o3);
	v[7] = sub(e3, o3);
}

// 9 = 3 x 3: DFT3 over n1 of x[3 n1 + n2], twiddle W9^{n2 k1}, DFT3 over n2, transpose.
template <class C>
__device__ __forceinline__ void dft9(C *v) {
	using S = decltype(v[0].x);
	const S c1 = S(0.76604444311897803520), s1 = S(0.64278760968653932632);  // cos, sin 2 pi/9
	const S c2 = S(0.17364817766693034885), s2 = S(0.98480775301220805936);  // cos, sin 4 pi/9
	const S c4 = S(-0.93969262078590838405), s4 = S(0.34202014332566873304); // cos, sin 8 pi/9
#pragma unroll
	for (int n2 = 0; n2 < 3; ++n2) dft3(v[n2], v[n2 + 3], v[n2 + 6]);
	v[4] = mul(v[4], mkc(c1, -s1));  // W9^1
	v[7] = mul(v[7], mkc(c2, -s2));  // W9^2
	v[5] = mul(v[5], mkc(c2, -s2));  // W9^2
	v[8] = mul(v[8], mkc(c4, -s4));  // W9^4
#pragma unroll
	for (int k1 = 0; k1 < 3; ++k1) dft3(v[3 * k1], v[3 * k1 + 1], v[3 * k1 + 2]);
	C t[9];
#pragma unroll
	for (int k1 = 0; k1 < 3; ++k1)
#pragma unroll
		for (int k2 = 0; k2 < 3; ++k2) t[k1 + 3 * k2] = v[3 * k1 + k2];
#pragma unroll
	for (int k = 0; k < 9; ++k) v[k] = t[k];
}

// 16 = 4 x 4: DFT4 over n1 of x[4 n1 + n2], twiddle W16^{n2 k1}, DFT4 over n2, transpose.
template <class C>
__device__ __forceinline__ void dft16(C *v) {
	using S = decltype(v[0].x);
	const S c1 = S(0.92387953251128675613);  // cos(pi/8)
	const S s1 = S(0.38268343236508977173);  // sin(pi/8)
	const S a = S(0.70710678118654752440);
#pragma unroll
	for (int n2 = 0; n2 < 4; ++n2) dft4(v[n2], v[n2 + 4], v[n2 + 8], v[n2 + 12]);
	v[5] = mul(v[5], mkc(c1, -s1));    // W16^1
	v[9] = mul(v[9], mkc(a, -a));      // W16^2
	v[13] = mul(v[13], mkc(s1, -c1));  // W16^3
	v[6] = mul(v[6], mkc(a, -a));      // W16^2
	v[10] = mul_ni(v[10]);             // W16^4
	v[14] = mul(v[14], mkc(-a, -a));   // W16^6
	v[7] = mul(v[7], mkc(s1, -c1));    // W16^3
	v[11] = mul(v[11], mkc(-a, -a));   // W16^6
	v[15] = mul(v[15], mkc(-c1, s1));  // W16^9
#pragma unroll
	for (int k1 = 0; k1 < 4; ++k1) dft4(v[4 * k1], v[4 * k1 + 1], v[4 * k1 + 2], v[4 * k1 + 3]);
	C t[16];
#pragma unroll
	for (int k1 = 0; k1 < 4; ++k1)
#pragma unroll
		for (int k2 = 0; k2 < 4; ++k2) t[k1 + 4 * k2] = v[4 * k1 + k2];
#pragma unroll
	for (int k = 0; k < 16; ++k) v[k] = t[k];
}

// Prime-factor (Good-Thomas) composites R = A * B with gcd(A, B) = 1: input n = (B a + A b) mod R,
// output k = (B (B^-1 mod A) ka + A (A^-1 mod B) kb) mod R; an A-point DFT over a for each b,
// then a B-point DFT over b for each ka, with no twiddles in between.  The index maps are
// register renaming only.
template <int A>
struct SmallDft;
template <>
struct SmallDft<2> {
	template <class C>
	__device__ __forceinline__ static void run(C *v) { dft2(v[0], v[1]); }
};
template <>
struct SmallDft<3> {
	template <class C>
	__device__ __forceinline__ static void run(C *v) { dft3(v[0], v[1], v[2]); }
};
template <>
struct SmallDft<4> {
	template <class C>
	__device__ __forceinline__ static void run(C *v) { dft4(v[0], v[1], v[2], v[3]); }
};
template <>
struct SmallDft<5> {
	template <class C>
	__device__ __forceinline__ static void run(C *v) { dft5(v[0], v[1], v[2], v[3], v[4]); }
};

template <int A, int B, int KA, int KB, class C>
__device__ __forceinline__ void dft_pfa(C *v) {
	constexpr int R = A * B;
	C t[B][A];
#pragma unroll
	for (int b = 0; b < B; ++b) {
#pragma unroll
		for (int a = 0; a < A; ++a) t[b][a] = v[(B * a + A * b) % R];
		SmallDft<A>::run(t[b]);
	}
#pragma unroll
	for (int ka = 0; ka < A; ++ka) {
		C u[B];
#pragma unroll
		for (int b = 0; b < B; ++b) u[b] = t[b][ka];
		SmallDft<B>::run(u);
#pragma unroll
		for (int kb = 0; kb < B; ++kb) v[(KA * ka + KB * kb) % R] = u[kb];
	}
}

template <int R>
struct Specialised {
	static constexpr bool value = R == 1 || R == 2 || R == 3 || R == 4 || R == 5 || R == 6 || R == 8 || R == 9 ||
	                              R == 10 || R == 12 || R == 15 || R == 16;
};

template <int R, class C>
__device__ __forceinline__ void dft(C *v) {
	if constexpr (R == 2) dft2(v[0], v[1]);
	else if constexpr (R == 3) dft3(v[0], v[1], v[2]);
	else if constexpr (R == 4) dft4(v[0], v[1], v[2], v[3]);
	else if constexpr (R == 5) dft5(v[0], v[1], v[2], v[3], v[4]);
	else if constexpr (R == 6) dft_pfa<2, 3, 3, 4>(v);     // 3 (3^-1 mod 2), 2 (2^-1 mod 3)
	else if constexpr (R == 8) dft8(v);
	else if constexpr (R == 9) dft9(v);
	else if constexpr (R == 10) dft_pfa<2, 5, 5, 6>(v);    // 5 (5^-1 mod 2), 2 (2^-1 mod 5)
	else if constexpr (R == 12) dft_pfa<4, 3, 9, 4>(v);    // 3 (3^-1 mod 4), 4 (4^-1 mod 3)
	else if constexpr (R == 15) dft_pfa<3, 5, 10, 6>(v);   // 5 (5^-1 mod 3), 3 (3^-1 mod 5)
	else if constexpr (R == 16) dft16(v);
}

// ------------------------------------------------------------------ per-thread context

// CIN / COUT: conjugate complex data on global load / store (the inverse runs forward passes on
// conjugated data; a multi-pass inverse conjugates at its first load and its last store).
template <typename T, int KIND, bool CIN, bool COUT>
struct Ctx {
	using C = typename Cx<T>::C;
	C *sm;         // this transform's shared-memory slots (padded)
	const T *gin;  // this transform's input, in scalars
	T *gout;       // this transform's output, in scalars
	const C *rot;  // half-shift rotations
	const C *st;   // staged kernels: this transform's input in the unpadded staging buffer
	int t;         // thread index inside the transform
	bool valid;    // the transform exists (the last CTA may be partial)
};

// Element e of the staged input (same meaning as gload, but from shared memory).
template <typename T, int KIND, bool CIN, bool COUT>
__device__ __forceinline__ typename Cx<T>::C sload(const Ctx<T, KIND, CIN, COUT> &c, int e) {
	using C = typename Cx<T>::C;
	C v = c.st[e];
	if constexpr (KIND == kComplex) {
		return CIN ? conj(v) : v;
	} else {
		if constexpr (KIND == kRealHalfShift) v = mul(v, __ldg(c.rot + e));
		return v;
	}
}

// Global element e of the pass input / output, with the conjugation of the inverse and the
// real packing folded in.
template <typename T, int KIND, bool CIN, bool COUT, bool ODD>
__device__ __forceinline__ typename Cx<T>::C gload(const Ctx<T, KIND, CIN, COUT> &c, int e) {
	using C = typename Cx<T>::C;
	if constexpr (KIND == kComplex) {
		const C v = __ldcs(reinterpret_cast<const C *>(c.gin) + e);
		return CIN ? conj(v) : v;
	} else {
		// forward real input z[e] = {x[2e], x[2e+1]} (signalsmith-fft.h:449-454)
		C v;
		if constexpr (ODD) v = mkc(__ldcs(c.gin + 2 * e), __ldcs(c.gin + 2 * e + 1));
		else v = __ldcs(reinterpret_cast<const C *>(c.gin) + e);
		if constexpr (KIND == kRealHalfShift) v = mul(v, __ldg(c.rot + e));
		return v;
	}
}

template <typename T, int KIND, bool CIN, bool COUT, bool ODD>
__device__ __forceinline__ void gstore(const Ctx<T, KIND, CIN, COUT> &c, int e, typename Cx<T>::C v) {
	using C = typename Cx<T>::C;
	if constexpr (KIND == kComplex) {
		__stcs(reinterpret_cast<C *>(c.gout) + e, COUT ? conj(v) : v);
	} else {
		// inverse real output: the data carry conj(ifft); x[2e], x[2e+1] = ifft value, un-rotated
		// for the half-shift variant (signalsmith-fft.h:496-501)
		C y = conj(v);
		if constexpr (KIND == kRealHalfShift) y = mulc(y, __ldg(c.rot + e));
		if constexpr (ODD) {
			__stcs(c.gout + 2 * e, y.x);
			__stcs(c.gout + 2 * e + 1, y.y);
		} else {
			__stcs(reinterpret_cast<C *>(c.gout) + e, y);
		}
	}
}

// ------------------------------------------------------------------ one pass

template <typename T, int N, int THREADS, int R, int NS, int TWO, int ROOTS, int SRC, int DST, int KIND, bool CIN,
          bool COUT, bool ODD, int EMAX>
__device__ __forceinline__ void pass(const Ctx<T, KIND, CIN, COUT> &c, const typename Cx<T>::C *tw,
                                     const typename Cx<T>::C *roots) {
	using C = typename Cx<T>::C;
	constexpr int PS = Cx<T>::kPadShift;
	constexpr int NB = N / R;
	if constexpr (Specialised<R>::value) {
		constexpr int NBPT = (NB + THREADS - 1) / THREADS;  // butterflies per thread
		constexpr bool GUARD = NB % THREADS != 0;
		C v[NBPT][R];
#pragma unroll
		for (int i = 0; i < NBPT; ++i) {
			const int j = c.t + i * THREADS;
			if (c.valid && (!GUARD || j < NB)) {
#pragma unroll
				for (int r = 0; r < R; ++r) {
					if constexpr (SRC == kSmem) v[i][r] = c.sm[pidx<PS>(j + r * NB)];
					else if constexpr (SRC == kStage) v[i][r] = sload(c, j + r * NB);
					else v[i][r] = gload<T, KIND, CIN, COUT, ODD>(c, j + r * NB);
				}
			}
		}
#pragma unroll
		for (int i = 0; i < NBPT; ++i) {
			const int j = c.t + i * THREADS;
			if (c.valid && (!GUARD || j < NB)) {
				if constexpr (NS > 1) {
					const int m = j % NS;
#pragma unroll
					for (int r = 1; r < R; ++r) v[i][r] = mul(v[i][r], __ldg(tw + TWO + (r - 1) * NS + m));
				}
				dft<R>(v[i]);
			}
		}
		if constexpr (SRC == kSmem && DST == kSmem) __syncthreads();
#pragma unroll
		for (int i = 0; i < NBPT; ++i) {
			const int j = c.t + i * THREADS;
			if (c.valid && (!GUARD || j < NB)) {
				const int base = (j / NS) * NS * (R - 1) + j;  // (j - j mod NS) * R + j mod NS
#pragma unroll
				for (int r = 0; r < R; ++r) {
					if constexpr (DST == kSmem) c.sm[pidx<PS>(base + r * NS)] = v[i][r];
					else gstore<T, KIND, CIN, COUT, ODD>(c, base + r * NS, v[i][r]);
				}
			}
		}
	} else {
		// Direct O(R^2) pass for other radices (the reference's fftStepGeneric,
		// signalsmith-fft.h:187-215, with precomputed roots W_R^k instead of cos/sin per term).
		// Output e = t + i*THREADS is bin k = e / NB of butterfly j = e mod NB.
		constexpr int OPT = (N + THREADS - 1) / THREADS;
		static_assert(OPT <= EMAX, "direct pass holds at most EMAX outputs per thread");
		C acc[OPT];
#pragma unroll
		for (int i = 0; i < OPT; ++i) {
			const int e = c.t + i * THREADS;
			if (c.valid && e < N) {
				const int k = e / NB, j = e - (e / NB) * NB, m = j % NS;
				C s;
				if constexpr (SRC == kSmem) s = c.sm[pidx<PS>(j)];
				else if constexpr (SRC == kStage) s = sload(c, j);
				else s = gload<T, KIND, CIN, COUT, ODD>(c, j);
				int w = 0;
				for (int r = 1; r < R; ++r) {
					C x;
					if constexpr (SRC == kSmem) x = c.sm[pidx<PS>(j + r * NB)];
					else if constexpr (SRC == kStage) x = sload(c, j + r * NB);
					else x = gload<T, KIND, CIN, COUT, ODD>(c, j + r * NB);
					if constexpr (NS > 1) x = mul(x, __ldg(tw + TWO + (r - 1) * NS + m));
					w += k;
					if (w >= R) w -= R;
					s = add(s, mul(x, __ldg(roots + ROOTS + w)));
				}
				acc[i] = s;
			}
		}
		if constexpr (SRC == kSmem && DST == kSmem) __syncthreads();
#pragma unroll
		for (int i = 0; i < OPT; ++i) {
			const int e = c.t + i * THREADS;
			if (c.valid && e < N) {
				const int k = e / NB, j = e - (e / NB) * NB, m = j % NS;
				const int d = (j - m) * R + m + k * NS;
				if constexpr (DST == kSmem) c.sm[pidx<PS>(d)] = acc[i];
				else gstore<T, KIND, CIN, COUT, ODD>(c, d, acc[i]);
			}
		}
	}
	if constexpr (DST == kSmem) __syncthreads();
}

// Twiddle slots used by a pass of radix R after NS points (none for the first pass).
template <int R, int NS>
struct TwCount {
	static constexpr int value = NS > 1 ? NS * (R - 1) : 0;
};
template <int R>
struct RootCount {
	static constexpr int value = Specialised<R>::value ? 0 : R;
};

struct NoHook {
	__device__ __forceinline__ void operator()() const {}
};

// All passes of the transform; `after_first` runs (on every thread) once the first pass has
// consumed its input.
template <typename T, int N, int THREADS, int NS, int TWO, int ROOTS, int FIRST_SRC, int LAST_DST, int KIND, bool CIN,
          bool COUT, bool ODD, int EMAX, int R, int... Rest, class Hook = NoHook>
__device__ __forceinline__ void passes(const Ctx<T, KIND, CIN, COUT> &c, const typename Cx<T>::C *tw,
                                       const typename Cx<T>::C *roots, const Hook &after_first = Hook()) {
	constexpr bool last = sizeof...(Rest) == 0;
	constexpr int SRC = NS == 1 ? FIRST_SRC : kSmem;
	constexpr int DST = last ? LAST_DST : kSmem;
	pass<T, N, THREADS, R, NS, TWO, ROOTS, SRC, DST, KIND, CIN, COUT, ODD, EMAX>(c, tw, roots);
	if constexpr (NS == 1) after_first();
	if constexpr (!last)
		passes<T, N, THREADS, NS * R, TWO + TwCount<R, NS>::value, ROOTS + RootCount<R>::value, FIRST_SRC, LAST_DST,
		       KIND, CIN, COUT, ODD, EMAX, Rest...>(c, tw, roots, NoHook());
}

// ------------------------------------------------------------------ real split / merge

// Which of the reference loop's two writes per pair i survives (signalsmith-fft.h:463-472,
// :482-492): pairs i in [s, h/2] write out[i] then out[conj(i)]; a later pair overwrites.
__device__ __forceinline__ void pair_writes(int i, int ci, int s, int last, bool &write_i, bool &write_ci) {
	const bool ci_in = ci >= s && ci <= last;
	write_i = !ci_in || ci < i;
	write_ci = !ci_in || i >= ci;
}

// Forward split: Z (H points) in shared memory -> H bins in HBM (signalsmith-fft.h:459-472).
template <typename T, int H, int THREADS, int KIND, bool CIN, bool COUT>
__device__ __forceinline__ void real_post(const Ctx<T, KIND, CIN, COUT> &c, const typename Cx<T>::C *rtw) {
	using C = typename Cx<T>::C;
	constexpr int PS = Cx<T>::kPadShift;
	constexpr bool MOD = KIND == kRealHalfShift;
	constexpr int S = MOD ? 0 : 1, LAST = H / 2, NPAIRS = LAST - S + 1;
	C *out = reinterpret_cast<C *>(c.gout);
	if (!c.valid) return;
	if (!MOD && c.t == 0) {
		const C z0 = c.sm[0];
		__stcs(out, mkc(z0.x + z0.y, z0.x - z0.y));
	}
#pragma unroll 4
	for (int p = c.t; p < NPAIRS; p += THREADS) {
		const int i = S + p;
		const int ci = MOD ? H - 1 - i : H - i;
		const C zi = c.sm[pidx<PS>(i)];
		const C zc = conj(c.sm[pidx<PS>(ci)]);
		const C odd = scale(add(zi, zc), T(0.5));
		const C even = scale(sub(zi, zc), T(0.5));
		const C e = mul(even, __ldg(rtw + i));
		bool wi, wci;
		pair_writes(i, ci, S, LAST, wi, wci);
		if (wi) __stcs(out + i, add(odd, e));
		if (wci) __stcs(out + ci, conj(sub(odd, e)));
	}
}

// Inverse pre-twiddle: H bins in HBM -> conj(first-pass input) in shared memory
// (signalsmith-fft.h:477-492).
template <typename T, int H, int THREADS, int KIND, bool CIN, bool COUT, bool STAGED = false>
__device__ __forceinline__ void real_pre(const Ctx<T, KIND, CIN, COUT> &c, const typename Cx<T>::C *rtw) {
	using C = typename Cx<T>::C;
	constexpr int PS = Cx<T>::kPadShift;
	constexpr bool MOD = KIND == kRealHalfShift;
	constexpr int S = MOD ? 0 : 1, LAST = H / 2, NPAIRS = LAST - S + 1;
	const C *in = STAGED ? c.st : reinterpret_cast<const C *>(c.gin);
	if (c.valid) {
		if (!MOD && c.t == 0) {
			const C v = STAGED ? in[0] : __ldcs(in);
			c.sm[0] = conj(mkc(v.x + v.y, v.x - v.y));
		}
#pragma unroll 4
		for (int p = c.t; p < NPAIRS; p += THREADS) {
			const int i = S + p;
			const int ci = MOD ? H - 1 - i : H - i;
			const C v = STAGED ? in[i] : __ldcs(in + i);
			const C v2c = conj(STAGED ? in[ci] : __ldcs(in + ci));
			const C odd = add(v, v2c);
			const C even = mulc(sub(v, v2c), __ldg(rtw + i));
			bool wi, wci;
			pair_writes(i, ci, S, LAST, wi, wci);
			// stored conjugated: the passes run forward on conj(data)
			if (wi) c.sm[pidx<PS>(i)] = conj(add(odd, even));
			if (wci) c.sm[pidx<PS>(ci)] = sub(odd, even);
		}
	}
	__syncthreads();
}

// ------------------------------------------------------------------ the batch kernel

// SMEM_STRIDE: padded complex slots per transform.  EMAX bounds the values a thread holds in
// one pass.  MINB: CTAs the compiler must fit per SM (caps registers; more resident warps hide the
// first pass's HBM latency).
template <typename T, int N, int THREADS, int PER_CTA, int SMEM_STRIDE, int KIND, bool INV, bool ODD, int EMAX,
          int MINB, int... Rs>
__global__ void __launch_bounds__(THREADS *PER_CTA, MINB) batch(const Args a) {
	using C = typename Cx<T>::C;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	constexpr bool REAL = KIND != kComplex;
	constexpr bool R2C = REAL && !INV, C2R = REAL && INV;
	const int g = threadIdx.x / THREADS;
	const long long gi = (long long)blockIdx.x * PER_CTA + g;
	Ctx<T, KIND, INV, INV> c;
	c.t = threadIdx.x - g * THREADS;
	c.valid = gi < a.batch;
	c.sm = reinterpret_cast<C *>(smem_raw) + g * SMEM_STRIDE;
	long long oin = 0, oout = 0;
	if (c.valid) {
		if (a.offs) oin = oout = a.offs[gi];
		else oin = gi * a.in_dist, oout = gi * a.out_dist;
	}
	c.gin = reinterpret_cast<const T *>(a.in) + oin;
	c.gout = reinterpret_cast<T *>(a.out) + oout;
	c.rot = reinterpret_cast<const C *>(a.rot);
	const C *tw = reinterpret_cast<const C *>(a.tw);
	const C *roots = reinterpret_cast<const C *>(a.roots);
	const C *rtw = reinterpret_cast<const C *>(a.rtw);
	if constexpr (C2R) real_pre<T, N, THREADS, KIND, INV, INV>(c, rtw);
	passes<T, N, THREADS, 1, 0, 0, C2R ? kSmem : kGlobal, R2C ? kSmem : kGlobal, KIND, INV, INV, ODD, EMAX, Rs...>(
	    c, tw, roots);
	if constexpr (R2C) real_post<T, N, THREADS, KIND, INV, INV>(c, rtw);
}

// ------------------------------------------------------------------ asynchronous staging

// Bulk (TMA) copy of a contiguous block into shared memory, completed on an mbarrier.  Under a
// host emulation (no __CUDA_ARCH__) the copy is synchronous and the barrier a no-op.
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ unsigned smem_u32(const void *p) {
	unsigned long long a;
	asm volatile("cvta.to.shared.u64 %0, %1;" : "=l"(a) : "l"(p));
	return static_cast<unsigned>(a);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
	asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
	asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, unsigned long long *bar,
                                          bool drop = false) {
	asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
	if (drop) return;
	asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
	                 smem_u32(dst)),
	             "l"(src), "r"(bytes), "r"(smem_u32(bar))
	             : "memory");
}
// generic-proxy reads of the staging buffer must be ordered before the next bulk write into it
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned phase) {
	unsigned ok;
	asm volatile(
	    "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
	    : "=r"(ok)
	    : "r"(smem_u32(bar)), "r"(phase)
	    : "memory");
	return ok != 0;
}
#else
inline void mbar_init(unsigned long long *, unsigned) {}
inline void bulk_load(void *dst, const void *src, unsigned bytes, unsigned long long *, bool = false) {
	const unsigned char *s = static_cast<const unsigned char *>(src);
	unsigned char *d = static_cast<unsigned char *>(dst);
	for (unsigned i = 0; i < bytes; ++i) d[i] = s[i];
}
inline void fence_async_smem() {}
inline bool mbar_try_wait(unsigned long long *, unsigned) { return true; }
#endif

// Wait for phase `phase` of `bar`, giving up after `limit` attempts (each try_wait itself
// suspends for a bounded, hardware-defined time).
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned phase, unsigned limit) {
	for (unsigned i = 0; i < limit; ++i)
		if (mbar_try_wait(bar, phase)) return true;
	return false;
}

// The batch kernel with asynchronous input staging: persistent CTAs walk the groups of PER_CTA
// transforms; each group's input (contiguous in HBM) arrives in an unpadded staging buffer by
// one bulk copy, and the copy of the next group is issued as soon as the first pass (or the
// real pre-twiddle) has read the current one, so the HBM load overlaps the remaining passes.
// Requires in_bytes % 16 == 0 and 16-byte aligned input.  A bounded wait that runs out sets
// *err and the CTA returns without writing.  (Inside the persistent loop the compiler keeps far
// more registers live than one pass needs; MINB caps them.)
template <typename T, int N, int THREADS, int PER_CTA, int SMEM_STRIDE, int KIND, bool INV, int EMAX, int MINB,
          int... Rs>
__global__ void __launch_bounds__(THREADS *PER_CTA, MINB) batch_staged(const Args a) {
	using C = typename Cx<T>::C;
	constexpr bool REAL = KIND != kComplex;
	constexpr bool R2C = REAL && !INV, C2R = REAL && INV;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	__shared__ __align__(8) unsigned long long bar;
	const unsigned in_bytes = a.in_bytes;
	unsigned char *stage = smem_raw;
	C *work = reinterpret_cast<C *>(smem_raw + ((PER_CTA * in_bytes + 127u) & ~127u));
	const long long ngroups = (a.batch + PER_CTA - 1) / PER_CTA;
	const unsigned char *in = reinterpret_cast<const unsigned char *>(a.in);
	const int g = threadIdx.x / THREADS;
	Ctx<T, KIND, INV, INV> c;
	c.t = threadIdx.x - g * THREADS;
	c.sm = work + g * SMEM_STRIDE;
	c.st = reinterpret_cast<const C *>(stage + g * in_bytes);
	c.rot = reinterpret_cast<const C *>(a.rot);
	c.gin = nullptr;
	const C *tw = reinterpret_cast<const C *>(a.tw);
	const C *roots = reinterpret_cast<const C *>(a.roots);
	const C *rtw = reinterpret_cast<const C *>(a.rtw);
	auto issue = [&](long long grp) {
		const long long nt = a.batch - grp * PER_CTA < PER_CTA ? a.batch - grp * PER_CTA : PER_CTA;
		bulk_load(stage, in + grp * PER_CTA * (long long)in_bytes, (unsigned)(nt * in_bytes), &bar, a.drop_copy != 0);
	};
	if (threadIdx.x == 0) {
		mbar_init(&bar, 1);
		if (blockIdx.x < ngroups) issue(blockIdx.x);
	}
	__syncthreads();
	unsigned phase = 0;
	for (long long grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
		const bool ok = mbar_wait_bounded(&bar, phase, a.spin_limit);
		if (__syncthreads_or(!ok)) {
			if (threadIdx.x == 0) atomicOr(a.err, 1u);
			mbar_wait_bounded(&bar, phase, a.spin_limit);  // let the copy in flight land
			return;
		}
		phase ^= 1u;
		const long long gi = grp * PER_CTA + g;
		c.valid = gi < a.batch;
		c.gout = reinterpret_cast<T *>(a.out) + (c.valid ? gi * a.out_dist : 0);
		const long long next = grp + gridDim.x;
		auto refill = [&]() {
			__syncthreads();  // every thread has read the staging buffer
			if (threadIdx.x == 0 && next < ngroups) {
				fence_async_smem();
				issue(next);
			}
		};
		if constexpr (C2R) {
			real_pre<T, N, THREADS, KIND, INV, INV, true>(c, rtw);
			refill();
			passes<T, N, THREADS, 1, 0, 0, kSmem, kGlobal, KIND, INV, INV, false, EMAX, Rs...>(c, tw, roots);
		} else {
			passes<T, N, THREADS, 1, 0, 0, kStage, R2C ? kSmem : kGlobal, KIND, INV, INV, false, EMAX, Rs...>(c, tw, roots,
			                                                                                                refill);
		}
		if constexpr (R2C) real_post<T, N, THREADS, KIND, INV, INV>(c, rtw);
		__syncthreads();  // the work buffer is reused by the next group
	}
}

// ------------------------------------------------------------------ multi-pass (four-step) kernel

// One pass of a multi-pass transform: U = U2*U1*U0 sub-transforms of N points.  Sub-transform
// u = (u2, u1, u0) reads element e at in + u2*is2 + u1*is1 + u0*is0 + e*in_es and writes element
// k at out + u2*os2 + u1*os1 + u0*os0 + k*out_es (complex elements).  A CTA takes G consecutive
// u0 (adjacent in memory when is0 / os0 == 1), so a strided load (SLOAD) or store (SSTORE)
// through shared memory moves G-element contiguous segments.  TW multiplies output element k of
// sub-transform u0 by W_TWN^{u0 k} (the four-step inter-pass twiddle), from a two-level table:
// W^t = twhi[t >> LB] * twlo[t & (2^LB - 1)].  ROT (first pass of a half-shift real forward /
// last pass of its inverse) applies e^{-+2 pi i j / n_real} by the element's index j in the
// whole transform.
struct StridedArgs {
	const void *in;
	void *out;
	long long U0, U1, U2;
	long long is0, is1, is2, in_es;
	long long os0, os1, os2, out_es;
	const void *tw;     // pass twiddles of the N-point sub-transform
	const void *roots;
	const void *twlo;   // inter-pass twiddles, two-level table
	const void *twhi;
	const void *rot;    // half-shift rotations (ROT)
	long long rot_in_stride2, rot_out_stride2;  // u2 stride of the index j inside the whole transform
};

template <typename T, int N, int THREADS, int G, int STRIDE, bool CIN, bool COUT, int EMAX, bool SLOAD, bool SSTORE,
          long long TWN, int LB, int ROT, int... Rs>
__global__ void __launch_bounds__(THREADS *G) strided(const StridedArgs a) {
	using C = typename Cx<T>::C;
	constexpr int PS = Cx<T>::kPadShift;
	constexpr int CTA = THREADS * G;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	C *sm_all = reinterpret_cast<C *>(smem_raw);
	const long long blocks0 = (a.U0 + G - 1) / G;
	long long cta = blockIdx.x;
	const long long u0b = cta % blocks0;
	cta /= blocks0;
	const long long u1 = cta % a.U1, u2 = cta / a.U1;
	const long long u00 = u0b * G;
	const long long ib = u2 * a.is2 + u1 * a.is1, ob = u2 * a.os2 + u1 * a.os1;
	const C *in = reinterpret_cast<const C *>(a.in);
	C *out = reinterpret_cast<C *>(a.out);
	const int g = threadIdx.x / THREADS;
	Ctx<T, kComplex, CIN, COUT> c;
	c.t = threadIdx.x - g * THREADS;
	c.valid = u00 + g < a.U0;
	c.sm = sm_all + g * STRIDE;
	c.gin = reinterpret_cast<const T *>(in + (c.valid ? ib + (u00 + g) * a.is0 : 0));
	c.gout = reinterpret_cast<T *>(out + (c.valid ? ob + (u00 + g) * a.os0 : 0));
	c.rot = reinterpret_cast<const C *>(a.rot);
	if constexpr (SLOAD) {
		// G-element segments: consecutive threads take consecutive u0 of the same element
#pragma unroll 4
		for (int idx = threadIdx.x; idx < G * N; idx += CTA) {
			const int gg = idx % G, e = idx / G;
			if (u00 + gg < a.U0) {
				const long long off = ib + (u00 + gg) * a.is0 + (long long)e * a.in_es;
				C v = __ldcs(in + off);
				if constexpr (CIN) v = conj(v);
				if constexpr (ROT == 1) v = mul(v, __ldg(c.rot + (off - u2 * a.rot_in_stride2)));
				sm_all[gg * STRIDE + pidx<PS>(e)] = v;
			}
		}
		__syncthreads();
	}
	passes<T, N, THREADS, 1, 0, 0, SLOAD ? kSmem : kGlobal, SSTORE ? kSmem : kGlobal, kComplex, CIN, COUT, false, EMAX,
	       Rs...>(c, reinterpret_cast<const C *>(a.tw), reinterpret_cast<const C *>(a.roots));
	if constexpr (SSTORE) {
		const C *twlo = reinterpret_cast<const C *>(a.twlo);
		const C *twhi = reinterpret_cast<const C *>(a.twhi);
#pragma unroll 4
		for (int idx = threadIdx.x; idx < G * N; idx += CTA) {
			const int gg = idx % G, k = idx / G;
			const long long u0 = u00 + gg;
			if (u0 < a.U0) {
				C v = sm_all[gg * STRIDE + pidx<PS>(k)];
				if constexpr (TWN > 1) {
					const unsigned long long t = ((unsigned long long)u0 * (unsigned long long)k) % (unsigned long long)TWN;
					v = mul(v, mul(__ldg(twhi + (t >> LB)), __ldg(twlo + (t & ((1ull << LB) - 1)))));
				}
				const long long off = ob + u0 * a.os0 + (long long)k * a.out_es;
				if constexpr (ROT == 2) {
					// inverse half-shift real output: data carry conj(ifft), un-rotate by e^{-2 pi i j/n}
					C y = conj(v);
					y = mulc(y, __ldg(c.rot + (off - u2 * a.rot_out_stride2)));
					__stcs(out + off, y);
				} else {
					__stcs(out + off, COUT ? conj(v) : v);
				}
			}
		}
	}
}

// Real split / merge over global memory for real transforms longer than one CTA holds
// (signalsmith-fft.h:459-472 forward, :477-492 inverse).  One thread per pair (i, conj(i)),
// in place on `buf` (H complex per transform, batch transforms `dist` complex apart).
// Forward: buf holds Z = FFT(z) and receives the H bins.  Inverse: buf holds the H bins and
// receives conj(pre-twiddled input) for the forward passes that follow.
struct SplitArgs {
	void *buf;
	const void *src;   // inverse only: the caller's bins (buf may differ so the input is kept)
	long long batch, dist;
	const void *rtw;
};

template <typename T, long long H, bool MOD, bool INVERSE>
__global__ void __launch_bounds__(256) real_split(const SplitArgs a) {
	using C = typename Cx<T>::C;
	constexpr long long S = MOD ? 0 : 1, LAST = H / 2, NPAIRS = LAST - S + 1;
	const long long gid = (long long)blockIdx.x * 256 + threadIdx.x;
	const long long b = blockIdx.y;
	if (b >= a.batch) return;
	C *buf = reinterpret_cast<C *>(a.buf) + b * a.dist;
	const C *src = reinterpret_cast<const C *>(INVERSE ? a.src : a.buf) + b * a.dist;
	const C *rtw = reinterpret_cast<const C *>(a.rtw);
	if (!MOD && gid == 0) {
		const C v = src[0];
		if (INVERSE) buf[0] = conj(mkc(v.x + v.y, v.x - v.y));
		else buf[0] = mkc(v.x + v.y, v.x - v.y);
	}
	if (gid >= NPAIRS) return;
	const long long i = S + gid;
	const long long ci = MOD ? H - 1 - i : H - i;
	const bool ci_in = ci >= S && ci <= LAST;
	const bool wi = !ci_in || ci < i, wci = !ci_in || i >= ci;
	if (!INVERSE) {
		const C zi = src[i];
		const C zc = conj(src[ci]);
		const C odd = scale(add(zi, zc), T(0.5));
		const C even = scale(sub(zi, zc), T(0.5));
		const C e = mul(even, __ldg(rtw + i));
		if (wi) buf[i] = add(odd, e);
		if (wci) buf[ci] = conj(sub(odd, e));
	} else {
		const C v = src[i];
		const C v2c = conj(src[ci]);
		const C odd = add(v, v2c);
		const C even = mulc(sub(v, v2c), __ldg(rtw + i));
		if (wi) buf[i] = conj(add(odd, even));
		if (wci) buf[ci] = sub(odd, even);
	}
}

}  // namespace ssfft_cl

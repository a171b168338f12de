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
	const float *tcb;         // tensor-core kernels: the first pass's DFT as a 32 x 32 real matrix
	                          // [output column][input column] (FP32 values of FP64-built roots)
	long long pf_dist;        // batch kernel: CTA b prefetches into L2 the input of CTA b + pf_dist
	                          // (about one wave of resident CTAs ahead; 0 = off)
	const long long *offs_out;  // batch kernel with offs: if set, transform g's output starts
	                            // offs_out[g] scalars into out (else offs[g])
};

enum : int { kComplex = 0, kReal = 1, kRealHalfShift = 2 };
// element sources / destinations of a pass: padded shared memory, HBM, or the unpadded staging
// buffer a bulk copy filled
enum : int { kSmem = 0, kGlobal = 1, kStage = 2 };
// first pass of a split-staged kernel: rows r < K of the first pass (elements j + r NB) in the
// staging buffer, rows r >= K in the work buffer (unpadded, from element K NB on); the source
// code is kStageSplit + K
enum : int { kStageSplit = 16 };
__host__ __device__ constexpr bool is_stage(int src) { return src == kStage || src >= kStageSplit; }
// fused real split: the last pass of a RealFFT forward writes the bins (kFusedR2C), the first pass
// of its inverse reads the bins and pre-twiddles them (kFusedC2R)
enum : int { kFusedR2C = 3, kFusedC2R = 4 };

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

// 25 = 5 x 5: DFT5 over n1 of x[5 n1 + n2], twiddle W25^{n2 k1}, DFT5 over n2, transpose.
template <class C>
__device__ __forceinline__ void dft25(C *v) {
	using S = decltype(v[0].x);
	// W25^e = cos(2 pi e/25) - i sin(2 pi e/25) for the exponents n2 k1 that occur
	const C w1 = mkc(S(0.96858316112863108), S(-0.24868988716485479));
	const C w2 = mkc(S(0.87630668004386358), S(-0.48175367410171527));
	const C w3 = mkc(S(0.72896862742141155), S(-0.68454710592868873));
	const C w4 = mkc(S(0.53582679497899666), S(-0.84432792550201508));
	const C w6 = mkc(S(0.062790519529313527), S(-0.99802672842827156));
	const C w8 = mkc(S(-0.42577929156507266), S(-0.90482705246601953));
	const C w9 = mkc(S(-0.63742398974868971), S(-0.77051324277578925));
	const C w12 = mkc(S(-0.99211470131447788), S(-0.12533323356430454));
	const C w16 = mkc(S(-0.63742398974868949), S(0.77051324277578936));
#pragma unroll
	for (int n2 = 0; n2 < 5; ++n2) dft5(v[n2], v[n2 + 5], v[n2 + 10], v[n2 + 15], v[n2 + 20]);
	v[6] = mul(v[6], w1);    // n2 1, k1 1
	v[11] = mul(v[11], w2);  // n2 1, k1 2
	v[16] = mul(v[16], w3);
	v[21] = mul(v[21], w4);
	v[7] = mul(v[7], w2);    // n2 2
	v[12] = mul(v[12], w4);
	v[17] = mul(v[17], w6);
	v[22] = mul(v[22], w8);
	v[8] = mul(v[8], w3);    // n2 3
	v[13] = mul(v[13], w6);
	v[18] = mul(v[18], w9);
	v[23] = mul(v[23], w12);
	v[9] = mul(v[9], w4);    // n2 4
	v[14] = mul(v[14], w8);
	v[19] = mul(v[19], w12);
	v[24] = mul(v[24], w16);
#pragma unroll
	for (int k1 = 0; k1 < 5; ++k1) dft5(v[5 * k1], v[5 * k1 + 1], v[5 * k1 + 2], v[5 * k1 + 3], v[5 * k1 + 4]);
	C t[25];
#pragma unroll
	for (int k1 = 0; k1 < 5; ++k1)
#pragma unroll
		for (int k2 = 0; k2 < 5; ++k2) t[k1 + 5 * k2] = v[5 * k1 + k2];
#pragma unroll
	for (int k = 0; k < 25; ++k) v[k] = t[k];
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
template <>
struct SmallDft<8> {
	template <class C>
	__device__ __forceinline__ static void run(C *v) { dft8(v); }
};
template <>
struct SmallDft<9> {
	template <class C>
	__device__ __forceinline__ static void run(C *v) { dft9(v); }
};
template <>
struct SmallDft<16> {
	template <class C>
	__device__ __forceinline__ static void run(C *v) { dft16(v); }
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

// Cooley-Tukey composites R = A * B (A-point DFTs over n1 of x[B n1 + n2], twiddles
// W_R^{n2 k1} from the table w, B-point DFTs over n2, transpose to k = k1 + A k2).
template <int A, int B, int E, class C>
__device__ __forceinline__ void dft_ct(C *v, const C (&w)[E]) {
	constexpr int R = A * B;
#pragma unroll
	for (int n2 = 0; n2 < B; ++n2) {
		C u[A];
#pragma unroll
		for (int n1 = 0; n1 < A; ++n1) u[n1] = v[B * n1 + n2];
		SmallDft<A>::run(u);
#pragma unroll
		for (int k1 = 0; k1 < A; ++k1) v[B * k1 + n2] = (n2 && k1) ? mul(u[k1], w[n2 * k1]) : u[k1];
	}
#pragma unroll
	for (int k1 = 0; k1 < A; ++k1) SmallDft<B>::run(v + B * k1);
	C t[R];
#pragma unroll
	for (int k1 = 0; k1 < A; ++k1)
#pragma unroll
		for (int k2 = 0; k2 < B; ++k2) t[k1 + A * k2] = v[B * k1 + k2];
#pragma unroll
	for (int k = 0; k < R; ++k) v[k] = t[k];
}

// 27 = 3 x 9 and 32 = 4 x 8; w[e] = W_R^e = cos(2 pi e/R) - i sin(2 pi e/R)
template <class C>
__device__ __forceinline__ void dft27(C *v) {
	using S = decltype(v[0].x);
	const C w[17] = {
	    mkc(S(1.0), S(-0.0)), mkc(S(0.9730448705798238), S(-0.23061587074244017)),
	    mkc(S(0.8936326403234123), S(-0.44879918020046217)), mkc(S(0.766044443118978), S(-0.6427876096865393)),
	    mkc(S(0.5971585917027862), S(-0.8021231927550437)), mkc(S(0.3960797660391569), S(-0.918216106880274)),
	    mkc(S(0.17364817766693041), S(-0.984807753012208)), mkc(S(-0.058144828910475774), S(-0.9983081582712682)),
	    mkc(S(-0.2868032327110902), S(-0.9579895123154889)), mkc(S(-0.4999999999999998), S(-0.8660254037844387)),
	    mkc(S(-0.6862416378687335), S(-0.7273736415730488)), mkc(S(-0.8354878114129363), S(-0.5495089780708062)),
	    mkc(S(-0.9396926207859083), S(-0.3420201433256689)), mkc(S(-0.993238357741943), S(-0.11609291412522993)),
	    mkc(S(-0.993238357741943), S(0.11609291412523012)), mkc(S(-0.9396926207859085), S(0.3420201433256682)),
	    mkc(S(-0.8354878114129365), S(0.549508978070806)),
	};
	dft_ct<3, 9>(v, w);
}
template <class C>
__device__ __forceinline__ void dft32(C *v) {
	using S = decltype(v[0].x);
	const C w[22] = {
	    mkc(S(1.0), S(-0.0)), mkc(S(0.9807852804032304), S(-0.19509032201612825)),
	    mkc(S(0.9238795325112867), S(-0.3826834323650898)), mkc(S(0.8314696123025452), S(-0.5555702330196022)),
	    mkc(S(0.7071067811865476), S(-0.7071067811865475)), mkc(S(0.5555702330196023), S(-0.8314696123025452)),
	    mkc(S(0.38268343236508984), S(-0.9238795325112867)), mkc(S(0.19509032201612833), S(-0.9807852804032304)),
	    mkc(S(0.0), S(-1.0)), mkc(S(-0.1950903220161282), S(-0.9807852804032304)),
	    mkc(S(-0.3826834323650897), S(-0.9238795325112867)), mkc(S(-0.555570233019602), S(-0.8314696123025455)),
	    mkc(S(-0.7071067811865475), S(-0.7071067811865476)), mkc(S(-0.8314696123025453), S(-0.5555702330196022)),
	    mkc(S(-0.9238795325112867), S(-0.3826834323650899)), mkc(S(-0.9807852804032304), S(-0.1950903220161286)),
	    mkc(S(-1.0), S(-0.0)), mkc(S(-0.9807852804032304), S(0.19509032201612836)),
	    mkc(S(-0.9238795325112868), S(0.38268343236508967)), mkc(S(-0.8314696123025455), S(0.555570233019602)),
	    mkc(S(-0.7071067811865477), S(0.7071067811865475)), mkc(S(-0.5555702330196022), S(0.8314696123025452)),
	};
	dft_ct<4, 8>(v, w);
}

template <int R>
struct Specialised {
	static constexpr bool value = R == 1 || R == 2 || R == 3 || R == 4 || R == 5 || R == 6 || R == 8 || R == 9 ||
	                              R == 10 || R == 12 || R == 15 || R == 16 || R == 18 || R == 20 || R == 24 ||
	                              R == 25 || R == 27 || R == 32 || R == 36 || R == 40 || R == 45;
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
	else if constexpr (R == 18) dft_pfa<2, 9, 9, 10>(v);    // 9 (9^-1 mod 2), 2 (2^-1 mod 9 = 5)
	else if constexpr (R == 20) dft_pfa<4, 5, 5, 16>(v);    // 5 (5^-1 mod 4 = 1), 4 (4^-1 mod 5 = 4)
	else if constexpr (R == 24) dft_pfa<8, 3, 9, 16>(v);    // 3 (3^-1 mod 8 = 3), 8 (8^-1 mod 3 = 2)
	else if constexpr (R == 25) dft25(v);
	else if constexpr (R == 27) dft27(v);
	else if constexpr (R == 32) dft32(v);
	else if constexpr (R == 36) dft_pfa<4, 9, 9, 28>(v);    // 9 (9^-1 mod 4 = 1), 4 (4^-1 mod 9 = 7)
	else if constexpr (R == 40) dft_pfa<8, 5, 25, 16>(v);   // 5 (5^-1 mod 8 = 5), 8 (8^-1 mod 5 = 2)
	else if constexpr (R == 45) dft_pfa<9, 5, 10, 36>(v);   // 5 (5^-1 mod 9 = 2), 9 (9^-1 mod 5 = 4)
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
	const C *st2;  // split-staged kernels: the first pass's rows >= K (unpadded, in the work buffer)
	const C *rtw;  // real split twiddles (fused split passes)
	int t;         // thread index inside the transform
	bool valid;    // the transform exists (the last CTA may be partial)
};

// Element e of the staged input (same meaning as gload, but from shared memory).
template <typename T, int KIND, bool CIN, bool COUT>
__device__ __forceinline__ typename Cx<T>::C sfix(const Ctx<T, KIND, CIN, COUT> &c, int e, typename Cx<T>::C v) {
	if constexpr (KIND == kComplex) {
		return CIN ? conj(v) : v;
	} else {
		if constexpr (KIND == kRealHalfShift) v = mul(v, __ldg(c.rot + e));
		return v;
	}
}
template <typename T, int KIND, bool CIN, bool COUT>
__device__ __forceinline__ typename Cx<T>::C sload(const Ctx<T, KIND, CIN, COUT> &c, int e) {
	return sfix(c, e, c.st[e]);
}
// Element j + r NB of the first pass's input from a staging source SRC (kStage: all of it in the
// staging buffer; kStageSplit + K: rows r < K there, the others in the work buffer).  With r a
// compile-time constant (unrolled loops) the choice of buffer costs nothing.
template <int SRC, int NB, typename T, int KIND, bool CIN, bool COUT>
__device__ __forceinline__ typename Cx<T>::C sload_row(const Ctx<T, KIND, CIN, COUT> &c, int j, int r) {
	const int e = j + r * NB;
	if constexpr (SRC >= kStageSplit) {
		constexpr int K = SRC - kStageSplit;
		return sfix(c, e, r < K ? c.st[e] : c.st2[e - K * NB]);
	} else {
		return sload(c, e);
	}
}

// L2 prefetch of one line, or (bulk) of a 16-byte aligned range whose size is a multiple of 16
// bytes by the copy engine of the SM (hints: no data returns, nothing waits on them).
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ void prefetch_l2(const void *p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
__device__ __forceinline__ void prefetch_l2_bulk(const void *p, unsigned bytes) {
	asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}
#else
inline void prefetch_l2(const void *) {}
inline void prefetch_l2_bulk(const void *, unsigned) {}
#endif

// The input of the CTA pf_dist blocks ahead (transforms stored back to back), one 128-byte
// line per thread per step: by the time that CTA starts, about one wave later, its loads hit L2,
// and the HBM read stream keeps going while resident CTAs compute.
template <typename T, int PER_CTA, int CTA_THREADS>
__device__ __forceinline__ void prefetch_ahead(const Args &a) {
	if (a.pf_dist <= 0) return;
	const long long first = ((long long)blockIdx.x + a.pf_dist) * PER_CTA;
	if (first >= a.batch) return;
	const long long cnt = a.batch - first < PER_CTA ? a.batch - first : PER_CTA;
	const unsigned char *in = reinterpret_cast<const unsigned char *>(a.in);
	const long long per = a.in_dist * (long long)sizeof(T);  // input bytes of one transform
	if (!a.offs) {
		const unsigned char *base = in + first * per;
		const long long bytes = cnt * per;
		if ((((unsigned long long)base | (unsigned long long)bytes) & 15) == 0 && bytes < (1ll << 31)) {
			// one bulk prefetch for the whole range (TMA), issued by one thread
			if (threadIdx.x == 0) prefetch_l2_bulk(base, (unsigned)bytes);
		} else {
			for (long long off = (long long)threadIdx.x * 128; off < bytes; off += (long long)CTA_THREADS * 128)
				prefetch_l2(base + off);
		}
	} else {
		// scattered transforms (offset table): line k of transform g = k / lines
		const long long lines = (per + 127) / 128;
		for (long long k = threadIdx.x; k < cnt * lines; k += CTA_THREADS) {
			const long long g = k / lines;
			prefetch_l2(in + a.offs[first + g] * (long long)sizeof(T) + (k - g * lines) * 128);
		}
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

// Two adjacent elements e, e + 1 (e even) of the pass input / output in one 16-byte access
// (FP32 with paired layout; the caller has checked that the transform starts on a 16-byte
// boundary), with the same conjugation, packing and rotation as gload / gstore.
template <typename T, int KIND, bool CIN, bool COUT, bool ODD>
__device__ __forceinline__ void gload2(const Ctx<T, KIND, CIN, COUT> &c, int e, typename Cx<T>::C &a,
                                       typename Cx<T>::C &b) {
	static_assert(sizeof(T) == 4 && !ODD, "paired access is for FP32 data in complex pairs");
	const float4 q = __ldcs(reinterpret_cast<const float4 *>(c.gin) + e / 2);
	a = mkc(q.x, q.y);
	b = mkc(q.z, q.w);
	if constexpr (KIND == kComplex) {
		if (CIN) {
			a = conj(a);
			b = conj(b);
		}
	} else if constexpr (KIND == kRealHalfShift) {
		a = mul(a, __ldg(c.rot + e));
		b = mul(b, __ldg(c.rot + e + 1));
	}
}

template <typename T, int KIND, bool CIN, bool COUT, bool ODD>
__device__ __forceinline__ void gstore2(const Ctx<T, KIND, CIN, COUT> &c, int e, typename Cx<T>::C a,
                                        typename Cx<T>::C b) {
	static_assert(sizeof(T) == 4 && !ODD, "paired access is for FP32 data in complex pairs");
	if constexpr (KIND == kComplex) {
		if (COUT) {
			a = conj(a);
			b = conj(b);
		}
	} else {
		a = conj(a);
		b = conj(b);
		if constexpr (KIND == kRealHalfShift) {
			a = mulc(a, __ldg(c.rot + e));
			b = mulc(b, __ldg(c.rot + e + 1));
		}
	}
	__stcs(reinterpret_cast<float4 *>(c.gout) + e / 2, make_float4(a.x, a.y, b.x, b.y));
}

// ------------------------------------------------------------------ one pass

// A hook that does nothing (passes / pass take hooks at fixed points of the pass list).
struct NoHook {
	__device__ __forceinline__ void operator()() const {}
};


// Twiddle rows stored for a pass of radix R: FP32 register butterflies store exponents 1, 2, 4, 8,
// 16 (< R); FP64 passes (bound by FP64 arithmetic, not memory) and direct passes store every
// exponent 1..R-1.
template <typename T, int R>
struct TwRows {
	static constexpr bool kPow2 = Specialised<R>::value && sizeof(T) == 4;
	static constexpr int value = kPow2 ? (R > 32 ? 6 : R > 16 ? 5 : R > 8 ? 4 : R > 4 ? 3 : R > 2 ? 2 : 1) : R - 1;
};

// v[r] *= W_{NS R}^{m r}.  FP32: rows W^{m}, W^{2m}, W^{4m}, W^{8m}, W^{16m} are loaded, the other
// powers are products w_r = w_{r - lowbit(r)} * w_{lowbit(r)} (at most 4 products deep): a quarter
// to a half of the twiddle loads, which were most of the L1 traffic of the memory-bound FP32
// kernels.  FP64: every power is loaded (the products would cost FP64 arithmetic, the bound).
template <typename T, int R, int NS, int TWO>
__device__ __forceinline__ void apply_twiddles(typename Cx<T>::C (&v)[R], const typename Cx<T>::C *tw, int m) {
	using C = typename Cx<T>::C;
	if constexpr (!TwRows<T, R>::kPow2) {
#pragma unroll
		for (int r = 1; r < R; ++r) v[r] = mul(v[r], __ldg(tw + TWO + (r - 1) * NS + m));
	} else {
		C pw[TwRows<T, R>::value];
#pragma unroll
		for (int b = 0; b < TwRows<T, R>::value; ++b) pw[b] = __ldg(tw + TWO + b * NS + m);
		C w[R];
#pragma unroll
		for (int r = 1; r < R; ++r) {
			const int lb = r & -r;
			const int b = lb == 1 ? 0 : lb == 2 ? 1 : lb == 4 ? 2 : lb == 8 ? 3 : lb == 16 ? 4 : 5;
			w[r] = r == lb ? pw[b] : mul(w[r - lb], pw[b]);
			v[r] = mul(v[r], w[r]);
		}
	}
}

// `loaded` runs once every thread has its inputs of the pass in registers (the split-staged
// kernel refills the work buffer there, during the last pass).  A first pass that reads part of
// its input from the buffer it writes (split staging) waits for every thread's loads first.
template <typename T, int N, int THREADS, int R, int NS, int TWO, int ROOTS, int SRC, int DST, int KIND, bool CIN,
          bool COUT, bool ODD, int EMAX, class Loaded = NoHook>
__device__ __forceinline__ void pass(const Ctx<T, KIND, CIN, COUT> &c, const typename Cx<T>::C *tw,
                                     const typename Cx<T>::C *roots, const Loaded &loaded = Loaded()) {
	using C = typename Cx<T>::C;
	constexpr int PS = Cx<T>::kPadShift;
	constexpr int NB = N / R;
	constexpr bool IN_PLACE = (SRC == kSmem || SRC >= kStageSplit) && DST == kSmem;
	if constexpr (Specialised<R>::value) {
		constexpr int NBPT = (NB + THREADS - 1) / THREADS;  // butterflies per thread
		constexpr bool GUARD = NB % THREADS != 0;
		// 128-bit global access: when a thread holds two or more butterflies of a pass that reads
		// or writes HBM (the first / last pass), it takes adjacent pairs (j, j + 1), whose
		// elements j + r NB and j + 1 + r NB (and, in the last pass, outputs) are one 16-byte
		// load or store; transforms that do not start on a 16-byte boundary use 8-byte accesses
		constexpr int NPAIR = NB / 2;
		constexpr bool PAIRED = sizeof(T) == 4 && !ODD && (SRC == kGlobal || DST == kGlobal) && NB % 2 == 0 &&
		                        NBPT % 2 == 0 && 2 * ((NPAIR + THREADS - 1) / THREADS) == NBPT;
		constexpr bool PGUARD = NPAIR % THREADS != 0;
		auto jof = [&c](int i) { return PAIRED ? 2 * (c.t + (i >> 1) * THREADS) + (i & 1) : c.t + i * THREADS; };
		auto okof = [&c](int i) {
			return PAIRED ? (!PGUARD || c.t + (i >> 1) * THREADS < NPAIR) : (!GUARD || c.t + i * THREADS < NB);
		};
		C v[NBPT][R];
		if constexpr (PAIRED && SRC == kGlobal) {
			const bool al = (reinterpret_cast<unsigned long long>(c.gin) & 15ull) == 0;
#pragma unroll
			for (int i = 0; i < NBPT; i += 2) {
				const int j = jof(i);
				if (c.valid && okof(i)) {
					if (al) {
#pragma unroll
						for (int r = 0; r < R; ++r)
							gload2<T, KIND, CIN, COUT, ODD>(c, j + r * NB, v[i][r], v[i + 1][r]);
					} else {
#pragma unroll
						for (int r = 0; r < R; ++r) {
							v[i][r] = gload<T, KIND, CIN, COUT, ODD>(c, j + r * NB);
							v[i + 1][r] = gload<T, KIND, CIN, COUT, ODD>(c, j + 1 + r * NB);
						}
					}
				}
			}
		} else {
#pragma unroll
			for (int i = 0; i < NBPT; ++i) {
				const int j = jof(i);
				if (c.valid && okof(i)) {
#pragma unroll
					for (int r = 0; r < R; ++r) {
						if constexpr (SRC == kSmem) v[i][r] = c.sm[pidx<PS>(j + r * NB)];
						else if constexpr (is_stage(SRC)) v[i][r] = sload_row<SRC, NB>(c, j, r);
						else v[i][r] = gload<T, KIND, CIN, COUT, ODD>(c, j + r * NB);
					}
				}
			}
		}
		loaded();
#pragma unroll
		for (int i = 0; i < NBPT; ++i) {
			const int j = jof(i);
			if (c.valid && okof(i)) {
				if constexpr (NS > 1) apply_twiddles<T, R, NS, TWO>(v[i], tw, j % NS);
				dft<R>(v[i]);
			}
		}
		if constexpr (IN_PLACE) __syncthreads();
		if constexpr (PAIRED && DST == kGlobal) {
			// the last pass (NS = NB): butterfly j writes outputs j + r NS, so a pair's outputs sit
			// side by side
			static_assert(NS == NB, "paired stores are for the last pass");
			const bool al = (reinterpret_cast<unsigned long long>(c.gout) & 15ull) == 0;
#pragma unroll
			for (int i = 0; i < NBPT; i += 2) {
				const int j = jof(i);
				if (c.valid && okof(i)) {
					if (al) {
#pragma unroll
						for (int r = 0; r < R; ++r)
							gstore2<T, KIND, CIN, COUT, ODD>(c, j + r * NS, v[i][r], v[i + 1][r]);
					} else {
#pragma unroll
						for (int r = 0; r < R; ++r) {
							gstore<T, KIND, CIN, COUT, ODD>(c, j + r * NS, v[i][r]);
							gstore<T, KIND, CIN, COUT, ODD>(c, j + 1 + r * NS, v[i + 1][r]);
						}
					}
				}
			}
		} else {
#pragma unroll
			for (int i = 0; i < NBPT; ++i) {
				const int j = jof(i);
				if (c.valid && okof(i)) {
					const int base = (j / NS) * NS * (R - 1) + j;  // (j - j mod NS) * R + j mod NS
#pragma unroll
					for (int r = 0; r < R; ++r) {
						if constexpr (DST == kSmem) c.sm[pidx<PS>(base + r * NS)] = v[i][r];
						else gstore<T, KIND, CIN, COUT, ODD>(c, base + r * NS, v[i][r]);
					}
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
				else if constexpr (is_stage(SRC)) s = sload_row<SRC, NB>(c, j, 0);
				else s = gload<T, KIND, CIN, COUT, ODD>(c, j);
				int w = 0;
				for (int r = 1; r < R; ++r) {
					C x;
					if constexpr (SRC == kSmem) x = c.sm[pidx<PS>(j + r * NB)];
					else if constexpr (is_stage(SRC)) x = sload_row<SRC, NB>(c, j, r);
					else x = gload<T, KIND, CIN, COUT, ODD>(c, j + r * NB);
					if constexpr (NS > 1) x = mul(x, __ldg(tw + TWO + (r - 1) * NS + m));
					w += k;
					if (w >= R) w -= R;
					s = add(s, mul(x, __ldg(roots + ROOTS + w)));
				}
				acc[i] = s;
			}
		}
		loaded();
		if constexpr (IN_PLACE) __syncthreads();
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

// Twiddle slots used by a pass of radix R after NS points (none for the first pass): rows of
// the exponents 1, 2, 4, 8 below R for register butterflies, every exponent 1..R-1 for direct
// passes.
template <typename T, int R, int NS>
struct TwCount {
	static constexpr int value = NS > 1 ? NS * TwRows<T, R>::value : 0;
};
template <int R>
struct RootCount {
	static constexpr int value = Specialised<R>::value ? 0 : R;
};

// ------------------------------------------------------------------ real split fused into a pass
//
// RealFFT (not the half-shift variant) pairs bin k with bin H - k in its forward split and input k
// with H - k in its inverse pre-twiddle (signalsmith-fft.h:459-472, :477-492).  In the last pass
// (radix R, NS = H/R) butterfly j produces X[j + r NS] and butterfly NS - j produces the mirrors
// X[H - j - r NS] = X[(NS - j) + (R - 1 - r) NS]; in the first pass butterfly j reads z[j + r NB]
// and butterfly NB - j reads the mirrors.  A thread that runs both butterflies of such a pair (a
// unit: j and M - j, M = NS or NB; j = 0 and j = M/2 are their own mirrors) has both ends of
// every pair in registers, so the split or pre-twiddle needs no shared-memory round trip.  A unit
// holds 2R values; the planner uses these passes for R <= 8.  Each output pair is computed once,
// with the reference's formulas; the self-paired bin H/2 gets the reference's surviving write.

// Forward split of the pair (i, H - i), 1 <= i <= H/2, from Z[i] and Z[H - i].
// (w = rtw[i], loaded by the caller ahead of its stores)
template <typename T, int H>
__device__ __forceinline__ void split_pair_w(typename Cx<T>::C *out, int i, typename Cx<T>::C w, typename Cx<T>::C zi,
                                             typename Cx<T>::C zci) {
	using C = typename Cx<T>::C;
	const C zc = conj(zci);
	const C odd = scale(add(zi, zc), T(0.5));
	const C even = scale(sub(zi, zc), T(0.5));
	const C e = mul(even, w);
	if (2 * i != H) __stcs(out + i, add(odd, e));
	__stcs(out + (H - i), conj(sub(odd, e)));
}
template <typename T, int H>
__device__ __forceinline__ void split_pair(typename Cx<T>::C *out, const typename Cx<T>::C *rtw, int i,
                                           typename Cx<T>::C zi, typename Cx<T>::C zci) {
	split_pair_w<T, H>(out, i, __ldg(rtw + i), zi, zci);
}

// Inverse pre-twiddle of the pair (i, H - i), 1 <= i <= H/2: the (conjugated) first-pass inputs
// z[i] and z[H - i] from bins B[i], B[H - i].
template <typename T, int H>
__device__ __forceinline__ void pretwiddle_pair(const typename Cx<T>::C *in, const typename Cx<T>::C *rtw, int i,
                                                typename Cx<T>::C &zi, typename Cx<T>::C &zci) {
	using C = typename Cx<T>::C;
	const C v = __ldcs(in + i);
	const C v2c = conj(__ldcs(in + (H - i)));
	const C odd = add(v, v2c);
	const C even = mulc(sub(v, v2c), __ldg(rtw + i));
	zi = conj(add(odd, even));
	zci = sub(odd, even);
}

// Units: unit 0 holds the self-mirrored butterflies 0 and (for even M) M/2, unit u >= 1 holds u
// and M - u, so every unit has two butterflies (but unit 0 of an odd M) and M/2 rounded up units
// cover the pass.

// Forward split of the outputs X[j + r NS] of a self-mirrored butterfly j (0 or NS/2).
template <typename T, int H, int R, int NS>
__device__ __forceinline__ void split_self(typename Cx<T>::C *out, const typename Cx<T>::C *rtw, int j,
                                           const typename Cx<T>::C (&v)[R]) {
	if (j == 0) {
		__stcs(out, mkc(v[0].x + v[0].y, v[0].x - v[0].y));  // DC and Nyquist in bin 0
#pragma unroll
		for (int r = 1; r < R; ++r)
			if (r <= R - r) split_pair<T, H>(out, rtw, r * NS, v[r], v[R - r]);
	} else {
#pragma unroll
		for (int r = 0; r < R; ++r)
			if (r <= R - 1 - r) split_pair<T, H>(out, rtw, j + r * NS, v[r], v[R - 1 - r]);
	}
}

// Last pass of a RealFFT forward with the split fused: shared memory -> H bins in HBM.
template <typename T, int H, int THREADS, int R, int NS, int TWO, int KIND, bool CIN, bool COUT>
__device__ __forceinline__ void pass_last_r2c(const Ctx<T, KIND, CIN, COUT> &c, const typename Cx<T>::C *tw) {
	using C = typename Cx<T>::C;
	constexpr int PS = Cx<T>::kPadShift;
	constexpr int U = (NS + 1) / 2, UPT = (U + THREADS - 1) / THREADS;
	static_assert(Specialised<R>::value && NS * R == H, "fused split needs a register butterfly as the last pass");
	C *out = reinterpret_cast<C *>(c.gout);
#pragma unroll
	for (int q = 0; q < UPT; ++q) {
		const int u = c.t + q * THREADS;
		if (c.valid && u < U) {
			const int j1 = u, j2 = u == 0 ? NS / 2 : NS - u;
			const bool has2 = u != 0 || NS % 2 == 0;
			C v1[R], v2[R], w[R];
#pragma unroll
			for (int r = 0; r < R; ++r) {
				v1[r] = c.sm[pidx<PS>(j1 + r * NS)];
				v2[r] = has2 ? c.sm[pidx<PS>(j2 + r * NS)] : v1[r];
			}
			// the split twiddles of the pairs, loaded ahead of the stores (which could alias them
			// as far as the compiler can tell)
			if (u != 0) {
#pragma unroll
				for (int r = 0; r < R; ++r) {
					const int k = j1 + r * NS, mk = H - k;
					w[r] = __ldg(c.rtw + (k < mk ? k : mk));
				}
			}
			if constexpr (NS > 1) {
				apply_twiddles<T, R, NS, TWO>(v1, tw, j1);
				if (has2) apply_twiddles<T, R, NS, TWO>(v2, tw, j2);
			}
			dft<R>(v1);
			if (has2) dft<R>(v2);
			if (u != 0) {
#pragma unroll
				for (int r = 0; r < R; ++r) {
					const int k = j1 + r * NS, mk = H - k;
					if (k < mk) split_pair_w<T, H>(out, k, w[r], v1[r], v2[R - 1 - r]);
					else split_pair_w<T, H>(out, mk, w[r], v2[R - 1 - r], v1[r]);
				}
			} else {
				split_self<T, H, R, NS>(out, c.rtw, 0, v1);
				if (has2) split_self<T, H, R, NS>(out, c.rtw, NS / 2, v2);
			}
		}
	}
}

// Inverse pre-twiddle of the inputs z[j + r NB] of a self-mirrored butterfly j (0 or NB/2).
template <typename T, int H, int R, int NB>
__device__ __forceinline__ void pretwiddle_self(const typename Cx<T>::C *in, const typename Cx<T>::C *rtw, int j,
                                                typename Cx<T>::C (&v)[R]) {
	using C = typename Cx<T>::C;
	if (j == 0) {
		const C x = __ldcs(in);
		v[0] = conj(mkc(x.x + x.y, x.x - x.y));
#pragma unroll
		for (int r = 1; r < R; ++r) {
			C unused;
			if (r < R - r) pretwiddle_pair<T, H>(in, rtw, r * NB, v[r], v[R - r]);
			else if (r == R - r) pretwiddle_pair<T, H>(in, rtw, r * NB, unused, v[r]);
		}
	} else {
#pragma unroll
		for (int r = 0; r < R; ++r) {
			C unused;
			if (r < R - 1 - r) pretwiddle_pair<T, H>(in, rtw, j + r * NB, v[r], v[R - 1 - r]);
			else if (r == R - 1 - r) pretwiddle_pair<T, H>(in, rtw, j + r * NB, unused, v[r]);
		}
	}
}

// First pass of a RealFFT inverse with the pre-twiddle fused: H bins in HBM -> shared memory.
template <typename T, int H, int THREADS, int R, int KIND, bool CIN, bool COUT>
__device__ __forceinline__ void pass_first_c2r(const Ctx<T, KIND, CIN, COUT> &c) {
	using C = typename Cx<T>::C;
	constexpr int PS = Cx<T>::kPadShift;
	constexpr int NB = H / R, U = (NB + 1) / 2, UPT = (U + THREADS - 1) / THREADS;
	static_assert(Specialised<R>::value && NB * R == H, "fused pre-twiddle needs a register butterfly first");
	const C *in = reinterpret_cast<const C *>(c.gin);
	// every unit's HBM loads first: the shared-memory stores could alias them as far as the
	// compiler can tell, which would otherwise serialise one HBM round trip per unit
	C v1[UPT][R], v2[UPT][R];
#pragma unroll
	for (int q = 0; q < UPT; ++q) {
		const int u = c.t + q * THREADS;
		if (c.valid && u < U) {
			const int j1 = u;
			const bool has2 = u != 0 || NB % 2 == 0;
			if (u != 0) {
#pragma unroll
				for (int r = 0; r < R; ++r) {
					const int k = j1 + r * NB, mk = H - k;
					if (k < mk) pretwiddle_pair<T, H>(in, c.rtw, k, v1[q][r], v2[q][R - 1 - r]);
					else pretwiddle_pair<T, H>(in, c.rtw, mk, v2[q][R - 1 - r], v1[q][r]);
				}
			} else {
				pretwiddle_self<T, H, R, NB>(in, c.rtw, 0, v1[q]);
				if (has2) pretwiddle_self<T, H, R, NB>(in, c.rtw, NB / 2, v2[q]);
			}
		}
	}
#pragma unroll
	for (int q = 0; q < UPT; ++q) {
		const int u = c.t + q * THREADS;
		if (c.valid && u < U) {
			const int j1 = u, j2 = u == 0 ? NB / 2 : NB - u;
			const bool has2 = u != 0 || NB % 2 == 0;
			dft<R>(v1[q]);
#pragma unroll
			for (int r = 0; r < R; ++r) c.sm[pidx<PS>(j1 * R + r)] = v1[q][r];
			if (has2) {
				dft<R>(v2[q]);
#pragma unroll
				for (int r = 0; r < R; ++r) c.sm[pidx<PS>(j2 * R + r)] = v2[q][r];
			}
		}
	}
	__syncthreads();
}

// All passes of the transform; `after_first` runs (on every thread) once the first pass has
// consumed its input, `last_loaded` once every thread holds the inputs of the last (register or
// direct) pass.
template <typename T, int N, int THREADS, int NS, int TWO, int ROOTS, int FIRST_SRC, int LAST_DST, int KIND, bool CIN,
          bool COUT, bool ODD, int EMAX, int R, int... Rest, class Hook = NoHook, class LastLoaded = NoHook>
__device__ __forceinline__ void passes(const Ctx<T, KIND, CIN, COUT> &c, const typename Cx<T>::C *tw,
                                       const typename Cx<T>::C *roots, const Hook &after_first = Hook(),
                                       const LastLoaded &last_loaded = LastLoaded()) {
	constexpr bool last = sizeof...(Rest) == 0;
	constexpr int SRC = NS == 1 ? FIRST_SRC : kSmem;
	constexpr int DST = last ? LAST_DST : kSmem;
	static_assert(!(SRC == kFusedC2R && last) && !(DST == kFusedR2C && NS == 1), "fused split needs two passes or more");
	if constexpr (SRC == kFusedC2R) pass_first_c2r<T, N, THREADS, R, KIND, CIN, COUT>(c);
	else if constexpr (DST == kFusedR2C) pass_last_r2c<T, N, THREADS, R, NS, TWO, KIND, CIN, COUT>(c, tw);
	else if constexpr (last) pass<T, N, THREADS, R, NS, TWO, ROOTS, SRC, DST, KIND, CIN, COUT, ODD, EMAX>(c, tw, roots, last_loaded);
	else pass<T, N, THREADS, R, NS, TWO, ROOTS, SRC, DST, KIND, CIN, COUT, ODD, EMAX>(c, tw, roots);
	if constexpr (NS == 1) after_first();
	if constexpr (!last)
		passes<T, N, THREADS, NS * R, TWO + TwCount<T, R, NS>::value, ROOTS + RootCount<R>::value, FIRST_SRC, LAST_DST,
		       KIND, CIN, COUT, ODD, EMAX, Rest...>(c, tw, roots, NoHook(), last_loaded);
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
	constexpr int PPT = NPAIRS > THREADS ? (NPAIRS + THREADS - 1) / THREADS : 1;  // pairs a thread takes
	C *out = reinterpret_cast<C *>(c.gout);
	if (!c.valid) return;
	if (!MOD && c.t == 0) {
		const C z0 = c.sm[0];
		__stcs(out, mkc(z0.x + z0.y, z0.x - z0.y));
	}
	// every load of the thread first: the stores below could alias them as far as the compiler
	// can tell, which would otherwise serialise the pairs
	C zi[PPT], zc[PPT], w[PPT];
#pragma unroll
	for (int q = 0; q < PPT; ++q) {
		const int p = c.t + q * THREADS;
		if (p < NPAIRS) {
			const int i = S + p;
			const int ci = MOD ? H - 1 - i : H - i;
			zi[q] = c.sm[pidx<PS>(i)];
			zc[q] = conj(c.sm[pidx<PS>(ci)]);
			w[q] = __ldg(rtw + i);
		}
	}
#pragma unroll
	for (int q = 0; q < PPT; ++q) {
		const int p = c.t + q * THREADS;
		if (p < NPAIRS) {
			const int i = S + p;
			const int ci = MOD ? H - 1 - i : H - i;
			const C odd = scale(add(zi[q], zc[q]), T(0.5));
			const C even = scale(sub(zi[q], zc[q]), T(0.5));
			const C e = mul(even, w[q]);
			bool wi, wci;
			pair_writes(i, ci, S, LAST, wi, wci);
			if (wi) __stcs(out + i, add(odd, e));
			if (wci) __stcs(out + ci, conj(sub(odd, e)));
		}
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
	constexpr int PPT = NPAIRS > THREADS ? (NPAIRS + THREADS - 1) / THREADS : 1;  // pairs a thread takes
	const C *in = STAGED ? c.st : reinterpret_cast<const C *>(c.gin);
	if (c.valid) {
		// every HBM load of the thread first: the shared-memory stores below could alias them as
		// far as the compiler can tell, which would otherwise serialise one HBM round trip per pair
		C v[PPT], v2c[PPT], w[PPT], v0;
		if (!MOD && c.t == 0) v0 = STAGED ? in[0] : __ldcs(in);
#pragma unroll
		for (int q = 0; q < PPT; ++q) {
			const int p = c.t + q * THREADS;
			if (p < NPAIRS) {
				const int i = S + p;
				const int ci = MOD ? H - 1 - i : H - i;
				v[q] = STAGED ? in[i] : __ldcs(in + i);
				v2c[q] = conj(STAGED ? in[ci] : __ldcs(in + ci));
				w[q] = __ldg(rtw + i);
			}
		}
		if (!MOD && c.t == 0) c.sm[0] = conj(mkc(v0.x + v0.y, v0.x - v0.y));
#pragma unroll
		for (int q = 0; q < PPT; ++q) {
			const int p = c.t + q * THREADS;
			if (p < NPAIRS) {
				const int i = S + p;
				const int ci = MOD ? H - 1 - i : H - i;
				const C odd = add(v[q], v2c[q]);
				const C even = mulc(sub(v[q], v2c[q]), w[q]);
				bool wi, wci;
				pair_writes(i, ci, S, LAST, wi, wci);
				// stored conjugated: the passes run forward on conj(data)
				if (wi) c.sm[pidx<PS>(i)] = conj(add(odd, even));
				if (wci) c.sm[pidx<PS>(ci)] = sub(odd, even);
			}
		}
	}
	__syncthreads();
}

// ------------------------------------------------------------------ the batch kernel

// SMEM_STRIDE: padded complex slots per transform.  EMAX bounds the values a thread holds in
// one pass.  MINB: CTAs the compiler must fit per SM (caps registers; more resident warps hide the
// first pass's HBM latency).
template <typename T, int N, int THREADS, int PER_CTA, int SMEM_STRIDE, int KIND, bool INV, bool ODD, int EMAX,
          int MINB, bool FUSE, int... Rs>
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
		if (a.offs) {
			oin = a.offs[gi];
			oout = a.offs_out ? a.offs_out[gi] : oin;
		} else {
			oin = gi * a.in_dist, oout = gi * a.out_dist;
		}
	}
	c.gin = reinterpret_cast<const T *>(a.in) + oin;
	c.gout = reinterpret_cast<T *>(a.out) + oout;
	c.rot = reinterpret_cast<const C *>(a.rot);
	const C *tw = reinterpret_cast<const C *>(a.tw);
	const C *roots = reinterpret_cast<const C *>(a.roots);
	const C *rtw = reinterpret_cast<const C *>(a.rtw);
	c.rtw = rtw;
	prefetch_ahead<T, PER_CTA, THREADS * PER_CTA>(a);
	if constexpr (FUSE) {
		// real split / pre-twiddle inside the last / first pass (KIND == kReal, even length)
		static_assert(KIND == kReal && !ODD, "fused split is for RealFFT of even length");
		passes<T, N, THREADS, 1, 0, 0, C2R ? kFusedC2R : kGlobal, R2C ? kFusedR2C : kGlobal, KIND, INV, INV, ODD, EMAX,
		       Rs...>(c, tw, roots);
	} else {
		if constexpr (C2R) real_pre<T, N, THREADS, KIND, INV, INV>(c, rtw);
		passes<T, N, THREADS, 1, 0, 0, C2R ? kSmem : kGlobal, R2C ? kSmem : kGlobal, KIND, INV, INV, ODD, EMAX, Rs...>(
		    c, tw, roots);
		if constexpr (R2C) real_post<T, N, THREADS, KIND, INV, INV>(c, rtw);
	}
}

// ------------------------------------------------------------------ uneven batches: a work-item queue

// Per-member device tables of a queue kernel.
struct QSched {
	const void *tw;          // pass twiddles
	const void *roots;       // direct-pass roots
	long long n;             // complex points per transform
	long long threads;       // threads per transform
};
// The queue of one class launch: item b (CTA b) runs member kidx[b]; thread t of item b works on
// the transform whose first complex element is toff[b * CTA + t] elements into in and out
// (-1: none -- a partial item, or threads past the member's transforms per CTA).  Both loads
// depend on blockIdx and threadIdx only, so a thread issues its first data load one load after
// it starts.
struct QueueArgs {
	const void *in;
	void *out;
	const int *kidx;
	const int *toff;
	long long nitems;
	const QSched *sch;
	long long pf_dist;       // after its first pass, CTA b prefetches into L2 the inputs of item
	                         // b + pf_dist (0 = off)
};

// A member schedule of a queue kernel: N points, THREADS threads a transform, SMEM_STRIDE padded
// slots a transform, EMAX values a thread, radix list Rs.
template <int N, int THREADS, int SMEM_STRIDE, int EMAX, int... Rs>
struct QS {};

// Inputs of item pf_dist ahead: thread t takes the 128-byte lines r, r + THREADS, ... of the
// transform it would work on (r = its index in that transform's threads), so every address lies
// inside a transform of that item.
template <typename T, int CTA>
__device__ __forceinline__ void queue_prefetch(const QueueArgs &a) {
	if (a.pf_dist <= 0) return;
	const long long b = (long long)blockIdx.x + a.pf_dist;
	if (b >= a.nitems) return;
	const int o = a.toff[b * CTA + threadIdx.x];
	if (o < 0) return;
	const QSched &s = a.sch[a.kidx[b]];
	const long long th = s.threads;
	const long long lines = (2 * s.n * (long long)sizeof(T) + 127) / 128;
	const unsigned char *p = reinterpret_cast<const unsigned char *>(a.in) + 2ll * o * (long long)sizeof(T);
	for (long long q = (long long)threadIdx.x % th; q < lines; q += th) prefetch_l2(p + q * 128);
}

template <typename T, bool INV, int CTA, int I, class... Ss>
struct QDispatch {
	static __device__ __forceinline__ void run(const QueueArgs &, int, int, unsigned char *) {}
};
template <typename T, bool INV, int CTA, int I, int N, int THREADS, int SMEM_STRIDE, int EMAX, int... Rs,
          class... Rest>
struct QDispatch<T, INV, CTA, I, QS<N, THREADS, SMEM_STRIDE, EMAX, Rs...>, Rest...> {
	static __device__ __forceinline__ void run(const QueueArgs &a, int k, int off, unsigned char *smem) {
		if (k != I) {
			QDispatch<T, INV, CTA, I + 1, Rest...>::run(a, k, off, smem);
			return;
		}
		using C = typename Cx<T>::C;
		// transform g of the item: threads [g THREADS, (g + 1) THREADS); threads without one only
		// join the barriers
		const int g = threadIdx.x / THREADS;
		Ctx<T, kComplex, INV, INV> c;
		c.t = threadIdx.x - g * THREADS;
		c.valid = off >= 0;
		c.sm = reinterpret_cast<C *>(smem) + g * SMEM_STRIDE;
		const long long o = c.valid ? 2ll * off : 0;
		c.gin = reinterpret_cast<const T *>(a.in) + o;
		c.gout = reinterpret_cast<T *>(a.out) + o;
		c.rot = nullptr;
		c.rtw = nullptr;
		c.st = nullptr;
		const QSched &s = a.sch[I];
		auto pf = [&a] { queue_prefetch<T, CTA>(a); };
		passes<T, N, THREADS, 1, 0, 0, kGlobal, kGlobal, kComplex, INV, INV, false, EMAX, Rs...>(
		    c, reinterpret_cast<const C *>(s.tw), reinterpret_cast<const C *>(s.roots), pf);
	}
};

// One launch runs every item of an uneven batch whose schedules share this CTA shape: CTA b takes
// item b (the host orders the queue longest transforms first, so the hardware's in-order CTA
// dispatch hands out the long work first and the short work fills the last wave) and runs the
// size-specialised passes of the item's schedule; the schedules are the compile-time members Ss.
template <typename T, bool INV, int CTA, int MINB, class... Ss>
__global__ void __launch_bounds__(CTA, MINB) queue(const QueueArgs a) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	const long long b = blockIdx.x;
	const int off = a.toff[b * CTA + threadIdx.x];
	const int k = a.kidx[b];
	QDispatch<T, INV, CTA, 0, Ss...>::run(a, k, off, smem_raw);
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
// suspends for a bounded, hardware-defined time).  On the device the polling loop is one asm
// statement: as a C++ loop, the compiler moved address arithmetic of the code after it above
// it and kept the results live (the staged kernel went from ~69 to 93+ registers).
#if defined(__CUDA_ARCH__)
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long *bar, unsigned phase, unsigned limit) {
	unsigned ok;
	asm volatile(
	    "{\n\t"
	    ".reg .pred p, q;\n\t"
	    ".reg .u32 i;\n\t"
	    "mov.u32 i, 0;\n\t"
	    "mov.u32 %0, 0;\n"
	    "LAB_WAIT:\n\t"
	    "setp.ge.u32 q, i, %3;\n\t"
	    "@q bra LAB_DONE;\n\t"
	    "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
	    "add.u32 i, i, 1;\n\t"
	    "@!p bra LAB_WAIT;\n\t"
	    "mov.u32 %0, 1;\n"
	    "LAB_DONE:\n\t"
	    "}"
	    : "=r"(ok)
	    : "r"(smem_u32(bar)), "r"(phase), "r"(limit)
	    : "memory");
	return ok != 0;
}
#else
inline bool mbar_wait_bounded(unsigned long long *bar, unsigned phase, unsigned limit) {
	for (unsigned i = 0; i < limit; ++i)
		if (mbar_try_wait(bar, phase)) return true;
	return false;
}
#endif

template <int R, int... Rest>
struct FirstRadix {
	static constexpr int value = R;
};

// The batch kernel with asynchronous input staging: persistent CTAs walk the groups of PER_CTA
// transforms; each group's input (contiguous in HBM) arrives in an unpadded staging buffer by
// one bulk copy, and the copy of the next group is issued as soon as the first pass (or the
// real pre-twiddle) has read the current one, so the HBM load overlaps the remaining passes.
// Requires in_bytes % 16 == 0 and 16-byte aligned input.  A bounded wait that runs out sets
// *err and the CTA returns without writing.  (Inside the persistent loop the compiler keeps far
// more registers live than one pass needs; MINB caps them.)
//
// SK > 0 (complex, one transform per CTA, a transform too long for a staging buffer and a work
// buffer of its whole size): only rows r < SK of the first pass (elements j + r NB, the first
// SK NB elements) are staged; rows r >= SK arrive by a second bulk copy into the start of the work
// buffer, issued once every thread holds the previous group's last-pass inputs.  The first pass
// reads both and, after a barrier, writes the work buffer.
template <typename T, int N, int THREADS, int PER_CTA, int SMEM_STRIDE, int KIND, bool INV, int EMAX, int MINB, int SK,
          int... Rs>
__global__ void __launch_bounds__(THREADS *PER_CTA, MINB) batch_staged(const Args a) {
	using C = typename Cx<T>::C;
	constexpr bool REAL = KIND != kComplex;
	constexpr bool R2C = REAL && !INV, C2R = REAL && INV;
	constexpr int NB0 = N / FirstRadix<Rs...>::value;
	static_assert(SK == 0 || (!REAL && PER_CTA == 1 && SK < FirstRadix<Rs...>::value),
	              "split staging: complex, one transform per CTA, some rows in the work buffer");
	constexpr unsigned kStageBytes = (unsigned)SK * NB0 * sizeof(C);  // SK > 0: staged bytes per transform
	extern __shared__ __align__(16) unsigned char smem_raw[];
	__shared__ __align__(8) unsigned long long bar[2];  // staging buffer, rows in the work buffer
	const unsigned in_bytes = a.in_bytes;
	unsigned char *stage = smem_raw;
	const unsigned stage_bytes = SK ? kStageBytes : PER_CTA * in_bytes;
	C *work = reinterpret_cast<C *>(smem_raw + ((stage_bytes + 127u) & ~127u));
	const long long ngroups = (a.batch + PER_CTA - 1) / PER_CTA;
	const unsigned char *in = reinterpret_cast<const unsigned char *>(a.in);
	const int g = threadIdx.x / THREADS;
	Ctx<T, KIND, INV, INV> c;
	c.t = threadIdx.x - g * THREADS;
	c.sm = work + g * SMEM_STRIDE;
	c.st = reinterpret_cast<const C *>(stage + g * in_bytes);
	c.st2 = work;
	c.rot = reinterpret_cast<const C *>(a.rot);
	c.gin = nullptr;
	const C *tw = reinterpret_cast<const C *>(a.tw);
	const C *roots = reinterpret_cast<const C *>(a.roots);
	const C *rtw = reinterpret_cast<const C *>(a.rtw);
	// the staged part of group grp (all of it unless SK > 0) and, SK > 0, the rest
	auto issue = [&](long long grp) {
		const long long nt = a.batch - grp * PER_CTA < PER_CTA ? a.batch - grp * PER_CTA : PER_CTA;
		const unsigned char *src = in + grp * PER_CTA * (long long)in_bytes;
		bulk_load(stage, src, SK ? kStageBytes : (unsigned)(nt * in_bytes), &bar[0], a.drop_copy != 0);
	};
	auto issue_rest = [&](long long grp) {
		const unsigned char *src = in + grp * (long long)in_bytes + kStageBytes;
		bulk_load(work, src, in_bytes - kStageBytes, &bar[1], a.drop_copy != 0);
	};
	if (threadIdx.x == 0) {
		mbar_init(&bar[0], 1);
		if constexpr (SK > 0) mbar_init(&bar[1], 1);
		if (blockIdx.x < ngroups) {
			issue(blockIdx.x);
			if constexpr (SK > 0) issue_rest(blockIdx.x);
		}
	}
	__syncthreads();
	unsigned phase = 0;
	for (long long grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
		bool ok = mbar_wait_bounded(&bar[0], phase, a.spin_limit);
		if constexpr (SK > 0) ok = mbar_wait_bounded(&bar[1], phase, a.spin_limit) && ok;
		if (__syncthreads_or(!ok)) {
			if (threadIdx.x == 0) atomicOr(a.err, 1u);
			// let the copies in flight land
			mbar_wait_bounded(&bar[0], phase, a.spin_limit);
			if constexpr (SK > 0) mbar_wait_bounded(&bar[1], phase, a.spin_limit);
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
				// the rows the work buffer takes later: towards L2 now
				if constexpr (SK > 0)
					prefetch_l2_bulk(in + next * (long long)in_bytes + kStageBytes, in_bytes - kStageBytes);
			}
		};
		if constexpr (C2R) {
			real_pre<T, N, THREADS, KIND, INV, INV, true>(c, rtw);
			refill();
			passes<T, N, THREADS, 1, 0, 0, kSmem, kGlobal, KIND, INV, INV, false, EMAX, Rs...>(c, tw, roots);
		} else if constexpr (SK > 0) {
			auto refill_rest = [&]() {
				__syncthreads();  // every thread holds its last-pass inputs: the work buffer is free
				if (threadIdx.x == 0 && next < ngroups) {
					fence_async_smem();
					issue_rest(next);
				}
			};
			passes<T, N, THREADS, 1, 0, 0, kStageSplit + SK, kGlobal, KIND, INV, INV, false, EMAX, Rs...>(
			    c, tw, roots, refill, refill_rest);
		} else {
			passes<T, N, THREADS, 1, 0, 0, kStage, R2C ? kSmem : kGlobal, KIND, INV, INV, false, EMAX, Rs...>(c, tw, roots,
			                                                                                                refill);
		}
		if constexpr (R2C) real_post<T, N, THREADS, KIND, INV, INV>(c, rtw);
		__syncthreads();  // the work buffer is reused by the next group
	}
}


// ------------------------------------------------------------------ split-BF16 tensor-core pass

// The first pass (radix R0 <= 16, no twiddles) as a matrix product on the tensor cores.  Each
// butterfly j of transform g is one row of A: [Re x_r | Im x_r] for r < R0 (x_r = element
// j + r*NB), zero-padded to 32 columns; B is the radix-R0 DFT in the same real form, so row
// [Re y_k | Im y_k] of D = A B holds the butterfly's outputs.  FP32 operands do not feed the
// tensor cores, so each is split into three BF16 parts, x = x0 + x1 + x2 (8 significant bits
// each, exact to ~2^-24 |x|), and the six products x_a w_b with a + b <= 2 accumulate in FP32
// in tensor memory (the three dropped products are below 2^-24 relative).  128 rows form one
// M=128, N=32, K=16 tcgen05.mma tile; 6 products x 2 K-steps = 12 MMAs per tile, issued by one
// thread, completed on an mbarrier (bounded wait), read back with tcgen05.ld (one row per lane
// of warps 0-3) and written to shared memory in the Stockham order the next pass expects.
//
// Operand layout in shared memory: the no-swizzle K-major canonical layout, 8-row x 16-byte
// core matrices stored as 128 contiguous bytes; core matrices adjacent in K are kTcLbo bytes
// apart, 8-row groups kTcSbo bytes apart.  One A part is 128 x 32 BF16 = 8 KiB, one B part
// 32 x 32 BF16 = 2 KiB.
constexpr unsigned kTcLbo = 128, kTcSbo = 512;
constexpr unsigned kTcAPart = 8192, kTcBPart = 2048;
__host__ __device__ constexpr unsigned tc_off_a(int per_cta, int stride) {
	return ((unsigned)per_cta * (unsigned)stride * 8u + 1023u) & ~1023u;
}
// With a single 128-row tile per CTA the A parts share the work buffer's space (they are dead
// once the MMAs complete, before the read-back writes the work buffer); B follows both.
__host__ __device__ constexpr unsigned tc_off_b(int per_cta, int stride, int tiles) {
	return tiles == 1 ? (tc_off_a(per_cta, stride) > 3 * kTcAPart ? tc_off_a(per_cta, stride) : 3 * kTcAPart)
	                  : tc_off_a(per_cta, stride) + 3 * kTcAPart;
}
__host__ __device__ constexpr unsigned tc_smem_bytes(int per_cta, int stride, int tiles) {
	return tc_off_b(per_cta, stride, tiles) + 3 * kTcBPart + 16;
}
__host__ __device__ constexpr unsigned tc_core_off(int row, int k) {
	return (unsigned)(row >> 3) * kTcSbo + (unsigned)(k >> 3) * kTcLbo + (unsigned)(row & 7) * 16u + (unsigned)(k & 7) * 2u;
}
// instruction descriptor (kind::f16): D FP32 (bits 4-5 = 1), A and B BF16 (bits 7-9 = 1,
// 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28
constexpr unsigned kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ unsigned short f2bf(float x) {
	unsigned short r;
	asm("cvt.rn.bf16.f32 %0, %1;" : "=h"(r) : "f"(x));
	return r;
}
__device__ __forceinline__ float bf2f(unsigned short h) { return __uint_as_float((unsigned)h << 16); }
// shared-memory matrix descriptor: start >> 4 (bits 0-13), LBO >> 4 (16-29), SBO >> 4 (32-45),
// fixed 0b001 at bits 46-48, no swizzle (bits 61-63 = 0)
__device__ __forceinline__ unsigned long long tc_desc(const void *p) {
	return (unsigned long long)((smem_u32(p) & 0x3FFFFu) >> 4) | ((unsigned long long)(kTcLbo >> 4) << 16) |
	       ((unsigned long long)(kTcSbo >> 4) << 32) | (1ull << 46);
}
__device__ __forceinline__ void tmem_alloc32(unsigned *slot) {
	asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 32;" ::"r"(smem_u32(slot)) : "memory");
	asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc32(unsigned taddr) {
	asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 32;" ::"r"(taddr) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_mma(unsigned d, unsigned long long a, unsigned long long b, int acc) {
	asm volatile(
	    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
	    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
	    "l"(a), "l"(b), "r"(kTcIdesc), "r"(acc)
	    : "memory");
}
__device__ __forceinline__ void tc_commit(unsigned long long *bar) {
	asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
	             : "memory");
}
// 32 consecutive FP32 columns of this thread's lane; the wait is inside the same statement so
// the values are complete when they are used
__device__ __forceinline__ void tc_ld32(unsigned taddr, float (&v)[32]) {
	unsigned r[32];
	asm volatile(
	    "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
	    "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
	    "tcgen05.wait::ld.sync.aligned;"
	    : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
	      "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
	      "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
	      "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
	    : "r"(taddr)
	    : "memory");
#pragma unroll
	for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
#elif defined(SSFFT_EMULATION)
// Host emulation: tensor memory is one 128-lane x 32-column array (the emulator runs one CTA at
// a time), the MMA decodes the same descriptors the device would and computes in FP32.
unsigned short f2bf(float x);
float bf2f(unsigned short h);
extern float emu_tmem[128][32];
inline unsigned long long tc_desc(const void *p) {
	const unsigned off = (unsigned)(static_cast<const unsigned char *>(p) - smem_raw);
	return (unsigned long long)((off & 0x3FFFFu) >> 4) | ((unsigned long long)(kTcLbo >> 4) << 16) |
	       ((unsigned long long)(kTcSbo >> 4) << 32) | (1ull << 46);
}
inline void tmem_alloc32(unsigned *slot) {
	if (threadIdx.x == 0) *slot = 0;
}
inline void tmem_dealloc32(unsigned) {}
inline void tc_fence_before() {}
inline void tc_fence_after() {}
inline void tc_mma(unsigned d, unsigned long long a, unsigned long long b, int acc) {
	const unsigned m_dim = ((kTcIdesc >> 24) & 31u) << 4, n_dim = ((kTcIdesc >> 17) & 63u) << 3;
	auto elem = [](unsigned long long desc, unsigned row, unsigned k) {
		const unsigned start = (unsigned)(desc & 0x3FFFu) << 4;
		const unsigned lbo = (unsigned)((desc >> 16) & 0x3FFFu) << 4, sbo = (unsigned)((desc >> 32) & 0x3FFFu) << 4;
		const unsigned off = start + (row >> 3) * sbo + (k >> 3) * lbo + (row & 7) * 16 + (k & 7) * 2;
		unsigned short h;
		std::memcpy(&h, smem_raw + off, 2);
		return bf2f(h);
	};
	const unsigned lane0 = d >> 16, col0 = d & 0xFFFFu;
	for (unsigned m = 0; m < m_dim; ++m)
		for (unsigned n = 0; n < n_dim; ++n) {
			float sum = 0;
			for (unsigned k = 0; k < 16; ++k) sum += elem(a, m, k) * elem(b, n, k);
			float &dst = emu_tmem[lane0 + m][col0 + n];
			dst = acc ? dst + sum : sum;
		}
}
inline void tc_commit(unsigned long long *) {}
inline void tc_ld32(unsigned taddr, float (&v)[32]) {
	const unsigned lane = (taddr >> 16) + (threadIdx.x & 31u), col = taddr & 0xFFFFu;
	for (int i = 0; i < 32; ++i) v[i] = emu_tmem[lane][col + i];
}
#else
// host pass of the library build: declarations only (the kernels are device code)
unsigned short f2bf(float x);
float bf2f(unsigned short h);
unsigned long long tc_desc(const void *p);
void tmem_alloc32(unsigned *slot);
void tmem_dealloc32(unsigned taddr);
void tc_fence_before();
void tc_fence_after();
void tc_mma(unsigned d, unsigned long long a, unsigned long long b, int acc);
void tc_commit(unsigned long long *bar);
void tc_ld32(unsigned taddr, float (&v)[32]);
#endif

// x = x0 + x1 + x2 in BF16 parts
__device__ __forceinline__ void split3(float x, unsigned short &h0, unsigned short &h1, unsigned short &h2) {
	h0 = f2bf(x);
	float r = x - bf2f(h0);
	h1 = f2bf(r);
	r -= bf2f(h1);
	h2 = f2bf(r);
}

// Complex FP32 transforms whose first pass (radix R0 <= 16) runs on the tensor cores and whose
// remaining passes (Rest...) are the FP32 passes of the batch kernel.  At least 128 threads per
// CTA (rows of a tile are built and read back by threads 0-127).  A bounded wait that runs out
// sets *err, waits once more (bounded) for the MMAs in flight, frees the tensor memory and
// returns without writing.
template <int N, int THREADS, int PER_CTA, int SMEM_STRIDE, bool INV, int EMAX, int MINB, int R0, int... Rest>
__global__ void __launch_bounds__(THREADS *PER_CTA, MINB) batch_tc(const Args a) {
	using T = float;
	using C = float2;
	constexpr int CT = THREADS * PER_CTA;
	static_assert(CT >= 128, "the tensor-core pass reads 128 accumulator lanes");
	static_assert(R0 >= 2 && R0 <= 16 && N % R0 == 0, "first radix must fit the 32-column tile");
	constexpr int NB = N / R0;
	constexpr int ROWS = NB * PER_CTA;
	constexpr int TILES = (ROWS + 127) / 128;
	constexpr int PS = Cx<T>::kPadShift;
	constexpr bool LAST = sizeof...(Rest) == 0;
	extern __shared__ __align__(16) unsigned char smem_raw[];
	constexpr unsigned OFF_A = TILES == 1 ? 0 : tc_off_a(PER_CTA, SMEM_STRIDE);
	constexpr unsigned OFF_B = tc_off_b(PER_CTA, SMEM_STRIDE, TILES);
	constexpr unsigned OFF_BAR = OFF_B + 3 * kTcBPart;
	unsigned char *tile_a = smem_raw + OFF_A;
	unsigned char *tile_b = smem_raw + OFF_B;
	unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem_raw + OFF_BAR);
	unsigned *slot = reinterpret_cast<unsigned *>(smem_raw + OFF_BAR + 8);
	const int tid = threadIdx.x;
	const int warp = tid >> 5;

	if (tid == 0) mbar_init(bar, 1);
	if (warp == 0) tmem_alloc32(slot);
	// B parts: the split DFT matrix (K-major: row n = output column, k = input column)
	for (int idx = tid; idx < 32 * 32; idx += CT) {
		const int n = idx >> 5, k = idx & 31;
		unsigned short h0, h1, h2;
		split3(__ldg(a.tcb + idx), h0, h1, h2);
		const unsigned o = tc_core_off(n, k);
		*reinterpret_cast<unsigned short *>(tile_b + o) = h0;
		*reinterpret_cast<unsigned short *>(tile_b + kTcBPart + o) = h1;
		*reinterpret_cast<unsigned short *>(tile_b + 2 * kTcBPart + o) = h2;
	}
	fence_async_smem();
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const unsigned taddr = *slot;
	const float2 *in = reinterpret_cast<const float2 *>(a.in);
	unsigned phase = 0;
	bool failed = false;

	for (int tile = 0; tile < TILES; ++tile) {
		const int row = tile * 128 + tid;
		const int g = row / NB, j = row - (row / NB) * NB;
		const long long gi = (long long)blockIdx.x * PER_CTA + g;
		const bool live = tid < 128 && row < ROWS && gi < a.batch;
		if (tid < 128) {
			// this row of the three A parts, packed two BF16 per word: columns 0-15 real parts,
			// 16-31 imaginary parts (zero beyond R0, so no stale shared memory meets the zero
			// rows of B), built in two halves of 8 columns to keep few values live
			const float2 *src = in + (live ? (a.offs ? a.offs[gi] : gi * a.in_dist) / 2 : 0);
#pragma unroll
			for (int hf = 0; hf < 2; ++hf) {
				unsigned w[3][2][4];
#pragma unroll
				for (int q = 0; q < 4; ++q) w[0][0][q] = w[0][1][q] = w[1][0][q] = w[1][1][q] = w[2][0][q] = w[2][1][q] = 0;
				if (live) {
#pragma unroll
					for (int rr = 0; rr < 8; ++rr) {
						const int r = 8 * hf + rr;
						if (r < R0) {
							float2 v = __ldcs(src + j + r * NB);
							if (INV) v.y = -v.y;
							unsigned short h[2][3];
							split3(v.x, h[0][0], h[0][1], h[0][2]);
							split3(v.y, h[1][0], h[1][1], h[1][2]);
#pragma unroll
							for (int part = 0; part < 2; ++part)
#pragma unroll
								for (int sp = 0; sp < 3; ++sp) w[sp][part][rr >> 1] |= (unsigned)h[part][sp] << ((rr & 1) * 16);
						}
					}
				}
#pragma unroll
				for (int sp = 0; sp < 3; ++sp)
#pragma unroll
					for (int part = 0; part < 2; ++part) {
						// column block (part * 16 + 8 hf) / 8
						unsigned *dst = reinterpret_cast<unsigned *>(tile_a + sp * kTcAPart +
						                                             tc_core_off(tid, (2 * part + hf) * 8));
						dst[0] = w[sp][part][0];
						dst[1] = w[sp][part][1];
						dst[2] = w[sp][part][2];
						dst[3] = w[sp][part][3];
					}
			}
		}
		fence_async_smem();
		tc_fence_before();
		__syncthreads();
		if (tid == 0) {
			tc_fence_after();
			// smallest products first: (x2 w0), (x1 w1), (x0 w2), (x1 w0), (x0 w1), (x0 w0)
			const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
#pragma unroll
			for (int q = 0; q < 6; ++q)
#pragma unroll
				for (int ks = 0; ks < 2; ++ks)
					tc_mma(taddr, tc_desc(tile_a + pa[q] * kTcAPart + ks * 2 * kTcLbo),
					       tc_desc(tile_b + pb[q] * kTcBPart + ks * 2 * kTcLbo), q + ks > 0);
			tc_commit(bar);
		}
		const bool ok = mbar_wait_bounded(bar, phase, a.spin_limit);
		phase ^= 1u;
		if (__syncthreads_or(!ok)) {
			if (tid == 0) atomicOr(a.err, 1u);
			mbar_wait_bounded(bar, phase ^ 1u, a.spin_limit);  // let the MMAs in flight finish
			failed = true;
			break;
		}
		tc_fence_after();
		if (tid < 128) {
			float v[32];
			tc_ld32(taddr + ((unsigned)(warp * 32) << 16), v);
			if (live) {
				if constexpr (LAST) {
					C *dst = reinterpret_cast<C *>(a.out) +
					         (a.offs ? (a.offs_out ? a.offs_out[gi] : a.offs[gi]) : gi * a.out_dist) / 2;
#pragma unroll
					for (int k = 0; k < R0; ++k) __stcs(dst + j * R0 + k, make_float2(v[k], INV ? -v[16 + k] : v[16 + k]));
				} else {
					C *sm = reinterpret_cast<C *>(smem_raw) + g * SMEM_STRIDE;
#pragma unroll
					for (int k = 0; k < R0; ++k) sm[pidx<PS>(j * R0 + k)] = make_float2(v[k], v[16 + k]);
				}
			}
		}
		tc_fence_before();
		__syncthreads();
	}
	if (warp == 0) {
		tc_fence_after();
		tmem_dealloc32(taddr);
	}
	if (failed) return;
	if constexpr (!LAST) {
		const int g = tid / THREADS;
		const long long gi = (long long)blockIdx.x * PER_CTA + g;
		Ctx<T, kComplex, INV, INV> c;
		c.t = tid - g * THREADS;
		c.valid = gi < a.batch;
		c.sm = reinterpret_cast<C *>(smem_raw) + g * SMEM_STRIDE;
		long long oout = 0;
		if (c.valid) oout = a.offs ? (a.offs_out ? a.offs_out[gi] : a.offs[gi]) : gi * a.out_dist;
		c.gin = nullptr;
		c.gout = reinterpret_cast<T *>(a.out) + oout;
		c.rot = nullptr;
		passes<T, N, THREADS, R0, 0, RootCount<R0>::value, kSmem, kGlobal, kComplex, INV, INV, false, EMAX, Rest...>(
		    c, reinterpret_cast<const C *>(a.tw), reinterpret_cast<const C *>(a.roots));
	}
}

// Failure-free check of the tensor-core tile on its own: D = A B for one 128 x 32 x 32 tile of
// FP32 inputs (A row-major 128 x 32, B given as its transpose 32 x 32 in a.tcb, D row-major
// 128 x 32 to a.out), through the same split, layout, MMA and read-back as batch_tc.
template <int UNUSED = 0>
__global__ void __launch_bounds__(128, 1) tc_tile_check(const Args a) {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	unsigned char *tile_a = smem_raw;
	unsigned char *tile_b = smem_raw + 3 * kTcAPart;
	unsigned long long *bar = reinterpret_cast<unsigned long long *>(smem_raw + 3 * kTcAPart + 3 * kTcBPart);
	unsigned *slot = reinterpret_cast<unsigned *>(smem_raw + 3 * kTcAPart + 3 * kTcBPart + 8);
	const int tid = threadIdx.x, warp = tid >> 5;
	const float *A = static_cast<const float *>(a.in);
	if (tid == 0) mbar_init(bar, 1);
	if (warp == 0) tmem_alloc32(slot);
	for (int idx = tid; idx < 32 * 32; idx += 128) {
		unsigned short h0, h1, h2;
		split3(__ldg(a.tcb + idx), h0, h1, h2);
		const unsigned o = tc_core_off(idx >> 5, idx & 31);
		*reinterpret_cast<unsigned short *>(tile_b + o) = h0;
		*reinterpret_cast<unsigned short *>(tile_b + kTcBPart + o) = h1;
		*reinterpret_cast<unsigned short *>(tile_b + 2 * kTcBPart + o) = h2;
	}
	for (int k = 0; k < 32; ++k) {
		unsigned short h0, h1, h2;
		split3(A[tid * 32 + k], h0, h1, h2);
		const unsigned o = tc_core_off(tid, k);
		*reinterpret_cast<unsigned short *>(tile_a + o) = h0;
		*reinterpret_cast<unsigned short *>(tile_a + kTcAPart + o) = h1;
		*reinterpret_cast<unsigned short *>(tile_a + 2 * kTcAPart + o) = h2;
	}
	fence_async_smem();
	tc_fence_before();
	__syncthreads();
	tc_fence_after();
	const unsigned taddr = *slot;
	if (tid == 0) {
		const int pa[6] = {2, 1, 0, 1, 0, 0}, pb[6] = {0, 1, 2, 0, 1, 0};
		for (int q = 0; q < 6; ++q)
			for (int ks = 0; ks < 2; ++ks)
				tc_mma(taddr, tc_desc(tile_a + pa[q] * kTcAPart + ks * 2 * kTcLbo),
				       tc_desc(tile_b + pb[q] * kTcBPart + ks * 2 * kTcLbo), q + ks > 0);
		tc_commit(bar);
	}
	const bool ok = mbar_wait_bounded(bar, 0, a.spin_limit);
	if (__syncthreads_or(!ok)) {
		if (tid == 0) atomicOr(a.err, 1u);
		mbar_wait_bounded(bar, 0, a.spin_limit);
	} else {
		tc_fence_after();
		float v[32];
		tc_ld32(taddr + ((unsigned)(warp * 32) << 16), v);
		float *D = static_cast<float *>(a.out);
		for (int k = 0; k < 32; ++k) D[tid * 32 + k] = v[k];
	}
	tc_fence_before();
	__syncthreads();
	if (warp == 0) {
		tc_fence_after();
		tmem_dealloc32(taddr);
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
	long long pf_dist;  // CTA b prefetches into L2 the input of CTA b + pf_dist (0 = off)
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
	// Inter-pass twiddles W^{u0 k} for this CTA's G sub-transforms, k = kh KL + kl:
	// W^{u0 KL kh} and W^{u0 kl} (KH + KL values per sub-transform, from the two-level table)
	// in shared memory after the transforms' slots; the store then needs two shared loads and one
	// product per element instead of two scattered global loads.
	// rows of TWS = (KH + KL) | 1 slots: an odd stride, so the G sub-transforms of one k (adjacent
	// threads in the store loop) read different banks
	constexpr int KL = 16, KH = (N + KL - 1) / KL, TWS = (KH + KL) | 1;
	C *twk = sm_all + G * STRIDE;
	if constexpr (SSTORE && TWN > 1) {
		const C *twlo = reinterpret_cast<const C *>(a.twlo);
		const C *twhi = reinterpret_cast<const C *>(a.twhi);
		for (int idx = threadIdx.x; idx < G * (KH + KL); idx += CTA) {
			const int gg = idx / (KH + KL), q = idx - gg * (KH + KL);
			const long long u0 = u00 + gg;
			if (u0 < a.U0) {
				const unsigned long long e = q < KH ? (unsigned long long)q * KL : (unsigned long long)(q - KH);
				const unsigned long long t = ((unsigned long long)u0 * e) % (unsigned long long)TWN;
				twk[gg * TWS + q] = mul(__ldg(twhi + (t >> LB)), __ldg(twlo + (t & ((1ull << LB) - 1))));
			}
		}
		// (read after the passes' barriers)
	}
	if (a.pf_dist > 0 && (long long)blockIdx.x + a.pf_dist < (long long)gridDim.x) {
		// the input the CTA pf_dist blocks ahead will read, one 128-byte line per prefetch
		long long pc = (long long)blockIdx.x + a.pf_dist;
		const long long pu00 = (pc % blocks0) * G;
		pc /= blocks0;
		const long long pib = (pc / a.U1) * a.is2 + (pc % a.U1) * a.is1;
		constexpr int PER_LINE = 128 / (int)sizeof(C);
		if constexpr (SLOAD) {
			// G-element segments (is0 == 1), one per element e
			constexpr int SEG_LINES = (G + PER_LINE - 1) / PER_LINE;
			for (int k = threadIdx.x; k < N * SEG_LINES; k += CTA) {
				const int e = k / SEG_LINES, l = k - e * SEG_LINES;
				if (pu00 + l * PER_LINE < a.U0) prefetch_l2(in + pib + (pu00 + l * PER_LINE) * a.is0 + (long long)e * a.in_es);
			}
		} else {
			// G contiguous rows of N elements (in_es == 1)
			constexpr int ROW_LINES = (N + PER_LINE - 1) / PER_LINE;
			for (int k = threadIdx.x; k < G * ROW_LINES; k += CTA) {
				const int gg = k / ROW_LINES, l = k - gg * ROW_LINES;
				if (pu00 + gg < a.U0) prefetch_l2(in + pib + (pu00 + gg) * a.is0 + (long long)l * PER_LINE * a.in_es);
			}
		}
	}
	if constexpr (SLOAD) {
		// G-element segments: consecutive threads take consecutive u0 of the same element.  Every
		// HBM load of the thread is issued before its shared-memory stores (interleaved, each
		// store waited for its load: one HBM round trip per element)
		constexpr int IT = (G * N + CTA - 1) / CTA;
		C v[IT];
#pragma unroll
		for (int q = 0; q < IT; ++q) {
			const int idx = threadIdx.x + q * CTA;
			const int gg = idx % G, e = idx / G;
			if (idx < G * N && u00 + gg < a.U0) {
				const long long off = ib + (u00 + gg) * a.is0 + (long long)e * a.in_es;
				v[q] = __ldcs(in + off);
				if constexpr (CIN) v[q] = conj(v[q]);
				if constexpr (ROT == 1) v[q] = mul(v[q], __ldg(c.rot + (off - u2 * a.rot_in_stride2)));
			}
		}
#pragma unroll
		for (int q = 0; q < IT; ++q) {
			const int idx = threadIdx.x + q * CTA;
			const int gg = idx % G, e = idx / G;
			if (idx < G * N && u00 + gg < a.U0) sm_all[gg * STRIDE + pidx<PS>(e)] = v[q];
		}
		__syncthreads();
	}
	passes<T, N, THREADS, 1, 0, 0, SLOAD ? kSmem : kGlobal, SSTORE ? kSmem : kGlobal, kComplex, CIN, COUT, false, EMAX,
	       Rs...>(c, reinterpret_cast<const C *>(a.tw), reinterpret_cast<const C *>(a.roots));
	if constexpr (SSTORE) {
#pragma unroll 4
		for (int idx = threadIdx.x; idx < G * N; idx += CTA) {
			const int gg = idx % G, k = idx / G;
			const long long u0 = u00 + gg;
			if (u0 < a.U0) {
				C v = sm_all[gg * STRIDE + pidx<PS>(k)];
				if constexpr (TWN > 1) {
					const int kh = k / KL, kl = k - kh * KL;
					v = mul(v, mul(twk[gg * TWS + kh], twk[gg * TWS + KH + kl]));
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

// ------------------------------------------------------------------ two-CTA (cluster) transforms
//
// Complex FP32 transforms of N = N1 N2 points too long for two CTAs of the batch kernel to share
// an SM (from ~8192 points one transform fills 64-140 KB of shared memory and 128+ registers a
// thread; with one CTA per SM its HBM and arithmetic phases cannot overlap).  A cluster of two
// CTAs (on two SMs) runs one transform as a four-step inside the cluster, each CTA holding half:
//   n = n1 N2 + n2, k = k1 + N1 k2,
//   phase A (CTA c, columns n2 = c N2/2 + v): Y[k1][n2] = W_N^{n2 k1} sum_n1 x[n1 N2 + n2] W_N1^{n1 k1}
//   phase B (CTA c, rows k1 = c N1/2 + u):    X[k1 + N1 k2] = sum_n2 Y[k1][n2] W_N2^{n2 k2}.
// Phase A reads N1 segments of N2/2 contiguous points from HBM; its last pass writes Y transposed
// (column-major, odd row length P) into its own shared memory; after a cluster barrier, phase B's
// first pass reads each row from both CTAs' shared memory (distributed shared memory), and a
// second barrier guards the buffers before they are overwritten.  Phase B's last pass writes N2
// segments of N1/2 contiguous points.  Inside a phase the passes are the batch kernel's Stockham
// passes over V interleaved columns (element (v, e) at s[e V + v]: consecutive threads take
// consecutive columns, so shared-memory and HBM accesses are unit-stride).  With half a transform
// per CTA, two CTAs of different transforms share each SM and overlap each other's phases.
template <int... Rs>
struct Radices {};

template <int NS, int... Rs>
struct TwTotal {
	static constexpr int value = 0;
};
template <int NS, int R, int... Rs>
struct TwTotal<NS, R, Rs...> {
	static constexpr int value = TwCount<float, R, NS>::value + TwTotal<NS * R, Rs...>::value;
};
template <class L>
struct RadixList;
template <int... Rs>
struct RadixList<Radices<Rs...>> {
	static constexpr int n = (1 * ... * Rs);
	static constexpr int tw = TwTotal<1, Rs...>::value;  // pass-twiddle slots
};

// inter-phase twiddle W_N^t = hi[t >> b] lo[t & (2^b - 1)], 4^b >= N
__host__ __device__ constexpr int pair_lo_bits(int n) {
	int b = 0;
	while ((1 << (2 * b)) < n) ++b;
	return b;
}

#if defined(__CUDA_ARCH__)
__device__ __forceinline__ unsigned pair_rank() {
	unsigned r;
	asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
	return r;
}
// all threads of both CTAs; release / acquire orders the shared-memory writes and reads around it
__device__ __forceinline__ void pair_sync() {
	asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ unsigned char *pair_smem() {
	extern __shared__ __align__(16) unsigned char smem_raw[];
	return smem_raw;
}
// shared memory of cluster CTA `rank` at the offset of `p` in this CTA's, as a cluster address
struct ClusterSmem {
	unsigned base;
};
__device__ __forceinline__ ClusterSmem cluster_smem(const void *p, unsigned rank) {
	unsigned a;
	asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(smem_u32(p)), "r"(rank));
	return ClusterSmem{a};
}
__device__ __forceinline__ float2 cluster_load(ClusterSmem s, int i) {
	float2 v;
	asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(s.base + 8u * (unsigned)i));
	return v;
}
#elif defined(SSFFT_EMULATION)
// Host emulation: the two CTAs of a cluster run at once, each with its own shared-memory array.
extern thread_local unsigned char *emu_cta_smem, *emu_peer_smem;
extern thread_local std::barrier<> *emu_cluster_barrier;
inline unsigned pair_rank() { return blockIdx.x & 1u; }
inline void pair_sync() { emu_cluster_barrier->arrive_and_wait(); }
inline unsigned char *pair_smem() { return emu_cta_smem; }
struct ClusterSmem {
	const float2 *base;
};
inline ClusterSmem cluster_smem(const void *p, unsigned rank) {
	const long off = static_cast<const unsigned char *>(p) - emu_cta_smem;
	unsigned char *b = rank == pair_rank() ? emu_cta_smem : emu_peer_smem;
	return ClusterSmem{reinterpret_cast<const float2 *>(b + off)};
}
float2 emu_cluster_load(ClusterSmem s, int i);  // bounds-checked (emu_main.cpp)
inline float2 cluster_load(ClusterSmem s, int i) { return emu_cluster_load(s, i); }
#else
// host pass of the library build: declarations only
unsigned pair_rank();
void pair_sync();
unsigned char *pair_smem();
struct ClusterSmem {
	unsigned base;
};
ClusterSmem cluster_smem(const void *p, unsigned rank);
float2 cluster_load(ClusterSmem s, int i);
#endif

template <typename T>
struct PairCtx {
	using C = typename Cx<T>::C;
	C *s;              // this CTA's shared-memory slots
	const C *lo, *hi;  // inter-phase twiddle table (shared memory)
	const C *gin;      // this CTA's first input column of the transform
	C *gout;           // this CTA's first output row
	ClusterSmem cl[2]; // both CTAs' slots, as cluster addresses
	unsigned rank;
	int t;
	bool valid;
};

// One pass of phase A: radix R over the N1-point columns, V = N2/2 of them interleaved.
template <typename T, int N1, int N2, int THREADS, bool INV, int EMAX, int R, int NS, int TWO, bool FIRST, bool LAST>
__device__ __forceinline__ void pair_a_pass(const PairCtx<T> &c, const typename Cx<T>::C *tw) {
	using C = typename Cx<T>::C;
	constexpr int V = N2 / 2, P = N1 | 1, NB = N1 / R, NBF = V * NB;
	constexpr int NBPT = (NBF + THREADS - 1) / THREADS;
	constexpr bool GUARD = NBF % THREADS != 0;
	constexpr int LB = pair_lo_bits(N1 * N2);
	static_assert(Specialised<R>::value, "pair passes use register butterflies");
	static_assert(NBPT * R <= EMAX, "a pass holds at most EMAX values a thread");
	C v[NBPT][R];
#pragma unroll
	for (int i = 0; i < NBPT; ++i) {
		const int b = c.t + i * THREADS;
		if (c.valid && (!GUARD || b < NBF)) {
			const int col = b % V, j = b / V;
#pragma unroll
			for (int r = 0; r < R; ++r) {
				const int e = j + r * NB;
				if constexpr (FIRST) {
					const C x = __ldcs(c.gin + (long long)e * N2 + col);
					v[i][r] = INV ? conj(x) : x;
				} else {
					v[i][r] = c.s[e * V + col];
				}
			}
			if constexpr (NS > 1) apply_twiddles<T, R, NS, TWO>(v[i], tw, j % NS);
			dft<R>(v[i]);
		}
	}
	if constexpr (!FIRST) __syncthreads();
#pragma unroll
	for (int i = 0; i < NBPT; ++i) {
		const int b = c.t + i * THREADS;
		if (c.valid && (!GUARD || b < NBF)) {
			const int col = b % V, j = b / V;
			const int base = (j / NS) * NS * (R - 1) + j;
#pragma unroll
			for (int r = 0; r < R; ++r) {
				const int k = base + r * NS;
				if constexpr (LAST) {
					const int t = ((int)c.rank * V + col) * k;  // n2 k1 < N
					c.s[col * P + k] = mul(v[i][r], mul(c.hi[t >> LB], c.lo[t & ((1 << LB) - 1)]));
				} else {
					c.s[k * V + col] = v[i][r];
				}
			}
		}
	}
	if constexpr (LAST) pair_sync();
	else __syncthreads();
}

// One pass of phase B: radix R over the N2-point rows, V = N1/2 of them interleaved.  The first
// pass reads the rows from both CTAs (column n2 lives in CTA n2 / (N2/2)).
template <typename T, int N1, int N2, int THREADS, bool INV, int EMAX, int R, int NS, int TWO, bool FIRST, bool LAST>
__device__ __forceinline__ void pair_b_pass(const PairCtx<T> &c, const typename Cx<T>::C *tw) {
	using C = typename Cx<T>::C;
	constexpr int VA = N2 / 2, V = N1 / 2, P = N1 | 1, NB = N2 / R, NBF = V * NB;
	constexpr int NBPT = (NBF + THREADS - 1) / THREADS;
	constexpr bool GUARD = NBF % THREADS != 0;
	static_assert(Specialised<R>::value, "pair passes use register butterflies");
	static_assert(NBPT * R <= EMAX, "a pass holds at most EMAX values a thread");
	static_assert(!FIRST || R % 2 == 0, "the first phase-B radix is even (half its inputs in each CTA)");
	C v[NBPT][R];
#pragma unroll
	for (int i = 0; i < NBPT; ++i) {
		const int b = c.t + i * THREADS;
		if (c.valid && (!GUARD || b < NBF)) {
			const int row = b % V, j = b / V;
#pragma unroll
			for (int r = 0; r < R; ++r) {
				if constexpr (FIRST) {
					// n2 = j + r NB: CTA q = r / (R/2), column n2 - q VA
					constexpr int H = R / 2;
					const int q = r / H;
					v[i][r] = cluster_load(c.cl[q], (j + (r - q * H) * NB) * P + (int)c.rank * V + row);
				} else {
					v[i][r] = c.s[(j + r * NB) * V + row];
				}
			}
			if constexpr (NS > 1) apply_twiddles<T, R, NS, TWO>(v[i], tw, j % NS);
			dft<R>(v[i]);
		}
	}
	if constexpr (FIRST) pair_sync();  // both CTAs have read their rows: the buffers may be reused
	else __syncthreads();
#pragma unroll
	for (int i = 0; i < NBPT; ++i) {
		const int b = c.t + i * THREADS;
		if (c.valid && (!GUARD || b < NBF)) {
			const int row = b % V, j = b / V;
			const int base = (j / NS) * NS * (R - 1) + j;
#pragma unroll
			for (int r = 0; r < R; ++r) {
				const int k = base + r * NS;
				if constexpr (LAST) __stcs(c.gout + (long long)k * N1 + row, INV ? conj(v[i][r]) : v[i][r]);
				else c.s[k * V + row] = v[i][r];
			}
		}
	}
	if constexpr (!LAST) __syncthreads();
}

template <typename T, int N1, int N2, int THREADS, bool INV, int EMAX, bool B, int NS, int TWO, int R, int... Rest>
__device__ __forceinline__ void pair_passes(const PairCtx<T> &c, const typename Cx<T>::C *tw) {
	constexpr bool FIRST = NS == 1, LAST = sizeof...(Rest) == 0;
	if constexpr (B) pair_b_pass<T, N1, N2, THREADS, INV, EMAX, R, NS, TWO, FIRST, LAST>(c, tw);
	else pair_a_pass<T, N1, N2, THREADS, INV, EMAX, R, NS, TWO, FIRST, LAST>(c, tw);
	if constexpr (!LAST)
		pair_passes<T, N1, N2, THREADS, INV, EMAX, B, NS * R, TWO + TwCount<T, R, NS>::value, Rest...>(c, tw);
}
template <class L>
struct PairPhase;
template <int... Rs>
struct PairPhase<Radices<Rs...>> {
	template <typename T, int N1, int N2, int THREADS, bool INV, int EMAX, bool B, int TWO>
	__device__ __forceinline__ static void run(const PairCtx<T> &c, const typename Cx<T>::C *tw) {
		pair_passes<T, N1, N2, THREADS, INV, EMAX, B, 1, TWO, Rs...>(c, tw);
	}
};

// shared-memory slots of a pair CTA: the larger of the interleaved halves (N/2) and the
// transposed phase-A output (N2/2 rows of P), then the inter-phase table
__host__ __device__ constexpr int pair_slots(int n1, int n2) {
	const int data = (n2 / 2) * (n1 | 1) > (n1 * n2) / 2 ? (n2 / 2) * (n1 | 1) : (n1 * n2) / 2;
	const int lb = pair_lo_bits(n1 * n2);
	return data + (1 << lb) + (n1 * n2 + (1 << lb) - 1) / (1 << lb);
}

// Args: in / out / batch / in_dist / out_dist / offs as for the batch kernel; tw = phase A's pass
// twiddles, phase B's, then the inter-phase table (lo, hi); pf_dist in transforms.  Grid: two CTAs
// per transform.
template <typename T, int N1, int N2, int THREADS, bool INV, int EMAX, int MINB, class LA, class LB>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(THREADS, MINB) pair(const Args a) {
	using C = typename Cx<T>::C;
	static_assert(RadixList<LA>::n == N1 && RadixList<LB>::n == N2, "radix lists multiply to N1 and N2");
	static_assert(N1 % 2 == 0 && N2 % 2 == 0, "both factors even");
	constexpr int N = N1 * N2, LOB = pair_lo_bits(N), LO = 1 << LOB, HI = (N + LO - 1) / LO;
	constexpr int DATA = pair_slots(N1, N2) - LO - HI;
	PairCtx<T> c;
	c.s = reinterpret_cast<C *>(pair_smem());
	c.lo = c.s + DATA;
	c.hi = c.s + DATA + LO;
	c.rank = pair_rank();
	c.t = threadIdx.x;
	const long long g = (long long)(blockIdx.x >> 1);
	c.valid = g < a.batch;
	long long oin = 0, oout = 0;
	if (c.valid) {
		if (a.offs) oin = a.offs[g], oout = a.offs_out ? a.offs_out[g] : oin;
		else oin = g * a.in_dist, oout = g * a.out_dist;
	}
	c.gin = reinterpret_cast<const C *>(reinterpret_cast<const T *>(a.in) + oin) + c.rank * (N2 / 2);
	c.gout = reinterpret_cast<C *>(reinterpret_cast<T *>(a.out) + oout) + c.rank * (N1 / 2);
	c.cl[0] = cluster_smem(c.s, 0);
	c.cl[1] = cluster_smem(c.s, 1);
	const C *tw = reinterpret_cast<const C *>(a.tw);
	C *tab = c.s + DATA;
	for (int i = threadIdx.x; i < LO + HI; i += THREADS)
		tab[i] = __ldg(tw + RadixList<LA>::tw + RadixList<LB>::tw + i);
	// L2 prefetch of the transform pf_dist ahead: each CTA one contiguous half of it
	if (a.pf_dist > 0 && g + a.pf_dist < a.batch) {
		const long long pg = g + a.pf_dist;
		const long long po = a.offs ? a.offs[pg] : pg * a.in_dist;
		const unsigned half = (unsigned)(N / 2 * sizeof(C));
		const unsigned char *base =
		    reinterpret_cast<const unsigned char *>(reinterpret_cast<const T *>(a.in) + po) + c.rank * half;
		if (((unsigned long long)base & 15) == 0 && half % 16 == 0) {
			if (threadIdx.x == 0) prefetch_l2_bulk(base, half);
		} else {
			for (unsigned off = threadIdx.x * 128u; off < half; off += THREADS * 128u) prefetch_l2(base + off);
		}
	}
	__syncthreads();
	PairPhase<LA>::template run<T, N1, N2, THREADS, INV, EMAX, false, 0>(c, tw);
	PairPhase<LB>::template run<T, N1, N2, THREADS, INV, EMAX, true, RadixList<LA>::tw>(c, tw);
}

// Bluestein's algorithm for lengths whose prime factors the pass kernels cannot take (beyond
// one CTA): with w_k = e^{-i pi k^2 / N}, X_k = w_k sum_j (x_j w_j) conj(w_{k-j}), a circular
// convolution of length M >= 2N - 1 done by two M-point transforms: the chirp product and zero
// padding (blue_pre), the product with the precomputed spectrum of conj(w) (blue_mul) and the
// final chirp product scaled by 1/M (blue_post).  CONJ conjugates the input (pre) or the output
// (post) for the inverse.  One thread per element, blockIdx.y = transform.
struct BlueArgs {
	const void *in;     // N complex per transform, `dist` apart
	void *out;
	void *work;         // M complex per transform
	const void *chirp;  // w_k, k < N
	const void *bhat;   // M-point spectrum of b (b_m = conj(w_|m|), |m| < N, zero elsewhere)
	long long n, m, batch, dist;
	// half-shift RealFFT (ModifiedRealFFT): the packed input is multiplied by rot_k before the
	// transform (forward, rot_in), or the output by conj(rot_k) after it (inverse, rot_out)
	const void *rot_in;
	const void *rot_out;
};

template <typename T, bool CONJ>
__global__ void __launch_bounds__(256) blue_pre(const BlueArgs a) {
	using C = typename Cx<T>::C;
	const long long k = (long long)blockIdx.x * 256 + threadIdx.x, b = blockIdx.y;
	if (k >= a.m || b >= a.batch) return;
	C v = mkc(T(0), T(0));
	if (k < a.n) {
		C x = __ldcs(reinterpret_cast<const C *>(a.in) + b * a.dist + k);
		if (CONJ) x = conj(x);
		if (a.rot_in) x = mul(x, __ldg(reinterpret_cast<const C *>(a.rot_in) + k));
		v = mul(x, __ldg(reinterpret_cast<const C *>(a.chirp) + k));
	}
	reinterpret_cast<C *>(a.work)[b * a.m + k] = v;
}

template <typename T>
__global__ void __launch_bounds__(256) blue_mul(const BlueArgs a) {
	using C = typename Cx<T>::C;
	const long long k = (long long)blockIdx.x * 256 + threadIdx.x, b = blockIdx.y;
	if (k >= a.m || b >= a.batch) return;
	C *w = reinterpret_cast<C *>(a.work) + b * a.m + k;
	*w = mul(*w, __ldg(reinterpret_cast<const C *>(a.bhat) + k));
}

template <typename T, bool CONJ>
__global__ void __launch_bounds__(256) blue_post(const BlueArgs a) {
	using C = typename Cx<T>::C;
	const long long k = (long long)blockIdx.x * 256 + threadIdx.x, b = blockIdx.y;
	if (k >= a.n || b >= a.batch) return;
	C y = mul(reinterpret_cast<const C *>(a.work)[b * a.m + k], __ldg(reinterpret_cast<const C *>(a.chirp) + k));
	y = scale(y, T(1) / T(a.m));
	if (CONJ) y = conj(y);
	if (a.rot_out) y = mulc(y, __ldg(reinterpret_cast<const C *>(a.rot_out) + k));
	__stcs(reinterpret_cast<C *>(a.out) + b * a.dist + k, y);
}

// Odd real lengths beyond one CTA: the transform runs on h = floor(n/2) complex points
// z_i = {x_2i, x_2i+1} (the last real is neither read nor written, as the reference's RealFFT
// reads and writes pairs only, signalsmith-fft.h:446-502).  Rows of n reals do not keep the
// pairs aligned, so they are packed into (unpacked from) rows of h complex around the passes.
struct PackArgs {
	const void *src;
	void *dst;
	long long batch, n, h;
};

template <typename T, bool UNPACK>
__global__ void __launch_bounds__(256) real_pack(const PackArgs a) {
	using C = typename Cx<T>::C;
	const long long i = (long long)blockIdx.x * 256 + threadIdx.x, b = blockIdx.y;
	if (i >= a.h || b >= a.batch) return;
	if constexpr (!UNPACK) {
		const T *x = reinterpret_cast<const T *>(a.src) + b * a.n;
		reinterpret_cast<C *>(a.dst)[b * a.h + i] = mkc(__ldcs(x + 2 * i), __ldcs(x + 2 * i + 1));
	} else {
		const C v = __ldcs(reinterpret_cast<const C *>(a.src) + b * a.h + i);
		T *x = reinterpret_cast<T *>(a.dst) + b * a.n;
		__stcs(x + 2 * i, v.x);
		__stcs(x + 2 * i + 1, v.y);
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

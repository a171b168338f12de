/*
 * oracle/ssfft_oracle.c -- CPU oracle for the Signalsmith FFT transform path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference header
 * signalsmith-fft.h (FFT<V>, RealFFT<V>, ModifiedRealFFT<V>, the fast-size helpers), used to
 * check the GPU library's results and to time the reference's CPU algorithm.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it (as liboracle.so); the
 * shipped library (fft_gb300/) never links or calls it.
 *
 * Parity pin: tests/test_oracle.py checks it against the fixtures under tests/golden/, which
 * tests/golden/make_golden.py produced by running the unmodified reference header
 * (compiled through oracle/ref_shim.cpp) on the same seeded inputs.
 *
 * Build: oracle/Makefile (gcc -O3 -ffp-contract=off, so that the operation order below, which
 * follows the reference's, gives the same roundings on x86-64 and aarch64).
 */
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846264338327950288
#endif

/* ------------------------------------------------------------------ fast-size helpers */

/*
 * FFT::validSize (signalsmith-fft.h:317-325): below 32 the accepted "fast" remainders are 0
 * and the numbers 2^a * 3^b with b <= 2 (1 2 3 4 6 8 9 12 16 18 24).  Computed, not tabulated.
 */
static int small_fast(size_t s) {
	if (s == 0) return 1;
	if (s >= 32) return 0;
	int threes = 0;
	while (s % 3 == 0) { s /= 3; ++threes; }
	while (s % 2 == 0) s /= 2;
	return s == 1 && threes <= 2;
}

/* FFT::sizeMinimum (signalsmith-fft.h:327-337) */
size_t oracle_size_minimum(size_t size) {
	size_t p2 = 1;
	while (size >= 32) {
		size = (size - 1) / 2 + 1;
		p2 *= 2;
	}
	while (size < 32 && !small_fast(size)) ++size;
	return p2 * size;
}

/* FFT::sizeMaximum (signalsmith-fft.h:338-348) */
size_t oracle_size_maximum(size_t size) {
	size_t p2 = 1;
	while (size >= 32) {
		size /= 2;
		p2 *= 2;
	}
	while (size > 1 && !small_fast(size)) --size;
	return p2 * size;
}

/* RealFFT::sizeMinimum (signalsmith-fft.h:403-405): (FFT::sizeMinimum((n-1)/2) + 1) * 2 */
size_t oracle_real_size_minimum(size_t size) {
	return (oracle_size_minimum((size - 1) / 2) + 1) * 2;
}

/* RealFFT::sizeMaximum (signalsmith-fft.h:406-408): FFT::sizeMinimum(n/2) * 2 (sic) */
size_t oracle_real_size_maximum(size_t size) {
	return oracle_size_minimum(size / 2) * 2;
}

/* ------------------------------------------------------------------ FP64 and FP32 bodies */

#define OR_REAL double
#define OR_SFX f64
#define OR_COS cos
#define OR_SIN sin
#include "oracle_impl.h"
#undef OR_REAL
#undef OR_SFX
#undef OR_COS
#undef OR_SIN

/* FFT<float> rounds each phase to float (signalsmith-fft.h:123, :204); the unqualified cos/sin
 * calls inside the reference's namespace then resolve to the double ::cos/::sin of that float
 * value, and the results are narrowed to float (:124, :205). */
#define OR_REAL float
#define OR_SFX f32
#define OR_COS(x) ((float)cos((double)(x)))
#define OR_SIN(x) ((float)sin((double)(x)))
#include "oracle_impl.h"
#undef OR_REAL
#undef OR_SFX
#undef OR_COS
#undef OR_SIN

/* Number of radix steps and twiddles in the FP64 plan of size n (for plan-shape tests). */
int oracle_plan_shape_f64(size_t n, size_t *nsteps, size_t *ntwiddles, size_t *factors_out, size_t *nfactors) {
	plan_f64 *p = oracle_plan_new_f64(n);
	if (!p) return -1;
	*nsteps = p->nsteps;
	*ntwiddles = p->ntw;
	*nfactors = p->nfactors;
	for (size_t i = 0; i < p->nfactors; ++i) factors_out[i] = p->factors[i];
	oracle_plan_free_f64(p);
	return 0;
}

/* Radix of each step in execution order (4 for a merged 2*2). */
int oracle_plan_steps_f64(size_t n, size_t *radix_out, size_t *stride_out, size_t cap) {
	plan_f64 *p = oracle_plan_new_f64(n);
	if (!p) return -1;
	size_t k = 0;
	for (; k < p->nsteps && k < cap; ++k) {
		radix_out[k] = p->steps[k].factor;
		stride_out[k] = p->steps[k].inner;
	}
	oracle_plan_free_f64(p);
	return (int)k;
}

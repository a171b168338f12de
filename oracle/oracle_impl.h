/*
 * oracle/oracle_impl.h -- type-generic body of the CPU oracle (TEST INFRASTRUCTURE ONLY).
 *
 * Included twice by oracle/ssfft_oracle.c, once with OR_REAL=double / OR_SFX=f64 and once with
 * OR_REAL=float / OR_SFX=f32.  It restates, in plain C, the algorithm of the reference
 * header signalsmith-fft.h (Signalsmith FFT v5):
 *   - FFT<V>     : plan (factorise, radix-step tree, twiddle table, digit-reversal pairs),
 *                  permute, radix-2/3/4/generic decimation-in-time passes, unnormalised ifft;
 *   - RealFFT<V> : half-size complex FFT + even/odd split with FP64-built twiddles,
 *                  DC/Nyquist packed into bin 0, optional half-bin shift (ModifiedRealFFT).
 * The order of floating-point operations follows the reference so that, compiled without
 * FMA contraction, results are bit-identical to the reference's on the same inputs.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use this code; the
 * GPU product path never calls it.
 */

#define OR_CAT2(a, b) a##_##b
#define OR_CAT(a, b) OR_CAT2(a, b)
#define OR_FN(name) OR_CAT(name, OR_SFX)

typedef struct {
	OR_REAL re, im;
} OR_FN(cplx);
#define CPLX OR_FN(cplx)

/* perf::complexMul<false> (signalsmith-fft.h:32-41): a*b */
static inline CPLX OR_FN(cmul)(CPLX a, CPLX b) {
	CPLX r;
	r.re = a.re * b.re - a.im * b.im;
	r.im = a.re * b.im + a.im * b.re;
	return r;
}
/* perf::complexMul<true> (signalsmith-fft.h:34-36): a*conj(b), operand order as there */
static inline CPLX OR_FN(cmulc)(CPLX a, CPLX b) {
	CPLX r;
	r.re = b.re * a.re + b.im * a.im;
	r.im = b.re * a.im - b.im * a.re;
	return r;
}
/* complexMul<inverse> */
static inline CPLX OR_FN(cmul_dir)(CPLX a, CPLX b, int inverse) {
	return inverse ? OR_FN(cmulc)(a, b) : OR_FN(cmul)(a, b);
}
/* perf::complexAddI<flipped> (signalsmith-fft.h:43-52): a + i*b (flipped: a - i*b) */
static inline CPLX OR_FN(caddi)(CPLX a, CPLX b, int flipped) {
	CPLX r;
	if (flipped) {
		r.re = a.re + b.im;
		r.im = a.im - b.re;
	} else {
		r.re = a.re - b.im;
		r.im = a.im + b.re;
	}
	return r;
}
static inline CPLX OR_FN(cadd)(CPLX a, CPLX b) {
	CPLX r = {a.re + b.re, a.im + b.im};
	return r;
}
static inline CPLX OR_FN(csub)(CPLX a, CPLX b) {
	CPLX r = {a.re - b.re, a.im - b.im};
	return r;
}
static inline CPLX OR_FN(cscale)(CPLX a, OR_REAL s) {
	CPLX r = {a.re * s, a.im * s};
	return r;
}
static inline CPLX OR_FN(cconj)(CPLX a) {
	CPLX r = {a.re, -a.im};
	return r;
}

/* One radix step of the plan (FFT::Step, signalsmith-fft.h:78-85). */
typedef struct {
	int kind; /* 0 generic, 2, 3, 4 */
	size_t factor, start, inner, outer, tw;
} OR_FN(step);

typedef struct {
	size_t n;
	size_t nfactors;
	size_t factors[128];
	OR_FN(step) * steps;
	size_t nsteps, capsteps;
	CPLX *tw;
	size_t ntw, captw;
	size_t *perm_from, *perm_to;
	size_t nperm;
	CPLX *work; /* workingVector (signalsmith-fft.h:73) */
} OR_FN(plan);

static int OR_FN(push_step)(OR_FN(plan) * p, OR_FN(step) s) {
	if (p->nsteps == p->capsteps) {
		size_t cap = p->capsteps ? p->capsteps * 2 : 16;
		void *m = realloc(p->steps, cap * sizeof(OR_FN(step)));
		if (!m) return -1;
		p->steps = (OR_FN(step) *)m;
		p->capsteps = cap;
	}
	p->steps[p->nsteps++] = s;
	return 0;
}
static int OR_FN(push_tw)(OR_FN(plan) * p, CPLX t) {
	if (p->ntw == p->captw) {
		size_t cap = p->captw ? p->captw * 2 : 64;
		void *m = realloc(p->tw, cap * sizeof(CPLX));
		if (!m) return -1;
		p->tw = (CPLX *)m;
		p->captw = cap;
	}
	p->tw[p->ntw++] = t;
	return 0;
}

/*
 * Recursive step builder, restating FFT::addPlanSteps (signalsmith-fft.h:93-138):
 * two successive factors of 2 merge into one radix-4 step (:97-102); twiddles
 * e^{-2 pi i i f / length} are laid out [subLength][factor] with the phase rounded to V
 * (:121-127) and shared between steps with equal (factor, innerRepeats) (:112-119);
 * sub-blocks larger than 64 KiB recurse depth-first (:130-133); each step is appended after its
 * children (:137), so execution runs from stride 1 upwards.
 */
static int OR_FN(add_steps)(OR_FN(plan) * p, size_t fi, size_t start, size_t length, size_t repeats) {
	if (fi >= p->nfactors) return 0;
	size_t factor = p->factors[fi];
	if (fi + 1 < p->nfactors && p->factors[fi] == 2 && p->factors[fi + 1] == 2) {
		++fi;
		factor = 4;
	}
	size_t sub = length / factor;
	OR_FN(step) s;
	s.kind = (factor == 2 || factor == 3 || factor == 4) ? (int)factor : 0;
	s.factor = factor;
	s.start = start;
	s.inner = sub;
	s.outer = repeats;
	s.tw = p->ntw;

	int shared = 0;
	for (size_t k = 0; k < p->nsteps; ++k) {
		if (p->steps[k].factor == s.factor && p->steps[k].inner == s.inner) {
			shared = 1;
			s.tw = p->steps[k].tw;
			break;
		}
	}
	if (!shared) {
		for (size_t i = 0; i < sub; ++i) {
			for (size_t f = 0; f < factor; ++f) {
				OR_REAL phase = (OR_REAL)(2 * M_PI * i * f / length);
				CPLX t;
				t.re = OR_COS(phase);
				t.im = -OR_SIN(phase);
				if (OR_FN(push_tw)(p, t)) return -1;
			}
		}
	}
	if (repeats == 1 && sizeof(CPLX) * sub > 65536) {
		for (size_t i = 0; i < factor; ++i) {
			if (OR_FN(add_steps)(p, fi + 1, start + i * sub, sub, 1)) return -1;
		}
	} else {
		if (OR_FN(add_steps)(p, fi + 1, start, sub, repeats * factor)) return -1;
	}
	return OR_FN(push_step)(p, s);
}

void OR_FN(oracle_plan_free)(OR_FN(plan) * p) {
	if (!p) return;
	free(p->steps);
	free(p->tw);
	free(p->perm_from);
	free(p->perm_to);
	free(p->work);
	free(p);
}

/*
 * FFT::setPlan (signalsmith-fft.h:139-185): ascending trial-division factorisation, the step
 * tree, then the digit-reversal pairs built by growing the index set from both ends of the
 * factor list.
 */
OR_FN(plan) * OR_FN(oracle_plan_new)(size_t n) {
	if (n == 0) return NULL;
	OR_FN(plan) *p = (OR_FN(plan) *)calloc(1, sizeof(OR_FN(plan)));
	if (!p) return NULL;
	p->n = n;
	size_t rem = n, f = 2;
	while (rem > 1) {
		if (rem % f == 0) {
			p->factors[p->nfactors++] = f;
			rem /= f;
		} else if (f > sqrt((double)rem)) {
			f = rem;
		} else {
			++f;
		}
	}
	p->work = (CPLX *)calloc(n, sizeof(CPLX));
	p->perm_from = (size_t *)malloc(n * sizeof(size_t));
	p->perm_to = (size_t *)malloc(n * sizeof(size_t));
	if (!p->work || !p->perm_from || !p->perm_to || OR_FN(add_steps)(p, 0, 0, n, 1)) {
		OR_FN(oracle_plan_free)(p);
		return NULL;
	}

	p->perm_from[0] = 0;
	p->perm_to[0] = 0;
	p->nperm = 1;
	size_t lo = 0, hi = p->nfactors;
	size_t in_lo = n, out_lo = 1, in_hi = 1, out_hi = n;
	while (out_lo * in_hi < n) {
		size_t fac, in_step, out_step;
		if (out_lo <= in_hi) {
			fac = p->factors[lo++];
			in_step = (in_lo /= fac);
			out_step = out_lo;
			out_lo *= fac;
		} else {
			fac = p->factors[--hi];
			in_step = in_hi;
			in_hi *= fac;
			out_step = (out_hi /= fac);
		}
		size_t old = p->nperm;
		for (size_t i = 1; i < fac; ++i) {
			for (size_t j = 0; j < old; ++j) {
				p->perm_from[p->nperm] = p->perm_from[j] + i * in_step;
				p->perm_to[p->nperm] = p->perm_to[j] + i * out_step;
				++p->nperm;
			}
		}
	}
	return p;
}

/* FFT::fftStepGeneric (signalsmith-fft.h:187-215): O(p^2) DFT with per-term cos/sin. */
static void OR_FN(step_generic)(OR_FN(plan) * p, CPLX *base, const OR_FN(step) * s, int inverse) {
	CPLX *work = p->work;
	const size_t stride = s->inner, factor = s->factor;
	CPLX *outer = base;
	for (size_t o = 0; o < s->outer; ++o) {
		CPLX *d = outer;
		const CPLX *tw = p->tw + s->tw;
		for (size_t rep = 0; rep < s->inner; ++rep) {
			for (size_t i = 0; i < factor; ++i) work[i] = OR_FN(cmul_dir)(d[i * stride], tw[i], inverse);
			for (size_t f = 0; f < factor; ++f) {
				CPLX sum = work[0];
				for (size_t i = 1; i < factor; ++i) {
					OR_REAL phase = (OR_REAL)(2 * M_PI * f * i / factor);
					CPLX w;
					w.re = OR_COS(phase);
					w.im = -OR_SIN(phase);
					CPLX t = OR_FN(cmul_dir)(work[i], w, inverse);
					sum.re += t.re;
					sum.im += t.im;
				}
				d[f * stride] = sum;
			}
			++d;
			tw += factor;
		}
		outer += factor * s->inner;
	}
}

/* FFT::fftStep2 (signalsmith-fft.h:217-233) */
static void OR_FN(step2)(OR_FN(plan) * p, CPLX *base, const OR_FN(step) * s, int inverse) {
	const size_t stride = s->inner;
	for (size_t o = 0; o < s->outer; ++o) {
		const CPLX *tw = p->tw + s->tw;
		for (CPLX *d = base; d < base + stride; ++d) {
			CPLX a = d[0];
			CPLX b = OR_FN(cmul_dir)(d[stride], tw[1], inverse);
			d[0] = OR_FN(cadd)(a, b);
			d[stride] = OR_FN(csub)(a, b);
			tw += 2;
		}
		base += 2 * stride;
	}
}

/* FFT::fftStep3 (signalsmith-fft.h:235-259) */
static void OR_FN(step3)(OR_FN(plan) * p, CPLX *base, const OR_FN(step) * s, int inverse) {
	const OR_REAL f3re = (OR_REAL)-0.5;
	const OR_REAL f3im = inverse ? (OR_REAL)0.8660254037844386 : (OR_REAL)-0.8660254037844386;
	const size_t stride = s->inner;
	for (size_t o = 0; o < s->outer; ++o) {
		const CPLX *tw = p->tw + s->tw;
		for (CPLX *d = base; d < base + stride; ++d) {
			CPLX a = d[0];
			CPLX b = OR_FN(cmul_dir)(d[stride], tw[1], inverse);
			CPLX c = OR_FN(cmul_dir)(d[stride * 2], tw[2], inverse);
			CPLX real_sum = OR_FN(cadd)(a, OR_FN(cscale)(OR_FN(cadd)(b, c), f3re));
			CPLX imag_sum = OR_FN(cscale)(OR_FN(csub)(b, c), f3im);
			d[0] = OR_FN(cadd)(OR_FN(cadd)(a, b), c);
			d[stride] = OR_FN(caddi)(real_sum, imag_sum, 0);
			d[stride * 2] = OR_FN(caddi)(real_sum, imag_sum, 1);
			tw += 3;
		}
		base += 3 * stride;
	}
}

/* FFT::fftStep4 (signalsmith-fft.h:261-286); twiddle slots 1 and 2 are read swapped (:270-271). */
static void OR_FN(step4)(OR_FN(plan) * p, CPLX *base, const OR_FN(step) * s, int inverse) {
	const size_t stride = s->inner;
	for (size_t o = 0; o < s->outer; ++o) {
		const CPLX *tw = p->tw + s->tw;
		for (CPLX *d = base; d < base + stride; ++d) {
			CPLX a = d[0];
			CPLX c = OR_FN(cmul_dir)(d[stride], tw[2], inverse);
			CPLX b = OR_FN(cmul_dir)(d[stride * 2], tw[1], inverse);
			CPLX dd = OR_FN(cmul_dir)(d[stride * 3], tw[3], inverse);
			CPLX sum_ac = OR_FN(cadd)(a, c), sum_bd = OR_FN(cadd)(b, dd);
			CPLX diff_ac = OR_FN(csub)(a, c), diff_bd = OR_FN(csub)(b, dd);
			d[0] = OR_FN(cadd)(sum_ac, sum_bd);
			d[stride] = OR_FN(caddi)(diff_ac, diff_bd, !inverse);
			d[stride * 2] = OR_FN(csub)(sum_ac, sum_bd);
			d[stride * 3] = OR_FN(caddi)(diff_ac, diff_bd, inverse);
			tw += 4;
		}
		base += 4 * stride;
	}
}

/*
 * FFT::run (signalsmith-fft.h:295-315): gather through the digit-reversal pairs (permute
 * :288-293), then every step in plan order.  `in` and `out` must not alias (out of place only).
 */
void OR_FN(oracle_plan_exec)(OR_FN(plan) * p, int inverse, const OR_REAL *in, OR_REAL *out) {
	const CPLX *src = (const CPLX *)in;
	CPLX *dst = (CPLX *)out;
	for (size_t k = 0; k < p->nperm; ++k) dst[p->perm_from[k]] = src[p->perm_to[k]];
	for (size_t k = 0; k < p->nsteps; ++k) {
		const OR_FN(step) *s = &p->steps[k];
		CPLX *base = dst + s->start;
		switch (s->kind) {
		case 2: OR_FN(step2)(p, base, s, inverse); break;
		case 3: OR_FN(step3)(p, base, s, inverse); break;
		case 4: OR_FN(step4)(p, base, s, inverse); break;
		default: OR_FN(step_generic)(p, base, s, inverse); break;
		}
	}
}

/* ---------------------------------------------------------------- RealFFT<V, optionFlags> */

typedef struct {
	size_t n;      /* real size */
	size_t h;      /* complex size n/2 */
	int modified;  /* FFTOptions::halfFreqShift */
	CPLX *buf1, *buf2, *tw_minus_i, *rot;
	OR_FN(plan) * cplan;
} OR_FN(rplan);

void OR_FN(oracle_rplan_free)(OR_FN(rplan) * r) {
	if (!r) return;
	free(r->buf1);
	free(r->buf2);
	free(r->tw_minus_i);
	free(r->rot);
	OR_FN(oracle_plan_free)(r->cplan);
	free(r);
}

/*
 * RealFFT::setSize (signalsmith-fft.h:416-435): twiddles -i*e^{-2 pi i (k or k+1/2)/n} for
 * k <= n/4, and (modified) rotations e^{-2 pi i k/n}, all computed in double then rounded.
 */
OR_FN(rplan) * OR_FN(oracle_rplan_new)(size_t n, int modified) {
	if (n / 2 == 0) return NULL; /* the reference reads an empty buffer here */
	OR_FN(rplan) *r = (OR_FN(rplan) *)calloc(1, sizeof(OR_FN(rplan)));
	if (!r) return NULL;
	r->n = n;
	r->h = n / 2;
	r->modified = modified ? 1 : 0;
	size_t hh = n / 4 + 1;
	r->buf1 = (CPLX *)calloc(r->h, sizeof(CPLX));
	r->buf2 = (CPLX *)calloc(r->h, sizeof(CPLX));
	r->tw_minus_i = (CPLX *)calloc(hh, sizeof(CPLX));
	r->rot = (CPLX *)calloc(r->h, sizeof(CPLX));
	r->cplan = OR_FN(oracle_plan_new)(r->h);
	if (!r->buf1 || !r->buf2 || !r->tw_minus_i || !r->rot || !r->cplan) {
		OR_FN(oracle_rplan_free)(r);
		return NULL;
	}
	for (size_t i = 0; i < hh; ++i) {
		double ph = -2 * M_PI * (modified ? i + 0.5 : (double)i) / n;
		r->tw_minus_i[i].re = (OR_REAL)sin(ph);
		r->tw_minus_i[i].im = (OR_REAL)-cos(ph);
	}
	if (modified) {
		for (size_t i = 0; i < r->h; ++i) {
			double ph = -2 * M_PI * i / n;
			r->rot[i].re = (OR_REAL)cos(ph);
			r->rot[i].im = (OR_REAL)sin(ph);
		}
	}
	return r;
}

/* RealFFT::fft (signalsmith-fft.h:446-473): n reals -> n/2 complex bins (bin 0 = {DC, Nyquist}). */
void OR_FN(oracle_rplan_forward)(OR_FN(rplan) * r, const OR_REAL *in, OR_REAL *out_ri) {
	CPLX *out = (CPLX *)out_ri;
	const size_t h = r->h;
	for (size_t i = 0; i < h; ++i) {
		CPLX v = {in[2 * i], in[2 * i + 1]};
		r->buf1[i] = r->modified ? OR_FN(cmul)(v, r->rot[i]) : v;
	}
	OR_FN(oracle_plan_exec)(r->cplan, 0, (const OR_REAL *)r->buf1, (OR_REAL *)r->buf2);
	const CPLX *z = r->buf2;
	if (!r->modified) {
		out[0].re = z[0].re + z[0].im;
		out[0].im = z[0].re - z[0].im;
	}
	for (size_t i = r->modified ? 0 : 1; i <= h / 2; ++i) {
		size_t ci = r->modified ? (h - 1 - i) : (h - i);
		CPLX zc = OR_FN(cconj)(z[ci]);
		CPLX odd = OR_FN(cscale)(OR_FN(cadd)(z[i], zc), (OR_REAL)0.5);
		CPLX even_i = OR_FN(cscale)(OR_FN(csub)(z[i], zc), (OR_REAL)0.5);
		CPLX e = OR_FN(cmul)(even_i, r->tw_minus_i[i]);
		out[i] = OR_FN(cadd)(odd, e);
		out[ci] = OR_FN(cconj)(OR_FN(csub)(odd, e));
	}
}

/* RealFFT::ifft (signalsmith-fft.h:475-502): n/2 complex bins -> n reals, scaled by n. */
void OR_FN(oracle_rplan_inverse)(OR_FN(rplan) * r, const OR_REAL *in_ri, OR_REAL *out) {
	const CPLX *in = (const CPLX *)in_ri;
	const size_t h = r->h;
	if (!r->modified) {
		r->buf1[0].re = in[0].re + in[0].im;
		r->buf1[0].im = in[0].re - in[0].im;
	}
	for (size_t i = r->modified ? 0 : 1; i <= h / 2; ++i) {
		size_t ci = r->modified ? (h - 1 - i) : (h - i);
		CPLX v = in[i], v2c = OR_FN(cconj)(in[ci]);
		CPLX odd = OR_FN(cadd)(v, v2c);
		CPLX erm = OR_FN(csub)(v, v2c);
		CPLX even_i = OR_FN(cmulc)(erm, r->tw_minus_i[i]);
		r->buf1[i] = OR_FN(cadd)(odd, even_i);
		r->buf1[ci] = OR_FN(cconj)(OR_FN(csub)(odd, even_i));
	}
	OR_FN(oracle_plan_exec)(r->cplan, 1, (const OR_REAL *)r->buf1, (OR_REAL *)r->buf2);
	for (size_t i = 0; i < h; ++i) {
		CPLX v = r->buf2[i];
		if (r->modified) v = OR_FN(cmulc)(v, r->rot[i]);
		out[2 * i] = v.re;
		out[2 * i + 1] = v.im;
	}
}

/* ---------------------------------------------------------------- one-shot and batched calls */

int OR_FN(oracle_fft)(size_t n, int inverse, const OR_REAL *in, OR_REAL *out) {
	OR_FN(plan) *p = OR_FN(oracle_plan_new)(n);
	if (!p) return -1;
	OR_FN(oracle_plan_exec)(p, inverse, in, out);
	OR_FN(oracle_plan_free)(p);
	return 0;
}

int OR_FN(oracle_rfft)(size_t n, int modified, int inverse, const OR_REAL *in, OR_REAL *out) {
	OR_FN(rplan) *r = OR_FN(oracle_rplan_new)(n, modified);
	if (!r) return -1;
	if (inverse) OR_FN(oracle_rplan_inverse)(r, in, out);
	else OR_FN(oracle_rplan_forward)(r, in, out);
	OR_FN(oracle_rplan_free)(r);
	return 0;
}

typedef struct {
	int real, modified, inverse;
	size_t n, b0, b1;
	size_t in_dist, out_dist;
	const OR_REAL *in;
	OR_REAL *out;
	size_t repeats;
	int status;
} OR_FN(job);

static void *OR_FN(job_run)(void *arg) {
	OR_FN(job) *j = (OR_FN(job) *)arg;
	j->status = 0;
	if (j->real) {
		/* one RealFFT instance per thread: an instance is not thread-safe (:398) */
		OR_FN(rplan) *r = OR_FN(oracle_rplan_new)(j->n, j->modified);
		if (!r) { j->status = -1; return NULL; }
		for (size_t rep = 0; rep < j->repeats; ++rep)
			for (size_t b = j->b0; b < j->b1; ++b) {
				if (j->inverse) OR_FN(oracle_rplan_inverse)(r, j->in + b * j->in_dist, j->out + b * j->out_dist);
				else OR_FN(oracle_rplan_forward)(r, j->in + b * j->in_dist, j->out + b * j->out_dist);
			}
		OR_FN(oracle_rplan_free)(r);
	} else {
		/* one FFT instance per thread: workingVector (:73) is mutable state */
		OR_FN(plan) *p = OR_FN(oracle_plan_new)(j->n);
		if (!p) { j->status = -1; return NULL; }
		for (size_t rep = 0; rep < j->repeats; ++rep)
			for (size_t b = j->b0; b < j->b1; ++b)
				OR_FN(oracle_plan_exec)(p, j->inverse, j->in + b * j->in_dist, j->out + b * j->out_dist);
		OR_FN(oracle_plan_free)(p);
	}
	return NULL;
}

/*
 * Batched driver for the CPU baseline: `batch` independent transforms split evenly over
 * `nthreads` POSIX threads, one plan instance per thread, each batch slice run `repeats` times.
 * real=0: complex n -> n (dist 2n reals each side); real=1: forward n reals -> n/2 complex
 * (in dist n, out dist 2*(n/2)) or inverse the other way round.
 */
int OR_FN(oracle_batch)(int real, int modified, int inverse, size_t n, size_t batch, const OR_REAL *in,
                        OR_REAL *out, int nthreads, size_t repeats) {
	if (nthreads < 1) nthreads = 1;
	if ((size_t)nthreads > batch) nthreads = (int)(batch ? batch : 1);
	size_t h2 = 2 * (n / 2);
	size_t in_dist = real ? (inverse ? h2 : n) : 2 * n;
	size_t out_dist = real ? (inverse ? n : h2) : 2 * n;
	OR_FN(job) *jobs = (OR_FN(job) *)calloc((size_t)nthreads, sizeof(OR_FN(job)));
	pthread_t *th = (pthread_t *)calloc((size_t)nthreads, sizeof(pthread_t));
	if (!jobs || !th) { free(jobs); free(th); return -1; }
	int status = 0;
	for (int t = 0; t < nthreads; ++t) {
		OR_FN(job) *j = &jobs[t];
		j->real = real; j->modified = modified; j->inverse = inverse; j->n = n;
		j->b0 = batch * (size_t)t / (size_t)nthreads;
		j->b1 = batch * (size_t)(t + 1) / (size_t)nthreads;
		j->in_dist = in_dist; j->out_dist = out_dist; j->in = in; j->out = out;
		j->repeats = repeats;
		if (t > 0 && pthread_create(&th[t], NULL, OR_FN(job_run), j) != 0) {
			jobs[t].status = -2; th[t] = 0;
		}
	}
	OR_FN(job_run)(&jobs[0]);
	for (int t = 1; t < nthreads; ++t) {
		if (jobs[t].status != -2) pthread_join(th[t], NULL);
	}
	for (int t = 0; t < nthreads; ++t) if (jobs[t].status) status = jobs[t].status;
	free(jobs);
	free(th);
	return status;
}

#undef CPLX

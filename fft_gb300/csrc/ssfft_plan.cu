// ssfft_plan.cu -- host planner, FP64 twiddle tables, kernel launches and the C ABI of
// libssfft.so (include/ssfft.h).
//
// Replaces the reference's FFT<V>::setPlan / addPlanSteps (signalsmith-fft.h:93-185) and
// RealFFT<V>::setSize (:416-435) with a GB300 schedule: n is split into Stockham passes of
// radix 16/8/4/2/3/5 (other primes run a direct O(p^2) pass, as the reference's generic step
// does), every pass of one transform runs inside one CTA, and every twiddle is computed in FP64
// on the host and rounded once to the plan's dtype.  The kernel for the schedule is compiled
// for the device at plan time (ssfft_jit.cu) with all of its sizes as constants.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <functional>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "ssfft_host.h"

namespace ssfft {

// ------------------------------------------------------------------ error plumbing

static thread_local std::string g_last_error;

long long debug_knob(const char *key, long long dflt) {
	const char *env = std::getenv("SSFFT_DEBUG");
	if (!env || !*env) return dflt;
	const size_t klen = std::strlen(key);
	for (const char *p = env; *p;) {
		const char *end = std::strchr(p, ',');
		if (!end) end = p + std::strlen(p);
		const char *eq = static_cast<const char *>(std::memchr(p, '=', (size_t)(end - p)));
		if (eq && (size_t)(eq - p) == klen && std::strncmp(p, key, klen) == 0) {
			char *num_end = nullptr;
			const long long v = std::strtoll(eq + 1, &num_end, 10);
			return num_end != eq + 1 ? v : dflt;
		}
		p = *end ? end + 1 : end;
	}
	return dflt;
}

ssfft_status cuda_fail(cudaError_t e, const char *what) {
	char buf[256];
	std::snprintf(buf, sizeof buf, "%s: %s", what, cudaGetErrorString(e));
	g_last_error = buf;
	return e == cudaErrorMemoryAllocation ? SSFFT_ERR_ALLOC : SSFFT_ERR_CUDA;
}

// ------------------------------------------------------------------ fast sizes

// FFT::validSize (signalsmith-fft.h:317-325): remainders below 32 that are 0 or 2^a 3^b, b <= 2.
static bool small_fast(size_t s) {
	if (s == 0) return true;
	if (s >= 32) return false;
	int threes = 0;
	while (s % 3 == 0) {
		s /= 3;
		++threes;
	}
	while (s % 2 == 0) s /= 2;
	return s == 1 && threes <= 2;
}

// FFT::sizeMinimum (signalsmith-fft.h:327-337)
size_t size_minimum(size_t size) {
	size_t p2 = 1;
	while (size >= 32) {
		size = (size - 1) / 2 + 1;
		p2 *= 2;
	}
	while (size < 32 && !small_fast(size)) ++size;
	return p2 * size;
}

// FFT::sizeMaximum (signalsmith-fft.h:338-348)
size_t size_maximum(size_t size) {
	size_t p2 = 1;
	while (size >= 32) {
		size /= 2;
		p2 *= 2;
	}
	while (size > 1 && !small_fast(size)) --size;
	return p2 * size;
}

// 5-smooth sizes (2^a 3^b 5^c), which the reference's helpers never return (its fast remainders
// are 2^a 3^b with b <= 2, :317-325) but which run at full speed here (radix-5 butterflies in
// registers).  Walks every 3^b 5^c <= limit and rounds each to its nearest power-of-two
// multiple: O(log^2 n) candidates.
static bool smooth_scale_up(size_t odd, size_t n, size_t &out) {
	// smallest odd * 2^a >= n; false if it overflows size_t
	size_t v = odd;
	while (v < n) {
		if (v > SIZE_MAX / 2) return false;
		v *= 2;
	}
	out = v;
	return true;
}

size_t smooth_minimum(size_t n) {
	if (n <= 1) return n;
	size_t best = 0;
	for (size_t t = 1;; ) {
		for (size_t f = t;; ) {
			size_t v;
			if (smooth_scale_up(f, n, v) && (best == 0 || v < best)) best = v;
			if (f >= n || f > SIZE_MAX / 5) break;
			f *= 5;
		}
		if (t >= n || t > SIZE_MAX / 3) break;
		t *= 3;
	}
	return best;  // 0 only when no 5-smooth size >= n fits in size_t
}

size_t smooth_maximum(size_t n) {
	if (n <= 1) return n;
	size_t best = 1;
	for (size_t t = 1; t <= n; ) {
		for (size_t f = t; f <= n; ) {
			size_t v = f;
			while (v <= n / 2) v *= 2;
			if (v > best) best = v;
			if (f > n / 5) break;
			f *= 5;
		}
		if (t > n / 3) break;
		t *= 3;
	}
	return best;
}

// ------------------------------------------------------------------ FP64 roots of unity

// e^{-2 pi i k / L} in double.  The angle is reduced to the first octant by exact integer
// arithmetic before cos/sin are evaluated, so the error stays near 1 ulp for every k and L.
void unit_root(unsigned long long k, unsigned long long L, double *re, double *im) {
	k %= L;
	// theta = 2 pi k / L = q pi/2 + phi, phi = (pi/2) r / L, 0 <= r < L (exact: 4k < 2^64)
	const unsigned long long k4 = 4ull * k;
	const unsigned long long q = k4 / L;
	const unsigned long long r = k4 - q * L;
	double c, s;
	if (2 * r <= L) {
		const double phi = (M_PI / 2) * (double)r / (double)L;
		c = std::cos(phi);
		s = std::sin(phi);
	} else {
		const double phi = (M_PI / 2) * (double)(L - r) / (double)L;
		c = std::sin(phi);
		s = std::cos(phi);
	}
	double x, y;  // e^{i theta} = i^q e^{i phi}
	switch (q & 3) {
	case 0: x = c; y = s; break;
	case 1: x = -s; y = c; break;
	case 2: x = -c; y = -s; break;
	default: x = s; y = -c; break;
	}
	*re = x;
	*im = -y;
}

// ------------------------------------------------------------------ schedules

static bool specialised(int r) {
	return r == 1 || r == 2 || r == 3 || r == 4 || r == 5 || r == 6 || r == 8 || r == 9 || r == 10 || r == 12 ||
	       r == 15 || r == 16 || r == 18 || r == 20 || r == 24 || r == 25 || r == 27 || r == 32 || r == 36 ||
	       r == 40 || r == 45;
}

// Largest radix whose mirror-paired pass (2R values a thread) carries the fused RealFFT split:
// 8 (debug switch fuse_radix overrides it for experiments).
static int fuse_radix_limit() {
	const long long x = debug_knob("fuse_radix", 8);
	return x >= 2 && x <= 16 ? (int)x : 8;
}

// Fewest passes for 2^a 3^b 5^c over the register radices including the large composites
// 18, 20, 24, 25, 27, 32, 36, 40, 45 (which hold up to 45 values a thread); ties prefer
// fewer and smaller large composites.
// Order: powers of two first (largest first), then the others (largest first).
static bool fewest_passes(int a, int b, int c, int max_radix, std::vector<int> &out) {
	struct Rd { int r, x, y, z; };
	static const Rd kR[] = {{2, 1, 0, 0},  {3, 0, 1, 0},  {4, 2, 0, 0},  {5, 0, 0, 1},  {6, 1, 1, 0},
	                        {8, 3, 0, 0},  {9, 0, 2, 0},  {10, 1, 0, 1}, {12, 2, 1, 0}, {15, 0, 1, 1},
	                        {16, 4, 0, 0}, {18, 1, 2, 0}, {20, 2, 0, 1}, {24, 3, 1, 0}, {25, 0, 0, 2},
	                        {27, 0, 3, 0}, {32, 5, 0, 0}, {36, 2, 2, 0}, {40, 3, 0, 1}, {45, 0, 2, 1}};
	if (a > 40 || b > 25 || c > 20) return false;
	const int A = a + 1, B = b + 1, Cc = c + 1;
	std::vector<int> cost((size_t)A * B * Cc, 1 << 29), pick((size_t)A * B * Cc, -1);
	auto at = [&](int x, int y, int z) { return ((size_t)x * B + y) * Cc + z; };
	cost[at(0, 0, 0)] = 0;
	for (int x = 0; x <= a; ++x)
		for (int y = 0; y <= b; ++y)
			for (int z = 0; z <= c; ++z) {
				if (!x && !y && !z) continue;
				for (int i = 0; i < (int)(sizeof kR / sizeof kR[0]); ++i) {
					const Rd &d = kR[i];
					if (d.x > x || d.y > y || d.z > z || d.r > max_radix) continue;
					// a pass costs 1000; larger butterflies a little more (registers)
					const int cst = cost[at(x - d.x, y - d.y, z - d.z)] + 1000 + (d.r > 16 ? 1 : 0) + (d.r > 25 ? 2 : 0);
					if (cst < cost[at(x, y, z)]) cost[at(x, y, z)] = cst, pick[at(x, y, z)] = i;
				}
			}
	if (pick[at(a, b, c)] < 0 && (a || b || c)) return false;
	std::vector<int> p2, rest;
	for (int x = a, y = b, z = c; x || y || z;) {
		const Rd &d = kR[pick[at(x, y, z)]];
		((d.y == 0 && d.z == 0) ? p2 : rest).push_back(d.r);
		x -= d.x, y -= d.y, z -= d.z;
	}
	std::sort(p2.begin(), p2.end(), std::greater<int>());
	std::sort(rest.begin(), rest.end(), std::greater<int>());
	out = p2;
	out.insert(out.end(), rest.begin(), rest.end());
	return true;
}

// Radices for n = 2^a 3^b 5^c * rest: 3 x 5 pairs become radix-15 prime-factor butterflies;
// with `borrow`, leftover 5s and 3s also take factors of two (10, 12, 6); leftover 3s pair into
// radix 9; the remaining powers of two run in ceil(a/4) balanced passes of 16/8/4/2; other primes
// run direct passes.
static void radices_for(int a, int b, int c, const std::vector<int> &rest, bool borrow, std::vector<int> &out) {
	std::vector<int> comp;
	const int k15 = std::min(b, c);
	for (int i = 0; i < k15; ++i) comp.push_back(15);
	b -= k15;
	c -= k15;
	if (borrow) {
		for (; c > 0 && a > 0; --c, --a) comp.push_back(10);
		for (; b > 0 && a >= 2; --b, a -= 2) comp.push_back(12);
		for (; b > 0 && a >= 1; --b, --a) comp.push_back(6);
	}
	std::vector<int> p2;
	if (a > 0) {
		const int passes = (a + 3) / 4;
		for (int p = 0; p < passes; ++p) p2.push_back(1 << (a / passes + (p < a % passes ? 1 : 0)));
		std::sort(p2.begin(), p2.end(), [](int x, int y) { return x > y; });
	}
	out = p2;
	out.insert(out.end(), comp.begin(), comp.end());
	for (; c > 0; --c) out.push_back(5);
	for (; b >= 2; b -= 2) out.push_back(9);
	for (; b > 0; --b) out.push_back(3);
	out.insert(out.end(), rest.begin(), rest.end());
}

bool choose_radices(int n, std::vector<int> &radices, bool large_composites, bool real_split) {
	radices.clear();
	if (n < 1) return false;
	if (n == 1) {
		radices.push_back(1);
		return true;
	}
	int m = n, a = 0, b = 0, c = 0;
	while (m % 2 == 0) m /= 2, ++a;
	while (m % 3 == 0) m /= 3, ++b;
	while (m % 5 == 0) m /= 5, ++c;
	std::vector<int> rest;
	for (int p = 7; m > 1;) {
		if ((long long)p * p > m) {
			rest.push_back(m);
			break;
		}
		if (m % p == 0) {
			rest.push_back(p);
			m /= p;
		} else {
			p += 2;
		}
	}
	std::vector<int> plain, borrowed, fewest;
	radices_for(a, b, c, rest, false, plain);
	radices_for(a, b, c, rest, true, borrowed);
	radices = borrowed.size() < plain.size() ? borrowed : plain;
	// The large composites only where they save a pass: for transforms of 4 passes or more (up
	// to radix 25), and for the long transforms that run one or two CTAs per SM anyway (from 8192
	// points, up to radix 45).  Measured on GB300: at a few thousand points and below, the
	// register cost of radix 24+ butterflies outweighs the saved pass.
	// For a RealFFT the split costs one more shared-memory round trip unless the list has a
	// radix <= 8 to fuse it into (see the fused split passes), so count that too.
	auto cost = [&](const std::vector<int> &l) {
		bool fusable = false;
		for (int r : l) fusable = fusable || (r >= 2 && r <= fuse_radix_limit());
		return (int)l.size() + (real_split && !fusable ? 1 : 0);
	};
	if (large_composites && rest.empty()) {
		const int max_radix = n >= 8192 ? 45 : radices.size() >= 4 ? 25 : 0;
		// (below 8192 points a RealFFT tie between a four-pass fusable list and three passes plus
		// the split goes to the three passes: RealFFT 15360 16-24-20 46% of the copy bandwidth,
		// 8-8-15-8 fused 42%; at 16384 points the fused four passes measured 2-4% faster)
		const bool tie_to_fewest = real_split && radices.size() >= 4 && n < 8192;
		if (max_radix && fewest_passes(a, b, c, max_radix, fewest) &&
		    (cost(fewest) < cost(radices) || (tie_to_fewest && cost(fewest) == cost(radices) &&
		                                      fewest.size() < radices.size())))
			radices = fewest;
		// a RealFFT list whose fewest passes have no radix <= 8: the same number of passes with
		// one fusable radix (8192 = 32 32 8 instead of 32 16 16) saves the split's round trip
		if (max_radix && real_split) {
			struct Fz { int r, x, y, z; };
			for (const Fz f : {Fz{8, 3, 0, 0}, Fz{4, 2, 0, 0}, Fz{6, 1, 1, 0}, Fz{5, 0, 0, 1}, Fz{3, 0, 1, 0},
			                   Fz{2, 1, 0, 0}}) {
				std::vector<int> sub;
				if (f.r > fuse_radix_limit() || f.x > a || f.y > b || f.z > c) continue;
				if (!fewest_passes(a - f.x, b - f.y, c - f.z, max_radix, sub)) continue;
				sub.push_back(f.r);
				if (cost(sub) < cost(radices)) radices = sub;
			}
		}
		// three passes from 8192 points (radices <= 32): the smallest radix in the middle
		// (measured on GB300, complex 16384 32-16-32 58.7% of the copy bandwidth against 55.4%
		// for 32-32-16, 10000 25-16-25 2-3% faster than 16-25-25; 15360 40-16-24 was slower than
		// 16-40-24)
		if (n >= 8192 && !real_split && radices.size() == 3 && *std::max_element(radices.begin(), radices.end()) <= 32) {
			std::sort(radices.begin(), radices.end());
			radices = {radices[2], radices[0], radices[1]};
		}
	}
	return radices.size() <= 24;
}

size_t device_smem_limit(int dev) {
	int v = 0;
	if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0)
		v = 227 * 1024;
	return (size_t)v;
}

// Threads per transform, transforms per CTA and shared memory for n points.
// Distinct radix lists worth timing for n complex points: the planner's choice and its pass
// orders, and the list without borrowed composite radices and its orders (at most 8 in all).
void radix_candidates(int n, std::vector<std::vector<int>> &out, bool real_split) {
	out.clear();
	std::vector<int> def;
	if (!choose_radices(n, def, true, real_split)) return;
	auto add_orders = [&](std::vector<int> r) {
		std::vector<int> sorted = r;
		std::sort(sorted.begin(), sorted.end());
		std::vector<std::vector<int>> perms;
		do perms.push_back(sorted);
		while (std::next_permutation(sorted.begin(), sorted.end()) && perms.size() < 24);
		// the given order first, then the others
		if (std::find(out.begin(), out.end(), r) == out.end() && out.size() < 8) out.push_back(r);
		for (auto &q : perms)
			if (std::find(out.begin(), out.end(), q) == out.end() && out.size() < 8) out.push_back(q);
	};
	add_orders(def);
	// the alternative grouping (with or without composite 10/12/6 radices)
	int m = n, a = 0, b = 0, c = 0;
	while (m % 2 == 0) m /= 2, ++a;
	while (m % 3 == 0) m /= 3, ++b;
	while (m % 5 == 0) m /= 5, ++c;
	if (m == 1) {
		std::vector<int> plain, borrowed;
		radices_for(a, b, c, {}, false, plain);
		radices_for(a, b, c, {}, true, borrowed);
		if (plain != def && plain.size() <= def.size() + 1) add_orders(plain);
		if (borrowed != def && borrowed.size() <= def.size() + 1) add_orders(borrowed);
	}
	// a RealFFT whose list has no radix <= 8 cannot fuse its split: also try one radix split in
	// two so that it can (one more pass, one shared-memory round trip less)
	bool fusable = false;
	for (int r : def) fusable = fusable || (r >= 2 && r <= fuse_radix_limit());
	if (real_split && !fusable) {
		static const int kSplit[][3] = {{16, 4, 4}, {16, 8, 2}, {15, 3, 5}, {12, 4, 3}, {10, 2, 5}, {9, 3, 3}};
		for (const auto &sp : kSplit) {
			auto it = std::find(def.begin(), def.end(), sp[0]);
			if (it == def.end()) continue;
			std::vector<int> l(def.begin(), it);
			l.push_back(sp[1]);
			l.push_back(sp[2]);
			l.insert(l.end(), it + 1, def.end());
			if (std::find(out.begin(), out.end(), l) == out.end() && out.size() < 12) out.push_back(l);
		}
	}
}

std::string Knobs::str() const {
	std::string r = "radices=";
	for (size_t i = 0; i < radices.size(); ++i) r += (i ? "." : "") + std::to_string(radices[i]);
	if (radices.empty()) r += "default";
	r += " cta=" + std::to_string(cta_threads) + " emax=" + std::to_string(emax) + " minb=" + std::to_string(minb);
	if (prefetch >= 0) r += " prefetch=" + std::to_string(prefetch) + "/4";
	if (precision == 1) r += " precision=split_bf16";
	if (pair >= 0) r += " pair=" + std::to_string(pair);
	if (staging) r += " staging=" + std::to_string(staging);
	return r;
}

bool make_schedule(ssfft_dtype dtype, int n, int kind, bool odd, size_t batch, Schedule &s, int allow_staged,
                   const Knobs *knobs, int fuse) {
	s = Schedule();
	s.dtype = dtype;
	s.n = n;
	s.kind = kind;
	s.odd = odd;
	if (knobs && !knobs->radices.empty()) {
		long long prod = 1;
		for (int r : knobs->radices) {
			if (r < 2 && n > 1) return false;
			prod *= r;
			if (prod > n) return false;
		}
		if (prod != n || knobs->radices.size() > 24) return false;
		s.radices = knobs->radices;
	} else if (!choose_radices(n, s.radices, !(knobs && knobs->precision == 1), kind == 1 && !odd)) {
		// (the tensor-core pass needs a first radix <= 16: no large composites there)
		return false;
	}
	// split-BF16 tensor-core first pass: complex FP32, first radix <= 16 (moved to the front)
	const bool want_tc = knobs && knobs->precision == 1 && kind == 0 && dtype == SSFFT_F32 && n >= 2;
	if (want_tc && s.radices[0] > 16) {
		auto it = std::find_if(s.radices.begin(), s.radices.end(), [](int r) { return r >= 2 && r <= 16; });
		if (it != s.radices.end()) std::rotate(s.radices.begin(), it, it + 1);
	}
	s.tc = want_tc && s.radices[0] >= 2 && s.radices[0] <= 16;
	// threads per transform: every pass must fit its butterflies into `emax` values per thread;
	// 16 normally, 32 when 16 would need more than one CTA's threads (long sizes whose composite
	// radices hold a single butterfly per thread)
	s.fuse = fuse;
	auto threads_for = [&](int emax) {
		int t = 1;
		for (size_t p = 0; p < s.radices.size(); ++p) {
			const int r = s.radices[p];
			const bool mirror = (fuse == 1 && p + 1 == s.radices.size()) || (fuse == 2 && p == 0);
			int need;
			if (mirror) {
				// mirror-paired pass: units of two butterflies (2r values), (n/r + 1)/2 of them
				const int units = (n / r + 1) / 2, per = std::max(1, emax / (2 * r));
				need = (units + per - 1) / per;
			} else {
				const int per = r == 1 ? 1 : std::max(1, emax / r);  // butterflies a thread holds
				need = specialised(r) ? (n / r + per - 1) / per : (n + emax - 1) / emax;
			}
			t = std::max(t, need);
		}
		return t;
	};
	int t;
	if (knobs && knobs->emax > 0) {
		if (knobs->emax > 2 * kElemsPerThread) return false;
		s.emax = knobs->emax;
		t = threads_for(s.emax);
	} else {
		// 16 values a thread, or 32 when a butterfly holds more than 16 (the smaller radices then
		// take two butterflies a thread, so the thread count follows the large one) or when 16
		// would need more than one CTA's threads
		const int rmax = *std::max_element(s.radices.begin(), s.radices.end());
		s.emax = rmax > kElemsPerThread ? 2 * kElemsPerThread : kElemsPerThread;
		t = threads_for(s.emax);
		if (t > kMaxCtaThreads && s.emax == kElemsPerThread) {
			s.emax = 2 * kElemsPerThread;
			t = threads_for(s.emax);
		}
	}
	if (t > kMaxCtaThreads) return false;
	s.threads = t;
	// Mid-length FP32 transforms (4097-8191 complex points, three passes, largest radix 17-25,
	// planner's own shape): 16 values a thread with the largest radix in the middle pass, and
	// as many CTAs per SM (<= 3) as leave each thread the registers its values need (about 2 per
	// complex value plus 12).  Measured on GB300 (complex, 512 MB per launch, fraction of the copy
	// bandwidth, against the 32-values-a-thread default): 5120 0.63 -> 0.81, 6144 0.67 -> 0.73,
	// 6400 0.64 -> 0.68, 7680 0.51 -> 0.66, 8000 0.47 -> 0.59, 5000 0.59 -> 0.64, 4608 0.64 ->
	// 0.71, 6000 0.58 -> 0.62; RealFFT 10240 / 12288 / 15360 0.53 / 0.55 / 0.43 -> 0.65 / 0.60 /
	// 0.54.  Beyond 512 threads (7200) the default stays.  debug switch mid_rule=0 turns it off.
	int mid_minb = 0;
	{
		const bool own_shape = !knobs || (knobs->radices.empty() && !knobs->emax && !knobs->cta_threads &&
		                                  !knobs->minb && knobs->precision == 0);
		const int rmax = *std::max_element(s.radices.begin(), s.radices.end());
		if (own_shape && dtype == SSFFT_F32 && n > 4096 && n < 8192 && s.radices.size() == 3 && rmax > 16 &&
		    rmax <= 25 && !s.tc && debug_knob("mid_rule", 1) != 0) {
			Schedule m = s;
			std::vector<int> rest = m.radices;
			rest.erase(std::find(rest.begin(), rest.end(), rmax));
			m.radices = {rest[0], rmax, rest[1]};
			const std::vector<int> saved = s.radices;
			s.radices = m.radices;
			const int t16 = threads_for(kElemsPerThread);
			s.radices = saved;
			int v = 0;  // most complex values a thread holds in a pass
			for (int r : m.radices) {
				const int nb = n / r;
				v = std::max(v, r * ((nb + t16 - 1) / t16));
			}
			const int w = (t16 + 31) / 32;
			const size_t smem1 = (size_t)((n - 1) + ((n - 1) >> 4) + 2) * 8;  // one FP32 transform's slots
			int k = 0;
			for (int c = 1; c <= 3; ++c) {
				// registers a thread gets at c CTAs per SM (the warps share four schedulers'
				// 16K-register files), rounded down to the allocation unit of 8
				const int per_smsp = (c * w + 3) / 4;
				const int cap = (16384 / (32 * per_smsp)) & ~7;
				if (cap >= 2 * v + 12 && (size_t)c * smem1 <= 227 * 1024) k = c;
			}
			const int w0 = (s.threads + 31) / 32;
			const int k0 = s.emax == 2 * kElemsPerThread && s.threads <= 256 ? 2 : 1;  // the default's CTAs per SM
			if (t16 <= 512 && k > 0 && k * w > k0 * w0) {
				s.radices = m.radices;
				s.emax = kElemsPerThread;
				s.threads = t = t16;
				mid_minb = k;
			}
		}
	}
	const size_t eb = dtype == SSFFT_F32 ? 8 : 16;
	const int shift = dtype == SSFFT_F32 ? 4 : 3;
	s.smem_stride = (n - 1) + ((n - 1) >> shift) + 1;
	if (s.smem_stride % 2 == 0) s.smem_stride += 1;  // neighbouring transforms start on other banks
	const size_t per = (size_t)s.smem_stride * eb;
	if (per > 227 * 1024) return false;
	// about 128 threads per CTA (debug switch cta_threads overrides), at most 48 KiB of shared
	// memory unless one transform needs more
	const long long cta_dbg = debug_knob("cta_threads", 0);
	const int cta_target = cta_dbg > 0 && cta_dbg <= kMaxCtaThreads ? (int)cta_dbg : 128;  // 128 measured best on GB300
	int g = std::max(1, (knobs && knobs->cta_threads > 0 ? knobs->cta_threads : cta_target) / t);
	const size_t soft = std::max<size_t>(per, 48 * 1024);
	while (g > 1 && (size_t)g * per > soft) --g;
	if (batch > 0 && (size_t)g > batch) g = (int)batch;
	s.per_cta = std::max(1, g);
	if (s.tc) {
		// the tensor-core pass needs 128 threads (one accumulator lane per row)
		while (s.per_cta * t < 128) ++s.per_cta;
		if (s.per_cta * t > kMaxCtaThreads) s.tc = false, s.per_cta = std::max(1, g);
	}
	s.smem_bytes = (size_t)s.per_cta * per;
	// a single-pass complex transform never touches shared memory
	if (kind == 0 && s.radices.size() == 1) s.smem_bytes = 0;
	if (s.tc) {
		const int rows = s.per_cta * (n / s.radices[0]);
		s.smem_bytes = ssfft_cl::tc_smem_bytes(s.per_cta, s.smem_stride, (rows + 127) / 128);
	}
	// Staged input (bulk copies into shared memory, persistent CTAs) when one transform's input is
	// a whole number of 16-byte units and a group of them fits the copy and shared-memory limits.
	const size_t sb = eb / 2;
	const size_t in_bytes = kind == 0 ? (size_t)n * eb : (size_t)2 * n * sb;  // real: n_real = 2h reals or h bins
	// Opt-in for every size (debug switch staged=1, read when a plan is made): measured slower than
	// the unstaged kernel on GB300 below 8192 points.  Long FP32 transforms (8192 complex points
	// and up, or RealFFT halves of that length) whose plain kernel runs one CTA per SM stage by
	// default (debug switch long_staged=0 turns it off): one transform per CTA at 224-384 threads,
	// where the persistent loop does not spill (checked when the kernels are built), with the
	// whole input staged when it fits beside the work buffer and (complex) the first pass's
	// leading rows otherwise.  Measured on GB300 (512 MB per launch, fraction of the copy
	// bandwidth): complex 8640 0.49 -> 0.65, 9216 0.53 -> 0.67, 10240 0.49 -> 0.67, 11520 0.48 ->
	// 0.53, 13824 0.57 -> 0.65, 16384 0.57 -> 0.59 (leading rows); RealFFT 24576 0.48 / 0.42 ->
	// 0.54 / 0.50 (forward / inverse; the split and pre-twiddle as separate steps); at 200
	// threads (10000) 0.46 -> 0.39, and where the plain kernel runs two CTAs per SM (complex 8192
	// 0.68 -> 0.66, RealFFT 16384 0.61 -> 0.59).
	auto staged_smem = [&](int gg) { return (((size_t)gg * in_bytes + 127) & ~(size_t)127) + (size_t)gg * per; };
	const int staging = knobs ? knobs->staging : 0;
	const bool staged_enabled = staging == 1 || (staging == 0 && debug_knob("staged", 0) == 1);
	const bool plain_two_per_sm = dtype == SSFFT_F32 && s.emax == 2 * kElemsPerThread &&
	                              s.per_cta * s.threads <= 256 && 2 * s.smem_bytes <= 227 * 1024;
	const bool long_ok = dtype == SSFFT_F32 && kind != ssfft_cl::kRealHalfShift && n >= kLongStagedMin && s.per_cta == 1 &&
	                     !plain_two_per_sm && !(knobs && (knobs->cta_threads || knobs->emax || knobs->minb)) &&
	                     staging == 0 && debug_knob("long_staged", 1) == 1;
	const Schedule plain = s;
	if (((allow_staged == 1 && staging >= 0 && (staged_enabled || long_ok)) || allow_staged == 2) && !s.tc && !odd &&
	    in_bytes % 16 == 0 && n >= 16) {
		// long lengths whose default list spills in the staged kernel but another list does not
		// (found by compiling the candidate lists of three radices <= 32 and of four radices <= 16
		// for sm_103a with the compiler's register report: 8748 27-18-18 268 B, 9600 25-16-24
		// 376 B, 12288 32-16-24 196 B of spills a thread against none, 10800 16-45-15 556 B
		// against 24 B for these; and measured faster than the plain kernel: 12288 0.54 -> 0.69,
		// 9600 0.45 -> 0.59, 10800 0.42 -> 0.50 of the copy bandwidth)
		if (long_ok && kind == 0 && !(knobs && !knobs->radices.empty())) {
			static const struct {
				int n, count, r[4], emax;  // radices, values a thread (the thread count follows)
			} kLongStagedLists[] = {{8748, 3, {27, 12, 27}, 32},
			                        {9600, 3, {24, 20, 20}, 48},
			                        {10800, 4, {16, 15, 3, 15}, 48},
			                        {12288, 3, {32, 12, 32}, 48}};
			for (const auto &e : kLongStagedLists)
				if (e.n == n) {
					s.radices.assign(e.r, e.r + e.count);
					s.emax = e.emax;
					s.threads = threads_for(s.emax);
				}
		}
		int gs = s.per_cta;
		while (gs > 1 && staged_smem(gs) > 76 * 1024) --gs;
		if ((size_t)gs * in_bytes < (1u << 20) && staged_smem(gs) <= kStagedSmemMax) {
			s.staged = true;
			s.per_cta = gs;
			s.in_bytes = (unsigned)in_bytes;
			s.smem_bytes = staged_smem(gs);
		} else if (gs == 1 && kind == 0 && dtype == SSFFT_F32) {
			// split staging: rows r < K of the first pass (K NB elements) staged, the rest copied
			// into the work buffer once the previous group's last pass has read it
			const int r0 = s.radices[0];
			const size_t row = (size_t)(n / r0) * eb;
			int k = per + 128 < kStagedSmemMax ? (int)((kStagedSmemMax - per - 128) / row) : 0;
			k = std::min(k, r0 - 1);
			if (row % 16) k &= ~1;  // staged and remaining bytes on 16-byte boundaries
			if (2 * k >= r0) {
				s.staged = true;
				s.stage_rows = k;
				s.in_bytes = (unsigned)in_bytes;
				s.smem_bytes = (((size_t)k * row + 127) & ~(size_t)127) + per;
			}
		}
		if (s.staged && s.per_cta == 1 && n >= kLongStagedMin && s.threads > kLongStagedThreads) {
			// fewer threads holding more values each: the persistent loop spills at 512 threads
			for (int em : {48, 64}) {
				const int t2 = threads_for(em);
				if (t2 <= kLongStagedThreads) {
					s.emax = em;
					s.threads = t2;
					break;
				}
			}
		}
		// a long staging the planner chose by itself keeps 224-384 threads per transform
		if (s.staged && long_ok && !staged_enabled && allow_staged != 2 &&
		    (s.threads < kLongStagedMinThreads || s.threads > kLongStagedThreads))
			s = plain;
	}
	const int minb_env = (int)debug_knob("minb", 0);
	// Measured on GB300: forcing more resident CTAs (register caps with small spills) did not
	// beat the compiler's own allocation for the plain kernel of small transforms; the staged
	// kernel's loop needs a cap of two CTAs where two fit in shared memory (a long transform whose
	// stage and work buffers leave room for one CTA keeps the compiler's allocation: a cap of two
	// there spills).  A FP32 transform holding 32 values a thread in a CTA
	// of at most 256 threads (8192 points and up) compiles to 128-170 registers, one CTA per SM:
	// capped at two CTAs (128 registers, no spills) it overlaps one CTA's HBM phase with the
	// other's arithmetic (complex 8192: 51% -> 74% of the copy bandwidth).  debug switch minb overrides
	// for experiments.
	int mb = s.staged && 2 * s.smem_bytes <= 227 * 1024 ? 2 : 1;
	if (!s.staged && dtype == SSFFT_F32 && s.emax == 2 * kElemsPerThread && s.per_cta * s.threads <= 256 &&
	    2 * s.smem_bytes <= 227 * 1024)
		mb = 2;
	// One transform of 16 values a thread per 256-thread CTA (2304-4096 complex points, RealFFT
	// 4608-8192): the compiler's 72 registers leave 3 CTAs per SM; capped at 5 (51 registers, a
	// few bytes of spills) more CTAs overlap their HBM phases (complex 4096 83% -> 88% of the copy
	// bandwidth, RealFFT 8192 67% -> 72%; caps of 7 or more spill heavily).
	if (!s.staged && !s.tc && dtype == SSFFT_F32 && s.emax == kElemsPerThread && s.per_cta == 1 &&
	    s.threads == 256 && 5 * s.smem_bytes <= 227 * 1024)
		mb = 5;
	if (mid_minb > 0 && !s.staged) mb = mid_minb;
	if (minb_env > 0) mb = minb_env;
	if (knobs && knobs->minb > 0) mb = knobs->minb;
	s.minb = std::max(1, mb);
	return true;
}

std::string Schedule::name(bool inverse) const {
	if (pair) {
		auto list = [&](size_t b, size_t e) {
			std::string l = "ssfft_cl::Radices<";
			for (size_t i = b; i < e; ++i) l += (i > b ? ", " : "") + std::to_string(radices[i]);
			return l + ">";
		};
		return "ssfft_cl::pair<float, " + std::to_string(n1) + ", " + std::to_string(n / n1) + ", " +
		       std::to_string(threads) + ", " + (inverse ? "true" : "false") + ", " + std::to_string(emax) + ", " +
		       std::to_string(minb) + ", " + list(0, (size_t)pair) + ", " + list((size_t)pair, radices.size()) + ">";
	}
	if (tc) {
		std::string r = "ssfft_cl::batch_tc<" + std::to_string(n) + ", " + std::to_string(threads) + ", " +
		                std::to_string(per_cta) + ", " + std::to_string(smem_stride) + ", " +
		                (inverse ? "true" : "false") + ", " + std::to_string(emax) + ", " + std::to_string(minb);
		for (int x : radices) r += ", " + std::to_string(x);
		return r + ">";
	}
	std::string r = staged ? "ssfft_cl::batch_staged<" : "ssfft_cl::batch<";
	r += dtype == SSFFT_F32 ? "float" : "double";
	r += ", " + std::to_string(n) + ", " + std::to_string(threads) + ", " + std::to_string(per_cta) + ", " +
	     std::to_string(smem_stride) + ", " + std::to_string(kind) + ", " + (inverse ? "true" : "false") + ", ";
	if (!staged) r += std::string(odd ? "true" : "false") + ", ";
	r += std::to_string(emax) + ", " + std::to_string(minb);
	if (!staged) r += std::string(", ") + (fuse ? "true" : "false");
	else r += ", " + std::to_string(stage_rows);
	for (int x : radices) r += ", " + std::to_string(x);
	r += ">";
	return r;
}

// Per-pass twiddles [pass][r-1][m] = W_{ns R}^{m r} (passes after the first) and the roots
// W_R^k of direct passes, in the order the kernel's compile-time offsets expect.
void schedule_twiddles(const Schedule &s, std::vector<double> &tw, std::vector<double> &roots) {
	if (s.pair) {
		// phase A's pass twiddles (an n1-point list), phase B's (n2 points), then the inter-phase
		// table W_n^t = hi[t >> b] lo[t & (2^b - 1)]: lo[k] = W_n^k (k < 2^b), hi[k] = W_n^{k 2^b}
		Schedule a = s, b = s;
		a.pair = b.pair = 0;
		a.radices.assign(s.radices.begin(), s.radices.begin() + s.pair);
		b.radices.assign(s.radices.begin() + s.pair, s.radices.end());
		schedule_twiddles(a, tw, roots);
		schedule_twiddles(b, tw, roots);
		const int lb = ssfft_cl::pair_lo_bits(s.n);
		const unsigned long long lo = 1ull << lb, hi = ((unsigned long long)s.n + lo - 1) / lo;
		for (unsigned long long k = 0; k < lo + hi; ++k) {
			double re, im;
			unit_root(k < lo ? k : (k - lo) * lo, (unsigned long long)s.n, &re, &im);
			tw.push_back(re);
			tw.push_back(im);
		}
		return;
	}
	long long ns = 1;
	for (int R : s.radices) {
		// FP32 register butterflies store the rows of exponents 1, 2, 4, 8, 16 (< R) and form the
		// other powers by products; FP64 passes and direct passes store every exponent 1..R-1
		std::vector<int> exps;
		if (specialised(R) && s.dtype == SSFFT_F32)
			for (int e = 1; e < R; e *= 2) exps.push_back(e);
		else
			for (int r = 1; r < R; ++r) exps.push_back(r);
		if (ns > 1)
			for (int r : exps)
				for (long long m = 0; m < ns; ++m) {
					double re, im;
					unit_root((unsigned long long)(m * r), (unsigned long long)(ns * R), &re, &im);
					tw.push_back(re);
					tw.push_back(im);
				}
		if (!specialised(R))
			for (int k = 0; k < R; ++k) {
				double re, im;
				unit_root((unsigned long long)k, (unsigned long long)R, &re, &im);
				roots.push_back(re);
				roots.push_back(im);
			}
		ns *= R;
	}
}

// ------------------------------------------------------------------ plan object

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

template <typename T>
static void put_table(std::vector<unsigned char> &blob, size_t off, const std::vector<double> &src) {
	T *dst = reinterpret_cast<T *>(blob.data() + off);
	for (size_t i = 0; i < src.size(); ++i) dst[i] = (T)src[i];
}

static int kind_code(ssfft_kind kind) {
	return kind == SSFFT_COMPLEX ? ssfft_cl::kComplex : kind == SSFFT_REAL ? ssfft_cl::kReal : ssfft_cl::kRealHalfShift;
}

// Fewest register-radix passes (radix <= max_radix) for m = 2^a 3^b 5^c.
static bool fewest_list(int m, int max_radix, std::vector<int> &out) {
	int a = 0, b = 0, c = 0;
	while (m % 2 == 0) m /= 2, ++a;
	while (m % 3 == 0) m /= 3, ++b;
	while (m % 5 == 0) m /= 5, ++c;
	return m == 1 && fewest_passes(a, b, c, max_radix, out);
}

// Threads of a pair CTA for phase lists (la, lb) of an n-point transform when a pass holds at
// most emax values a thread (0 if a radix does not fit).
static int pair_threads(int n, const std::vector<int> &la, const std::vector<int> &lb, int emax) {
	long long t = 32;
	for (const auto *l : {&la, &lb})
		for (int r : *l) {
			const int per = emax / r;
			if (per < 1) return 0;
			t = std::max<long long>(t, ((long long)n / 2 / r + per - 1) / per);
		}
	return (int)((t + 31) / 32 * 32);
}

// Values a thread holds (32, or 16 where 32 would need more than 384 threads) and threads of a
// pair CTA; false if the lists do not fit one CTA.
static bool pair_shape(int n, const std::vector<int> &la, const std::vector<int> &lb, const Knobs *knobs, int &emax,
                       int &t) {
	emax = knobs && knobs->emax > 0 ? knobs->emax : 2 * kElemsPerThread;
	t = pair_threads(n, la, lb, emax);
	if (!(knobs && knobs->emax > 0) && (!t || t > 384)) {
		emax = kElemsPerThread;
		t = pair_threads(n, la, lb, emax);
	}
	return t > 0 && t <= kMaxCtaThreads;
}

// The two-CTA cluster schedule of an n-point complex FP32 transform: n = n1 n2, both even, phase
// A's radices (n1) then phase B's (n2, an even radix first).  Default split: fewest passes, then
// few threads (at most 256, else 320), then the longer HBM segments (n1/2 and n2/2 points).  Two
// CTAs per SM (the register cap of two CTAs: 128 registers at 256 threads).
bool pair_schedule(int n, Schedule &s, const Knobs *knobs) {
	std::vector<int> la, lb;
	if (knobs && knobs->pair > 0) {
		if ((int)knobs->radices.size() <= knobs->pair) return false;
		la.assign(knobs->radices.begin(), knobs->radices.begin() + knobs->pair);
		lb.assign(knobs->radices.begin() + knobs->pair, knobs->radices.end());
	} else {
		long long best = 1ll << 40;
		static const int kMax[] = {32, 27, 25, 16};
		for (int n1 = 2; n1 <= n / 2; n1 += 2) {
			if (n % n1 || (n / n1) % 2) continue;
			const int n2 = n / n1;
			for (int ma : kMax)
				for (int mb : kMax) {
					std::vector<int> a, b;
					if (!fewest_list(n1, ma, a) || !fewest_list(n2, mb, b)) continue;
					auto it = std::find_if(b.begin(), b.end(), [](int r) { return r % 2 == 0; });
					if (it == b.end()) continue;
					std::rotate(b.begin(), it, it + 1);
					int em, t;
					if (!pair_shape(n, a, b, knobs, em, t)) continue;
					const long long cost = 100000ll * (long long)(a.size() + b.size()) + (t > 256 ? 20000 : 0) +
					                       (t > 320 ? 20000 : 0) + (em < 2 * kElemsPerThread ? 30000 : 0) -
					                       2 * std::min(n1, n2) + (n1 > n2);
					if (cost < best) best = cost, la = a, lb = b;
				}
		}
		if (la.empty()) return false;
	}
	long long n1 = 1, n2 = 1;
	for (int r : la) n1 *= r;
	for (int r : lb) n2 *= r;
	if (n1 * n2 != n || n1 % 2 || n2 % 2 || lb[0] % 2) return false;
	for (int r : la)
		if (!specialised(r) || r < 2 || r > 32) return false;
	for (int r : lb)
		if (!specialised(r) || r < 2 || r > 32) return false;
	int emax, t;
	if (!pair_shape(n, la, lb, knobs, emax, t)) return false;
	s = Schedule();
	s.dtype = SSFFT_F32;
	s.n = n;
	s.kind = ssfft_cl::kComplex;
	s.radices = la;
	s.radices.insert(s.radices.end(), lb.begin(), lb.end());
	s.pair = (int)la.size();
	s.n1 = (int)n1;
	s.threads = t;
	s.per_cta = 1;
	s.emax = emax;
	s.minb = knobs && knobs->minb > 0 ? knobs->minb : (t <= 512 ? 2 : 1);
	s.smem_bytes = (size_t)ssfft_cl::pair_slots((int)n1, (int)n2) * 8;
	return s.smem_bytes <= 227 * 1024;
}

// Whether the planner's default for a complex FP32 transform of n points is the two-CTA cluster
// schedule: off (measured on GB300 slower than the one-CTA schedules at 8192-16384 points:
// complex 16384 46-53% of the copy bandwidth against 55%, the cluster barriers and
// distributed-shared-memory reads cost more than the second CTA per SM gains).  debug switch pair_min
// sets the smallest such n for plans made while it is set.
static bool pair_default(int n) {
	const long long lo = debug_knob("pair_min", 0);
	return lo > 0 && n >= lo;
}

// The single-CTA schedule of (n, dtype, kind, batch), or false if n needs the multi-pass path.
bool single_schedule(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, Schedule &s, const Knobs *knobs,
                     int allow_staged, int dir) {
	const bool real = kind != SSFFT_COMPLEX;
	const size_t cn = real ? n / 2 : n;
	const int max_n = dtype == SSFFT_F32 ? kMaxSubTransform : kMaxSubTransform / 2;
	if (cn == 0 || cn > (size_t)max_n) return false;
	if (!real && dtype == SSFFT_F32 && allow_staged != 2) {
		// two-CTA cluster schedule: asked for, or the default for long transforms when no other
		// shape was asked for
		const bool asked = knobs && knobs->pair > 0;
		const bool other = knobs && (!knobs->radices.empty() || knobs->emax || knobs->cta_threads ||
		                             knobs->precision == 1 || knobs->pair == 0);
		if (asked || (!other && pair_default((int)cn))) {
			if (pair_schedule((int)cn, s, knobs)) return true;
			if (asked) return false;
		}
	}
	if (knobs && knobs->pair > 0) return false;
	if (!make_schedule(dtype, (int)cn, kind_code(kind), real && (n & 1), batch, s, allow_staged, knobs)) return false;
	if (dir < 0) return true;
	// RealFFT (not half-shift), even length, plain kernel, two passes or more, a register radix
	// <= 8: fuse the split into the last pass (forward) / the pre-twiddle into the first pass
	// (inverse), with that radix moved to the end / the front.  debug switch fuse=0 turns it off for
	// plans made while it is set; an explicit radix order keeps the base schedule.
	// (below 256 reals the unfused kernel measured faster on GB300)
	const int fuse_knob = knobs ? knobs->fuse : -1;
	if (debug_knob("fuse", 1) == 0 || kind != SSFFT_REAL || (n & 1) || (n < 256 && fuse_knob != 1) || s.staged ||
	    s.tc || s.radices.size() < 2 || fuse_knob == 0)
		return true;
	int best = -1;
	for (size_t i = 0; i < s.radices.size(); ++i) {
		const int r = s.radices[i];
		if (specialised(r) && r >= 2 && r <= fuse_radix_limit() && (best < 0 || r < s.radices[best])) best = (int)i;
	}
	if (best < 0) return true;
	std::vector<int> rot = s.radices;
	const int r = rot[best];
	rot.erase(rot.begin() + best);
	if (dir == 0) rot.push_back(r);
	else rot.insert(rot.begin(), r);
	Knobs k = knobs ? *knobs : Knobs();
	k.radices = rot;
	Schedule f;
	if (!make_schedule(dtype, (int)cn, kind_code(kind), false, batch, f, allow_staged, &k, dir == 0 ? 1 : 2))
		return true;
	if (f.staged || f.tc) return true;
	s = f;
	return true;
}

// FP64 tables of a single-CTA schedule: pass twiddles, direct-pass roots, and for real kinds
// the split twiddles and half-shift rotations.
void single_tables(const Schedule &s, size_t n_real, std::vector<double> &tw, std::vector<double> &roots,
                          std::vector<double> &rtw, std::vector<double> &rot) {
	schedule_twiddles(s, tw, roots);
	if (s.kind == ssfft_cl::kComplex) return;
	const size_t h = (size_t)s.n;
	// twiddlesMinusI (signalsmith-fft.h:420-425) = -i e^{-2 pi i (k + d)/n}, d = 0 or 1/2
	for (size_t i = 0; i <= h / 2; ++i) {
		double re, im;
		if (s.kind == ssfft_cl::kRealHalfShift) unit_root(2 * i + 1, 2 * (unsigned long long)n_real, &re, &im);
		else unit_root(i, n_real, &re, &im);
		rtw.push_back(im);  // -i (re + i im) = im - i re
		rtw.push_back(-re);
	}
	if (s.kind == ssfft_cl::kRealHalfShift)
		// modifiedRotations (signalsmith-fft.h:426-432) = e^{-2 pi i k / n}
		for (size_t i = 0; i < h; ++i) {
			double re, im;
			unit_root(i, n_real, &re, &im);
			rot.push_back(re);
			rot.push_back(im);
		}
}

// The radix-r0 DFT (r0 <= 16) as the 32 x 32 real matrix of the tensor-core pass, transposed
// (row = output column): inputs [Re x_r | Im x_r], outputs [Re y_k | Im y_k] in 16-column halves,
// y_k = sum_r x_r e^{-2 pi i r k / r0}; zero outside r, k < r0.  FP64 roots, rounded to FP32.
void tc_matrix(int r0, std::vector<float> &bt) {
	bt.assign(32 * 32, 0.0f);
	for (int k = 0; k < r0; ++k)
		for (int r = 0; r < r0; ++r) {
			double re, im;  // e^{-2 pi i rk/r0} = c - i s
			unit_root((unsigned long long)r * k, (unsigned long long)r0, &re, &im);
			const float c = (float)re, sn = (float)-im;
			bt[k * 32 + r] = c;             // Re y_k += Re x_r c
			bt[k * 32 + 16 + r] = sn;       // Re y_k += Im x_r s
			bt[(16 + k) * 32 + r] = -sn;    // Im y_k -= Re x_r s
			bt[(16 + k) * 32 + 16 + r] = c; // Im y_k += Im x_r c
		}
}

long long resident_ctas(CUfunction fwd, CUfunction inv, const Schedule &s, int device) {
	int sms = 0;
	cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
	const int occ = std::min(jit_occupancy(fwd, s.cta_threads(), s.smem_bytes),
	                         jit_occupancy(inv, s.cta_threads(), s.smem_bytes));
	return (long long)std::max(1, occ) * std::max(1, sms);
}

// The plain batch kernel prefetches into L2 the input of the CTA this many blocks ahead: by
// default one wave of resident CTAs (measured on GB300: complex N=1024 77% -> 92% of the copy
// bandwidth, RealFFT N=3840 62% -> 70%).  Knob: quarter waves (0 = off); debug switch prefetch=0 turns
// it off for plans made while it is set.
long long prefetch_distance(const Schedule &s, const Knobs &k, long long resident) {
	if (s.staged || s.tc) return 0;
	if (debug_knob("prefetch", 1) == 0) return 0;
	const int quarters = k.prefetch >= 0 ? k.prefetch : 4;
	// (cluster-pair schedules count in transforms, two CTAs each)
	return resident * quarters / 4 / (s.pair ? 2 : 1);
}

// Whether (n, dtype, kind) runs in one CTA per transform (otherwise: multi-pass or Bluestein,
// which hold per-plan scratch).  A direct pass of a prime above 1024 is O(p^2) per point; such
// lengths go to Bluestein instead (even real lengths and complex ones).
bool plan_single_cta(size_t n, ssfft_dtype dtype, ssfft_kind kind) {
	Schedule d;
	if (!single_schedule(n, dtype, kind, 1, d)) return false;
	const bool odd_real = kind != SSFFT_COMPLEX && (n & 1);
	for (int r : d.radices)
		if (!specialised(r) && r > 1024 && !odd_real) return false;
	return true;
}

ssfft_status plan_prepare_launch(const Plan *p);

// Whether `s` is a long staged schedule the planner chose by itself (not asked for by the debug
// switch staged=1 or by shape knobs).
static bool long_staged_default(const Schedule &s, const Knobs &k) {
	return s.staged && s.dtype == SSFFT_F32 && s.n >= kLongStagedMin && s.per_cta == 1 &&
	       k.staging == 0 && debug_knob("staged", 0) != 1 && !k.cta_threads && !k.emax && !k.minb;
}

static ssfft_status plan_build_single(Plan *p) {
	Schedule &s = p->main.sch;
	// the default schedule decides whether n runs in one CTA; explicit or tuned knobs refine it
	if (!plan_single_cta(p->n, p->dtype, p->kind)) return SSFFT_ERR_UNSUPPORTED;
	p->knobs_inv = p->knobs;
	if (p->autotune > 0 && p->knobs.empty()) {
		Knobs best, best_inv;
		ssfft_status st = autotune_single(p, p->autotune, best, best_inv, p->tune_log);
		if (st != SSFFT_SUCCESS) return st;
		best.staging = best_inv.staging = p->knobs.staging;  // not a tuned choice
		p->knobs = best;
		p->knobs_inv = best_inv;
	}
	Schedule &si = p->main.sch_inv;
	if (!single_schedule(p->n, p->dtype, p->kind, p->batch, s, &p->knobs, 1, 0) ||
	    !single_schedule(p->n, p->dtype, p->kind, p->batch, si, &p->knobs_inv, 1, 1))
		return SSFFT_ERR_INVALID_VALUE;  // explicit knobs that do not fit this size
	const size_t smem_limit = device_smem_limit(p->device);
	if (s.smem_bytes > smem_limit || si.smem_bytes > smem_limit) return SSFFT_ERR_UNSUPPORTED;
	{
		// a long staged schedule the planner chose on its own (per direction: tuned forward and
		// inverse knobs may differ) stays only if its kernel compiles without spilling (the
		// persistent loop holds more registers than one pass list)
		const bool chk = long_staged_default(s, p->knobs), chk_i = long_staged_default(si, p->knobs_inv);
		if (chk || chk_i) {
			std::vector<CUfunction> fns;
			ssfft_status st = jit_kernels({s.name(false), si.name(true)}, std::max(s.smem_bytes, si.smem_bytes), fns);
			if (st != SSFFT_SUCCESS) return st;
			if (chk && jit_local_bytes(fns[0]) > kLongStagedLocalMax &&
			    !single_schedule(p->n, p->dtype, p->kind, p->batch, s, &p->knobs, 0, 0))
				return SSFFT_ERR_INVALID_VALUE;
			if (chk_i && jit_local_bytes(fns[1]) > kLongStagedLocalMax &&
			    !single_schedule(p->n, p->dtype, p->kind, p->batch, si, &p->knobs_inv, 0, 1))
				return SSFFT_ERR_INVALID_VALUE;
		}
	}
	// the inverse has its own pass tables when its passes differ
	const bool split = si.radices != s.radices || si.pair != s.pair;
	std::vector<double> tw, roots, rtw, rot, tw_i, roots_i, unused_rtw, unused_rot;
	single_tables(s, p->n, tw, roots, rtw, rot);
	if (split) single_tables(si, p->n, tw_i, roots_i, unused_rtw, unused_rot);
	const size_t sb = p->dtype == SSFFT_F32 ? 4 : 8;
	const size_t off_tw = 0;
	const size_t off_roots = align_up(off_tw + tw.size() * sb, 256);
	const size_t off_tw_i = align_up(off_roots + roots.size() * sb, 256);
	const size_t off_roots_i = align_up(off_tw_i + tw_i.size() * sb, 256);
	const size_t off_rtw = align_up(off_roots_i + roots_i.size() * sb, 256);
	const size_t off_rot = align_up(off_rtw + rtw.size() * sb, 256);
	std::vector<float> tcb;
	if (s.tc) tc_matrix(s.radices[0], tcb);
	const size_t off_tcb = align_up(off_rot + rot.size() * sb, 256);
	const size_t off_err = align_up(off_tcb + tcb.size() * 4, 256);
	const size_t total = align_up(off_err + 16, 256);
	std::vector<unsigned char> blob(total, 0);
	const std::pair<size_t, const std::vector<double> *> parts[] = {
	    {off_tw, &tw}, {off_roots, &roots}, {off_tw_i, &tw_i}, {off_roots_i, &roots_i}, {off_rtw, &rtw}, {off_rot, &rot}};
	for (const auto &pt : parts) {
		if (sb == 4) put_table<float>(blob, pt.first, *pt.second);
		else put_table<double>(blob, pt.first, *pt.second);
	}
	if (!tcb.empty()) std::memcpy(blob.data() + off_tcb, tcb.data(), tcb.size() * 4);
	cudaError_t e = cudaMalloc(&p->d_tables, total);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc(tables)");
	p->table_bytes = total;
	e = cudaMemcpy(p->d_tables, blob.data(), total, cudaMemcpyHostToDevice);
	if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy(tables)");
	const unsigned char *base = static_cast<const unsigned char *>(p->d_tables);
	p->main.tab.tw = base + off_tw;
	p->main.tab.roots = base + off_roots;
	p->main.tab.rtw = base + off_rtw;
	p->main.tab.rot = base + off_rot;
	p->main.tab.tcb = tcb.empty() ? nullptr : reinterpret_cast<const float *>(base + off_tcb);
	p->main.tab_inv = p->main.tab;
	if (split) {
		p->main.tab_inv.tw = base + off_tw_i;
		p->main.tab_inv.roots = base + off_roots_i;
	}
	p->main.err = reinterpret_cast<unsigned *>(static_cast<unsigned char *>(p->d_tables) + off_err);

	std::vector<CUfunction> fns;
	ssfft_status st = jit_kernels({s.name(false), si.name(true)}, std::max(s.smem_bytes, si.smem_bytes), fns);
	if (st != SSFFT_SUCCESS) return st;
	p->main.fwd = fns[0];
	p->main.inv = fns[1];
	{
		const long long resident = resident_ctas(fns[0], fns[0], s, p->device);
		const long long resident_i = resident_ctas(fns[1], fns[1], si, p->device);
		if (s.staged) p->main.grid_cap = (int)resident;
		if (si.staged) p->main.grid_cap_inv = (int)resident_i;
		p->main.pf_dist = prefetch_distance(s, p->knobs, resident);
		p->main.pf_dist_inv = prefetch_distance(si, p->knobs_inv, resident_i);
	}
	p->launches_per_exec = 1;
	// a staged plan also runs the plain kernel of its order (scattered offsets, inputs off a
	// 16-byte boundary): compile it now, so that no launch compiles (a server's first requests, a
	// stream capture)
	return plan_prepare_launch(p);
}

// scalar distances between consecutive transforms
void plan_dists(const Plan *p, int inverse, long long &in_dist, long long &out_dist) {
	const long long n = (long long)p->n, h2 = 2 * (long long)(p->n / 2);
	if (p->kind == SSFFT_COMPLEX) {
		in_dist = out_dist = 2 * n;
	} else if (!inverse) {
		in_dist = n;
		out_dist = h2;
	} else {
		in_dist = h2;
		out_dist = n;
	}
}

size_t plan_in_bytes(const Plan *p, int inverse, size_t batch) {
	long long di, dout;
	plan_dists(p, inverse, di, dout);
	return (size_t)di * batch * (p->dtype == SSFFT_F32 ? 4 : 8);
}

size_t plan_out_bytes(const Plan *p, int inverse, size_t batch) {
	long long di, dout;
	plan_dists(p, inverse, di, dout);
	return (size_t)dout * batch * (p->dtype == SSFFT_F32 ? 4 : 8);
}

// A staged plan given an input that is not 16-byte aligned runs the plain kernel of the same
// schedule (compiled on first use): u / ui the forward / inverse schedules (each direction with
// its own knobs, so that its pass tables match), fns their kernels.
static ssfft_status unstaged_kernels(const Plan *p, Schedule &u, Schedule &ui, std::vector<CUfunction> &fns) {
	const Schedule &st = p->main.sch, &sti = p->main.sch_inv;
	// the plan's own radix order per direction (its pass tables follow it)
	Knobs k = p->knobs, ki = p->knobs_inv;
	k.radices = st.radices;
	ki.radices = sti.radices;
	if (!make_schedule(st.dtype, st.n, st.kind, st.odd, p->batch, u, 0, &k) ||
	    !make_schedule(sti.dtype, sti.n, sti.kind, sti.odd, p->batch, ui, 0, &ki))
		return SSFFT_ERR_UNSUPPORTED;
	// a direction that is not staged keeps its own kernel
	if (!st.staged) u = st;
	if (!sti.staged) ui = sti;
	return jit_kernels({u.name(false), ui.name(true)}, std::max(u.smem_bytes, ui.smem_bytes), fns);
}

// Compiles (and loads) what a later launch of `p` may need beyond the plan's own kernels, so that
// the launch makes no module-loading call (e.g. inside a stream capture).
ssfft_status plan_prepare_launch(const Plan *p) {
	if (!p->main.sch.staged && !p->main.sch_inv.staged) return SSFFT_SUCCESS;
	Schedule u, ui;
	std::vector<CUfunction> fns;
	return unstaged_kernels(p, u, ui, fns);
}

static ssfft_status launch_unstaged(const Plan *p, int inverse, const void *in, void *out, size_t batch,
                                    cudaStream_t s, const long long *offs = nullptr,
                                    const long long *offs_out = nullptr) {
	Schedule u, ui;
	std::vector<CUfunction> fns;
	ssfft_status rc = unstaged_kernels(p, u, ui, fns);
	if (rc != SSFFT_SUCCESS) return rc;
	const Schedule &sch = inverse ? ui : u;
	const Tables &tab = inverse ? p->main.tab_inv : p->main.tab;
	ssfft_cl::Args a;
	std::memset(&a, 0, sizeof a);
	a.in = in;
	a.out = out;
	a.batch = (long long)batch;
	plan_dists(p, inverse, a.in_dist, a.out_dist);
	a.tw = tab.tw;
	a.rtw = tab.rtw;
	a.rot = tab.rot;
	a.roots = tab.roots;
	a.offs = offs;
	a.offs_out = offs_out;
	const long long grid = sch.grid((long long)batch);
	if (grid > 0x7fffffffLL) return SSFFT_ERR_INVALID_SIZE;
	return jit_launch(inverse ? fns[1] : fns[0], (unsigned)grid, (unsigned)sch.cta_threads(), sch.smem_bytes, s, &a);
}

// Transforms at scattered offsets: transform g reads d_offs[g] scalars into `in` and writes
// d_offs_out[g] (d_offs[g] when d_offs_out is null) scalars into `out` (uneven-size batches;
// requests served straight from their host buffers).
ssfft_status launch_batch_offs(const Plan *p, int inverse, const void *in, void *out, size_t batch,
                               const long long *d_offs, cudaStream_t s, const long long *d_offs_out) {
	if (batch == 0) return SSFFT_SUCCESS;
	if (p->large) return SSFFT_ERR_UNSUPPORTED;
	const Schedule &sch = inverse ? p->main.sch_inv : p->main.sch;
	if (sch.staged) return launch_unstaged(p, inverse, in, out, batch, s, d_offs, d_offs_out);
	const Tables &tab = inverse ? p->main.tab_inv : p->main.tab;
	ssfft_cl::Args a;
	std::memset(&a, 0, sizeof a);
	a.in = in;
	a.out = out;
	a.batch = (long long)batch;
	plan_dists(p, inverse, a.in_dist, a.out_dist);
	a.tw = tab.tw;
	a.rtw = tab.rtw;
	a.rot = tab.rot;
	a.roots = tab.roots;
	a.tcb = tab.tcb;
	a.err = p->main.err;
	a.spin_limit = 1u << 22;
	a.offs = d_offs;
	a.offs_out = d_offs_out;
	a.pf_dist = inverse ? p->main.pf_dist_inv : p->main.pf_dist;
	const long long grid = sch.grid((long long)batch);
	if (grid > 0x7fffffffLL) return SSFFT_ERR_INVALID_SIZE;
	return jit_launch(inverse ? p->main.inv : p->main.fwd, (unsigned)grid, (unsigned)sch.cta_threads(),
	                  sch.smem_bytes, s, &a);
}

ssfft_status launch_batch(const Plan *p, int inverse, const void *in, void *out, size_t batch, cudaStream_t s) {
	if (batch == 0) return SSFFT_SUCCESS;
	const Schedule &sch = inverse ? p->main.sch_inv : p->main.sch;
	const Tables &tab = inverse ? p->main.tab_inv : p->main.tab;
	ssfft_cl::Args a;
	std::memset(&a, 0, sizeof a);
	a.in = in;
	a.out = out;
	a.batch = (long long)batch;
	plan_dists(p, inverse, a.in_dist, a.out_dist);
	a.tw = tab.tw;
	a.rtw = tab.rtw;
	a.rot = tab.rot;
	a.roots = tab.roots;
	a.err = p->main.err;
	a.spin_limit = 1u << 22;
	a.in_bytes = sch.in_bytes;
	a.tcb = tab.tcb;
	a.pf_dist = inverse ? p->main.pf_dist_inv : p->main.pf_dist;
	long long grid = sch.grid((long long)batch);
	if (sch.staged) {
		if ((uintptr_t)in % 16) return launch_unstaged(p, inverse, in, out, batch, s);
		grid = std::min<long long>(grid, inverse ? p->main.grid_cap_inv : p->main.grid_cap);
		if (grid < 1) return SSFFT_ERR_INVALID_VALUE;
	}
	if (grid > 0x7fffffffLL) return SSFFT_ERR_INVALID_SIZE;
	return jit_launch(inverse ? p->main.inv : p->main.fwd, (unsigned)grid, (unsigned)sch.cta_threads(),
	                  sch.smem_bytes, s, &a);
}

}  // namespace ssfft

// ====================================================================== C ABI

using namespace ssfft;

extern "C" {

const char *ssfft_status_string(ssfft_status s) {
	switch (s) {
	case SSFFT_SUCCESS: return "success";
	case SSFFT_ERR_INVALID_SIZE: return "invalid size";
	case SSFFT_ERR_INVALID_VALUE: return "invalid value";
	case SSFFT_ERR_CUDA: return "CUDA error";
	case SSFFT_ERR_ALLOC: return "allocation failed";
	case SSFFT_ERR_UNSUPPORTED: return "unsupported";
	case SSFFT_ERR_BUDGET: return "exceeds HBM budget";
	case SSFFT_ERR_TIMEOUT: return "timed out";
	case SSFFT_ERR_NOT_READY: return "not ready";
	case SSFFT_ERR_SHUTDOWN: return "shut down";
	}
	return "unknown status";
}

const char *ssfft_last_cuda_error(void) {
	const char *j = jit_last_log();
	return (j && *j) ? j : g_last_error.c_str();
}

size_t ssfft_size_minimum(size_t n) { return size_minimum(n); }
size_t ssfft_size_maximum(size_t n) { return size_maximum(n); }
size_t ssfft_real_size_minimum(size_t n) { return (size_minimum((n - 1) / 2) + 1) * 2; }
size_t ssfft_real_size_maximum(size_t n) { return size_minimum(n / 2) * 2; }
size_t ssfft_size_minimum_smooth(size_t n) { return smooth_minimum(n); }
size_t ssfft_size_maximum_smooth(size_t n) { return smooth_maximum(n); }
size_t ssfft_real_size_minimum_smooth(size_t n) {
	if (n == 0) return 0;
	const size_t h = smooth_minimum(n / 2 + (n & 1));
	return h && h <= SIZE_MAX / 2 ? 2 * h : 0;
}
size_t ssfft_real_size_maximum_smooth(size_t n) { return 2 * smooth_maximum(n / 2); }

static std::atomic<size_t> g_plans_created{0};

ssfft_status ssfft_plan_create(ssfft_plan_t *out, size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch) {
	return ssfft_plan_create_ex(out, n, dtype, kind, batch, nullptr);
}

ssfft_status ssfft_plan_create_ex(ssfft_plan_t *out, size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch,
                                  const ssfft_plan_options *opt) {
	if (!out) return SSFFT_ERR_INVALID_VALUE;
	*out = nullptr;
	if (dtype != SSFFT_F32 && dtype != SSFFT_F64) return SSFFT_ERR_INVALID_VALUE;
	if (kind != SSFFT_COMPLEX && kind != SSFFT_REAL && kind != SSFFT_REAL_HALFSHIFT) return SSFFT_ERR_INVALID_VALUE;
	if (n == 0 || (kind != SSFFT_COMPLEX && n < 2)) return SSFFT_ERR_INVALID_SIZE;
	if (n > (size_t)1 << 31) return SSFFT_ERR_INVALID_SIZE;
	if (batch == 0) batch = 1;
	Plan *p = new (std::nothrow) Plan();
	if (!p) return SSFFT_ERR_ALLOC;
	p->n = n;
	p->dtype = dtype;
	p->kind = kind;
	p->batch = batch;
	static const int autotune_env = [] {
		const long long e = debug_knob("autotune", 0);
		return (int)std::max(0ll, std::min(2ll, e));
	}();
	p->autotune = autotune_env;
	if (opt) {
		if (opt->autotune < 0 || opt->autotune > 2 || opt->cta_threads < 0 || opt->cta_threads > kMaxCtaThreads ||
		    opt->values_per_thread < 0 || opt->values_per_thread > 2 * kElemsPerThread || opt->min_ctas_per_sm < 0 ||
		    opt->min_ctas_per_sm > 32) {
			delete p;
			return SSFFT_ERR_INVALID_VALUE;
		}
		if (opt->autotune) p->autotune = opt->autotune;
		p->knobs.cta_threads = opt->cta_threads;
		p->knobs.emax = opt->values_per_thread;
		p->knobs.minb = opt->min_ctas_per_sm;
		if (opt->precision != SSFFT_PRECISION_FP32 && opt->precision != SSFFT_PRECISION_SPLIT_BF16) {
			delete p;
			return SSFFT_ERR_INVALID_VALUE;
		}
		p->knobs.precision = opt->precision;
		if (opt->prefetch_quarter_waves < -1 || opt->prefetch_quarter_waves > 64) {
			delete p;
			return SSFFT_ERR_INVALID_VALUE;
		}
		if (opt->prefetch_quarter_waves != 0) p->knobs.prefetch = std::max(0, opt->prefetch_quarter_waves);
		for (int i = 0; i < 24 && opt->radices[i] > 0; ++i) p->knobs.radices.push_back(opt->radices[i]);
		if (!p->knobs.radices.empty()) p->knobs.fuse = 0;  // the caller's order is kept as given
		if (opt->fuse_split < -1 || opt->fuse_split > 1) {
			delete p;
			return SSFFT_ERR_INVALID_VALUE;
		}
		if (opt->fuse_split) p->knobs.fuse = opt->fuse_split > 0 ? 1 : 0;
		if (opt->cluster_split < -1 || opt->cluster_split > 24 ||
		    (opt->cluster_split > 0 && (int)p->knobs.radices.size() <= opt->cluster_split)) {
			delete p;
			return SSFFT_ERR_INVALID_VALUE;
		}
		if (opt->cluster_split) p->knobs.pair = opt->cluster_split > 0 ? opt->cluster_split : 0;
		if (opt->staging < -1 || opt->staging > 1) {
			delete p;
			return SSFFT_ERR_INVALID_VALUE;
		}
		p->knobs.staging = opt->staging;
	}
	cudaError_t e = cudaGetDevice(&p->device);
	ssfft_status st = e == cudaSuccess ? SSFFT_SUCCESS : cuda_fail(e, "cudaGetDevice");
	if (st == SSFFT_SUCCESS) {
		st = plan_build_single(p);
		if (st == SSFFT_ERR_UNSUPPORTED) st = plan_build_large(p);
	}
	if (st != SSFFT_SUCCESS) {
		plan_release(p);
		delete p;
		return st;
	}
	*out = reinterpret_cast<ssfft_plan_t>(p);
	g_plans_created.fetch_add(1, std::memory_order_relaxed);
	return SSFFT_SUCCESS;
}

size_t ssfft_plans_created(void) { return g_plans_created.load(std::memory_order_relaxed); }

ssfft_status ssfft_plan_tuning(ssfft_plan_t plan, char *choice, size_t choice_len, char *log, size_t log_len) {
	if (!plan) return SSFFT_ERR_INVALID_VALUE;
	const Plan *p = reinterpret_cast<const Plan *>(plan);
	auto put = [](const std::string &src, char *dst, size_t len) {
		if (!dst || !len) return;
		const size_t k = std::min(len - 1, src.size());
		std::memcpy(dst, src.data(), k);
		dst[k] = 0;
	};
	std::string ch = p->knobs.str();
	if (p->knobs_inv.str() != ch) ch += " | inverse: " + p->knobs_inv.str();
	put(p->large ? std::string("multi-pass") : ch, choice, choice_len);
	put(p->tune_log, log, log_len);
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_plan_kernel(ssfft_plan_t plan, int inverse, char *name, size_t len) {
	if (!plan || !name || !len) return SSFFT_ERR_INVALID_VALUE;
	const Plan *p = reinterpret_cast<const Plan *>(plan);
	const std::string k = p->large ? std::string("multi-pass") : (inverse ? p->main.sch_inv : p->main.sch).name(inverse != 0);
	const size_t m = std::min(len - 1, k.size());
	std::memcpy(name, k.data(), m);
	name[m] = 0;
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_plan_destroy(ssfft_plan_t plan) {
	if (!plan) return SSFFT_ERR_INVALID_VALUE;
	Plan *p = reinterpret_cast<Plan *>(plan);
	plan_release(p);
	delete p;
	return SSFFT_SUCCESS;
}

size_t ssfft_plan_size(ssfft_plan_t plan) { return plan ? reinterpret_cast<Plan *>(plan)->n : 0; }
size_t ssfft_plan_batch(ssfft_plan_t plan) { return plan ? reinterpret_cast<Plan *>(plan)->batch : 0; }
size_t ssfft_plan_device_bytes(ssfft_plan_t plan) {
	if (!plan) return 0;
	const Plan *p = reinterpret_cast<Plan *>(plan);
	return p->table_bytes + p->scratch_bytes + p->stage_bytes;
}

ssfft_status ssfft_plan_describe(ssfft_plan_t plan, int *npasses, int *radices, int cap, int *threads_per_transform,
                                 int *transforms_per_cta, int *kernel_launches) {
	if (!plan) return SSFFT_ERR_INVALID_VALUE;
	const Plan *p = reinterpret_cast<Plan *>(plan);
	if (p->large) {
		std::vector<long long> F;
		large_describe(p->n, p->dtype, p->kind, F);
		if (npasses) *npasses = (int)F.size();
		if (radices)
			for (int i = 0; i < (int)F.size() && i < cap; ++i) radices[i] = (int)F[i];
		if (threads_per_transform) *threads_per_transform = 0;
		if (transforms_per_cta) *transforms_per_cta = 0;
		if (kernel_launches) *kernel_launches = p->launches_per_exec;
		return SSFFT_SUCCESS;
	}
	const Schedule &s = p->main.sch;
	if (npasses) *npasses = (int)s.radices.size();
	if (radices)
		for (int i = 0; i < (int)s.radices.size() && i < cap; ++i) radices[i] = s.radices[i];
	if (threads_per_transform) *threads_per_transform = s.threads;
	if (transforms_per_cta) *transforms_per_cta = s.per_cta;
	if (kernel_launches) *kernel_launches = p->launches_per_exec;
	return SSFFT_SUCCESS;
}

static ssfft_status check_exec(const Plan *p, const void *in, void *out) {
	if (!p || !in || !out) return SSFFT_ERR_INVALID_VALUE;
	const size_t align = p->dtype == SSFFT_F32 ? 8 : 16;
	// real data are read/written as {x[2k], x[2k+1]} pairs unless the real length is odd
	const size_t need = p->kind != SSFFT_COMPLEX && (p->n & 1) ? align / 2 : align;
	if ((uintptr_t)in % need || (uintptr_t)out % need) return SSFFT_ERR_INVALID_VALUE;
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_exec_batch(ssfft_plan_t plan, int inverse, const void *d_in, void *d_out, size_t batch,
                              void *stream) {
	Plan *p = reinterpret_cast<Plan *>(plan);
	ssfft_status st = check_exec(p, d_in, d_out);
	if (st != SSFFT_SUCCESS) return st;
	if (batch > p->batch) return SSFFT_ERR_INVALID_SIZE;
	cudaStream_t s = static_cast<cudaStream_t>(stream);
	if (p->large) return launch_large(p, inverse, d_in, d_out, batch, s);
	return launch_batch(p, inverse, d_in, d_out, batch, s);
}

ssfft_status ssfft_plan_error(ssfft_plan_t plan, unsigned *flags) {
	if (!plan || !flags) return SSFFT_ERR_INVALID_VALUE;
	Plan *p = reinterpret_cast<Plan *>(plan);
	*flags = 0;
	if (!p->main.err) return SSFFT_SUCCESS;
	cudaError_t e = cudaMemcpy(flags, p->main.err, sizeof(unsigned), cudaMemcpyDeviceToHost);
	if (e != cudaSuccess) return cuda_fail(e, "plan_error read");
	e = cudaMemset(p->main.err, 0, sizeof(unsigned));
	if (e != cudaSuccess) return cuda_fail(e, "plan_error clear");
	return *flags ? SSFFT_ERR_TIMEOUT : SSFFT_SUCCESS;
}

ssfft_status ssfft_exec(ssfft_plan_t plan, int inverse, const void *d_in, void *d_out, void *stream) {
	if (!plan) return SSFFT_ERR_INVALID_VALUE;
	return ssfft_exec_batch(plan, inverse, d_in, d_out, reinterpret_cast<Plan *>(plan)->batch, stream);
}

// Failure-detection check of the staged kernel: one launch over four `n`-point complex FP32
// transforms whose barrier expects each group's bytes while no copy is issued (a lost copy), with
// `spin_limit` wait attempts.  The kernel must give up, raise the error flag (returned in *flags)
// and return; nothing is in flight when it does, and the context stays usable.
ssfft_status ssfft_diag_staged_timeout(size_t n, unsigned spin_limit, unsigned *flags) {
	if (!flags || n < 16 || n > (size_t)kMaxSubTransform) return SSFFT_ERR_INVALID_VALUE;
	*flags = 0;
	Schedule s;
	if (!make_schedule(SSFFT_F32, (int)n, 0, false, 4, s, 2) || !s.staged) return SSFFT_ERR_UNSUPPORTED;
	std::vector<double> tw, roots, rtw, rot;
	single_tables(s, n, tw, roots, rtw, rot);
	std::vector<float> blob(tw.begin(), tw.end());
	blob.insert(blob.end(), roots.begin(), roots.end());
	const size_t tab_bytes = std::max<size_t>(blob.size() * 4, 16), io_bytes = 4 * n * 8;
	void *d_tab = nullptr, *d_in = nullptr, *d_out = nullptr;
	unsigned *d_err = nullptr;
	cudaError_t e = cudaMalloc(&d_tab, tab_bytes);
	if (e == cudaSuccess) e = cudaMalloc(&d_err, sizeof(unsigned));
	if (e == cudaSuccess) e = cudaMalloc(&d_in, io_bytes);
	if (e == cudaSuccess) e = cudaMalloc(&d_out, io_bytes);
	if (e == cudaSuccess && !blob.empty()) e = cudaMemcpy(d_tab, blob.data(), blob.size() * 4, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemset(d_err, 0, sizeof(unsigned));
	if (e == cudaSuccess) e = cudaMemset(d_in, 0, io_bytes);
	ssfft_status st = e == cudaSuccess ? SSFFT_SUCCESS : cuda_fail(e, "diag setup");
	std::vector<CUfunction> fns;
	if (st == SSFFT_SUCCESS) st = jit_kernels({s.name(false)}, s.smem_bytes, fns);
	if (st == SSFFT_SUCCESS) {
		ssfft_cl::Args a;
		std::memset(&a, 0, sizeof a);
		a.in = d_in;
		a.out = d_out;
		a.batch = 4;
		a.in_dist = a.out_dist = 2 * (long long)n;
		a.tw = d_tab;
		a.roots = static_cast<const float *>(d_tab) + tw.size();
		a.err = d_err;
		a.spin_limit = spin_limit;
		a.in_bytes = s.in_bytes;
		a.drop_copy = 1;
		const unsigned grid = (unsigned)((4 + s.per_cta - 1) / s.per_cta);
		st = jit_launch(fns[0], grid, (unsigned)s.cta_threads(), s.smem_bytes, nullptr, &a);
	}
	if (st == SSFFT_SUCCESS) {
		e = cudaDeviceSynchronize();
		if (e == cudaSuccess) e = cudaMemcpy(flags, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost);
		if (e != cudaSuccess) st = cuda_fail(e, "diag sync");
	}
	cudaFree(d_tab);
	cudaFree(d_err);
	cudaFree(d_in);
	cudaFree(d_out);
	return st;
}

// ---------------------------------------------------------------- diagnostics (no GPU needed)

// Compile the kernels a plan of this shape would use (build-time check).
static thread_local Knobs g_diag_knobs;  // options of the schedule diagnostics in this thread
static thread_local int g_diag_dir = 0;   // direction whose schedule info / tables report

ssfft_status ssfft_schedule_direction(int inverse) {
	g_diag_dir = inverse ? 1 : 0;
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_schedule_options(const ssfft_plan_options *opt) {
	g_diag_knobs = Knobs();
	if (!opt) return SSFFT_SUCCESS;
	if (opt->precision != SSFFT_PRECISION_FP32 && opt->precision != SSFFT_PRECISION_SPLIT_BF16)
		return SSFFT_ERR_INVALID_VALUE;
	g_diag_knobs.cta_threads = opt->cta_threads;
	g_diag_knobs.emax = opt->values_per_thread;
	g_diag_knobs.minb = opt->min_ctas_per_sm;
	g_diag_knobs.precision = opt->precision;
	for (int i = 0; i < 24 && opt->radices[i] > 0; ++i) g_diag_knobs.radices.push_back(opt->radices[i]);
	if (!g_diag_knobs.radices.empty()) g_diag_knobs.fuse = 0;
	if (opt->fuse_split) g_diag_knobs.fuse = opt->fuse_split > 0 ? 1 : 0;
	if (opt->cluster_split) g_diag_knobs.pair = opt->cluster_split > 0 ? opt->cluster_split : 0;
	if (opt->staging < -1 || opt->staging > 1) return SSFFT_ERR_INVALID_VALUE;
	g_diag_knobs.staging = opt->staging;
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_diag_tc_tile(const float *h_a, const float *h_bt, float *h_d, unsigned *flags) {
	if (!h_a || !h_bt || !h_d || !flags) return SSFFT_ERR_INVALID_VALUE;
	*flags = 0;
	float *d_a = nullptr, *d_b = nullptr, *d_d = nullptr;
	unsigned *d_err = nullptr;
	cudaError_t e = cudaMalloc(&d_a, 128 * 32 * 4);
	if (e == cudaSuccess) e = cudaMalloc(&d_b, 32 * 32 * 4);
	if (e == cudaSuccess) e = cudaMalloc(&d_d, 128 * 32 * 4);
	if (e == cudaSuccess) e = cudaMalloc(&d_err, sizeof(unsigned));
	if (e == cudaSuccess) e = cudaMemcpy(d_a, h_a, 128 * 32 * 4, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemcpy(d_b, h_bt, 32 * 32 * 4, cudaMemcpyHostToDevice);
	if (e == cudaSuccess) e = cudaMemset(d_d, 0, 128 * 32 * 4);
	if (e == cudaSuccess) e = cudaMemset(d_err, 0, sizeof(unsigned));
	ssfft_status st = e == cudaSuccess ? SSFFT_SUCCESS : cuda_fail(e, "tc tile setup");
	const size_t smem = 3 * ssfft_cl::kTcAPart + 3 * ssfft_cl::kTcBPart + 16;
	std::vector<CUfunction> fns;
	if (st == SSFFT_SUCCESS) st = jit_kernels({"ssfft_cl::tc_tile_check<0>"}, smem, fns);
	if (st == SSFFT_SUCCESS) {
		ssfft_cl::Args a;
		std::memset(&a, 0, sizeof a);
		a.in = d_a;
		a.out = d_d;
		a.tcb = d_b;
		a.err = d_err;
		a.spin_limit = 1u << 20;
		st = jit_launch(fns[0], 1, 128, smem, nullptr, &a);
	}
	if (st == SSFFT_SUCCESS) {
		e = cudaDeviceSynchronize();
		if (e == cudaSuccess) e = cudaMemcpy(h_d, d_d, 128 * 32 * 4, cudaMemcpyDeviceToHost);
		if (e == cudaSuccess) e = cudaMemcpy(flags, d_err, sizeof(unsigned), cudaMemcpyDeviceToHost);
		if (e != cudaSuccess) st = cuda_fail(e, "tc tile");
	}
	cudaFree(d_a);
	cudaFree(d_b);
	cudaFree(d_d);
	cudaFree(d_err);
	return st;
}

ssfft_status ssfft_jit_check(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, const char *arch,
                             size_t *image_bytes) {
	Schedule s, si;
	if (!single_schedule(n, dtype, kind, batch, s, &g_diag_knobs, 1, 0) ||
	    !single_schedule(n, dtype, kind, batch, si, &g_diag_knobs, 1, 1))
		return large_jit_check(n, dtype, kind, arch ? arch : "sm_103a", image_bytes);
	return jit_compile_only({s.name(false), si.name(true)}, arch ? arch : "sm_103a", image_bytes);
}

ssfft_status ssfft_diag_large_spec(size_t n, ssfft_dtype dtype, ssfft_kind kind, char *json, size_t json_len,
                                   void *blob, size_t *blob_bytes) {
	if (!blob_bytes) return SSFFT_ERR_INVALID_VALUE;
	if (plan_single_cta(n, dtype, kind)) return SSFFT_ERR_UNSUPPORTED;  // not a multi-pass plan
	std::string j;
	std::vector<unsigned char> b;
	const ssfft_status st = large_spec(n, dtype, kind, j, b);
	if (st != SSFFT_SUCCESS) return st;
	if (json && json_len) {
		if (j.size() + 1 > json_len) return SSFFT_ERR_INVALID_VALUE;
		std::memcpy(json, j.c_str(), j.size() + 1);
	}
	if (blob) {
		if (*blob_bytes < b.size()) return SSFFT_ERR_INVALID_VALUE;
		std::memcpy(blob, b.data(), b.size());
	}
	*blob_bytes = b.size();
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_schedule_info(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, int *radices, int cap,
                                 int *npasses, int *threads, int *per_cta, size_t *smem_bytes) {
	Schedule s;
	if (!single_schedule(n, dtype, kind, batch, s, &g_diag_knobs, 1, g_diag_dir)) return SSFFT_ERR_UNSUPPORTED;
	if (npasses) *npasses = (int)s.radices.size();
	if (radices)
		for (int i = 0; i < (int)s.radices.size() && i < cap; ++i) radices[i] = s.radices[i];
	if (threads) *threads = s.threads;
	if (per_cta) *per_cta = s.per_cta;
	if (smem_bytes) *smem_bytes = s.smem_bytes;
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_schedule_name(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, int inverse, char *buf,
                                 size_t cap) {
	Schedule s;
	if (!single_schedule(n, dtype, kind, batch, s, &g_diag_knobs, 1, inverse ? 1 : 0)) return SSFFT_ERR_UNSUPPORTED;
	const std::string name = s.name(inverse != 0);
	if (!buf || cap < name.size() + 1) return SSFFT_ERR_INVALID_VALUE;
	std::memcpy(buf, name.c_str(), name.size() + 1);
	return SSFFT_SUCCESS;
}

ssfft_status ssfft_schedule_tables(size_t n, ssfft_dtype dtype, ssfft_kind kind, size_t batch, double *tw,
                                   size_t *ntw, double *roots, size_t *nroots, double *rtw, size_t *nrtw, double *rot,
                                   size_t *nrot) {
	Schedule s;
	if (!single_schedule(n, dtype, kind, batch, s, &g_diag_knobs, 1, g_diag_dir)) return SSFFT_ERR_UNSUPPORTED;
	std::vector<double> vtw, vroots, vrtw, vrot;
	single_tables(s, n, vtw, vroots, vrtw, vrot);
	const std::vector<double> *src[4] = {&vtw, &vroots, &vrtw, &vrot};
	double *dst[4] = {tw, roots, rtw, rot};
	size_t *cnt[4] = {ntw, nroots, nrtw, nrot};
	for (int i = 0; i < 4; ++i) {
		if (!cnt[i]) return SSFFT_ERR_INVALID_VALUE;
		if (dst[i]) {
			if (*cnt[i] < src[i]->size()) return SSFFT_ERR_INVALID_VALUE;
			std::memcpy(dst[i], src[i]->data(), src[i]->size() * sizeof(double));
		}
		*cnt[i] = src[i]->size();
	}
	return SSFFT_SUCCESS;
}

}  // extern "C"

// tests/cpp/dropin_tests.cpp -- the reference test suite's checks (tests/00-fft.cpp and
// tests/01-real.cpp of Signalsmith FFT), written against the drop-in header
// include/signalsmith-fft.h so that they exercise the GPU library through the same API calls a
// reference user makes.  Built and run by tests/test_cpp_dropin.py; exit status 0 = all passed.
//
// Checks: individual-bin known answers, linearity, inverse round trip (first harmonic and
// random), the fast-size rules, real and half-shifted real against the complex transform
// (DC/Nyquist packing, untouched second half of the output), and the device-pointer overloads.
#include <cuda_runtime_api.h>

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "signalsmith-fft.h"

using std::complex;
using std::vector;

static int failures = 0;
#define CHECK(cond, ...)                         \
	do {                                         \
		if (!(cond)) {                           \
			std::printf("FAIL %s:%d ", __FILE__, __LINE__); \
			std::printf(__VA_ARGS__);            \
			std::printf("\n");                   \
			++failures;                          \
		}                                        \
	} while (0)

static std::mt19937_64 rng(12345);
static double urand() { return std::uniform_real_distribution<double>(-0.5, 0.5)(rng); }

// relative error with the reference tests' energy term (|a|^4 + |b|^4, tests/tests-common.h)
template <typename T>
static bool close_enough(const vector<complex<T>> &a, const vector<complex<T>> &b, double tol = 1e-6) {
	if (a.size() != b.size()) return false;
	double err = 0, energy = 0;
	for (size_t i = 0; i < a.size(); ++i) {
		err += std::norm(complex<double>(a[i]) - complex<double>(b[i]));
		energy += std::norm(complex<double>(a[i]) * complex<double>(a[i])) +
		          std::norm(complex<double>(b[i]) * complex<double>(b[i]));
	}
	return energy == 0 || std::sqrt(err / energy) < tol;
}

static vector<int> test_sizes() {
	return {1, 2, 4, 8, 16, 32, 64, 128, 256, 3, 6, 9, 12, 18, 24, 5, 10, 15, 20, 25, 7, 14, 21, 28, 49, 11, 13, 17,
	        19, 22, 23};
}

template <typename T>
static void individual_bins(double tol) {
	for (int n : test_sizes()) {
		signalsmith::FFT<T> fft(n);
		vector<complex<T>> in(n), copy(n), out(n), expected(n);
		for (int bin = 0; bin < n; ++bin) {
			for (int i = 0; i < n; ++i) {
				double ph = 2 * M_PI * i * bin / n;
				in[i] = copy[i] = complex<T>((T)std::cos(ph), (T)std::sin(ph));
				expected[i] = (i == bin) ? complex<T>((T)n) : complex<T>(0);
			}
			fft.fft(in, out);
			CHECK(in == copy, "input changed n=%d", n);
			CHECK(close_enough(out, expected, tol), "bin n=%d bin=%d", n, bin);
		}
	}
}

template <typename T>
static void linearity(double tol) {
	for (int n : test_sizes()) {
		signalsmith::FFT<T> fft(n);
		vector<complex<T>> a(n), b(n), ab(n), fa(n), fb(n), fab(n), sum(n);
		for (int i = 0; i < n; ++i) {
			a[i] = complex<T>((T)urand(), (T)urand());
			b[i] = complex<T>((T)urand(), (T)urand());
			ab[i] = a[i] + b[i];
		}
		fft.fft(a, fa);
		fft.fft(b, fb);
		fft.fft(ab, fab);
		for (int i = 0; i < n; ++i) sum[i] = fa[i] + fb[i];
		CHECK(close_enough(fab, sum, tol), "linearity n=%d", n);
	}
}

template <typename T>
static void inverse(int harmonic, double tol) {
	for (int n : test_sizes()) {
		vector<complex<T>> in(n), spec(n), out(n), expected(n);
		for (int i = 0; i < n; ++i) {
			if (harmonic >= 0) {
				double ph = 2 * M_PI * i * harmonic / n;
				in[i] = complex<T>((T)std::cos(ph), (T)std::sin(ph));
			} else {
				in[i] = complex<T>((T)urand(), (T)urand());
			}
			expected[i] = in[i] * (T)n;
		}
		signalsmith::FFT<T> fft(n);
		fft.fft(in, spec);
		fft.ifft(spec, out);
		CHECK(close_enough(out, expected, tol), "inverse n=%d harmonic=%d", n, harmonic);
	}
}

static void sizes() {
	for (size_t i = 1; i < 1000; ++i) {
		size_t above = signalsmith::FFT<double>::sizeMinimum(i), below = signalsmith::FFT<double>::sizeMaximum(i);
		CHECK(above >= i && below <= i, "size order %zu", i);
		for (size_t v : {above, below}) {
			size_t m = v, threes = 0, fives = 0;
			while (m % 2 == 0) m /= 2;
			while (m % 3 == 0) m /= 3, ++threes;
			while (m % 5 == 0) m /= 5, ++fives;
			CHECK(m == 1 && threes + fives <= 2, "fast size %zu -> %zu", i, v);
		}
	}
	signalsmith::FFT<double> f(1025, 1);
	CHECK(f.size() == 1152 || f.size() == signalsmith::FFT<double>::sizeMinimum(1025), "fastDirection");
	CHECK(f.setSizeMaximum(1025) == signalsmith::FFT<double>::sizeMaximum(1025), "setSizeMaximum");
}

template <bool modified>
static void real_vs_complex() {
	for (int n = 2; n < 100; n += 2) {
		vector<complex<double>> cin(n), cmid(n), cout(n);
		vector<double> rin(n), rout(n);
		vector<complex<double>> rmid(n);
		signalsmith::FFT<double> fft(n);
		typename std::conditional<modified, signalsmith::ModifiedRealFFT<double>, signalsmith::RealFFT<double>>::type
		    real(n);
		for (int i = 0; i < n; ++i) cin[i] = rin[i] = urand();
		if (modified)
			for (int i = 0; i < n; ++i) cin[i] *= std::polar(1.0, -M_PI * i / n);
		for (int i = n / 2; i < n; ++i) rmid[i] = complex<double>(52, 21);
		fft.fft(cin, cmid);
		real.fft(rin, rmid);
		if (!modified) {
			CHECK(std::abs(cmid[0].real() - rmid[0].real()) < 1e-6, "DC n=%d", n);
			CHECK(std::abs(cmid[n / 2].real() - rmid[0].imag()) < 1e-6, "Nyquist n=%d", n);
		}
		for (int i = modified ? 0 : 1; i < n / 2; ++i)
			CHECK(std::abs(cmid[i] - rmid[i]) < n * 1e-6, "bin n=%d i=%d", n, i);
		for (int i = n / 2; i < n; ++i) CHECK(rmid[i] == complex<double>(52, 21), "second half touched n=%d", n);
		fft.ifft(cmid, cout);
		real.ifft(rmid, rout);
		if (modified)
			for (int i = 0; i < n; ++i) cout[i] *= std::polar(1.0, M_PI * i / n);
		for (int i = 0; i < n; ++i) CHECK(std::abs(cout[i].real() - rout[i]) < n * 1e-6, "inverse n=%d i=%d", n, i);
	}
}

// Return values of setSize / setSizeMinimum / setSizeMaximum and size(), against the table the
// reference itself produced (tests/golden, passed in as a text file: one case per line,
// "class first n setSize size setSizeMinimum setSizeMaximum size"; class 0 FFT, 1 RealFFT,
// 2 ModifiedRealFFT).  RealFFT returns the complex half size (reference :434-441).
template <class T>
static void setsize_case(size_t first, size_t n, const size_t *want, int cls) {
	T f(first);
	size_t got[5];
	got[0] = f.setSize(n);
	got[1] = f.size();
	got[2] = f.setSizeMinimum(n);
	got[3] = f.setSizeMaximum(n);
	got[4] = f.size();
	for (int k = 0; k < 5; ++k)
		CHECK(got[k] == want[k], "setSize returns: class %d first %zu n %zu item %d: %zu != %zu", cls, first, n, k,
		      got[k], want[k]);
}

static void setsize_returns(const char *path) {
	FILE *fp = std::fopen(path, "r");
	CHECK(fp != nullptr, "cannot open %s", path);
	if (!fp) return;
	int cls;
	size_t first, n, w[5];
	int cases = 0;
	while (std::fscanf(fp, "%d %zu %zu %zu %zu %zu %zu %zu", &cls, &first, &n, &w[0], &w[1], &w[2], &w[3], &w[4]) == 8) {
		if (cls == 0) setsize_case<signalsmith::FFT<double>>(first, n, w, cls);
		if (cls == 1) setsize_case<signalsmith::RealFFT<double>>(first, n, w, cls);
		if (cls == 2) setsize_case<signalsmith::ModifiedRealFFT<double>>(first, n, w, cls);
		++cases;
	}
	std::fclose(fp);
	CHECK(cases > 0, "no setSize cases read");
	// an unchanged size keeps the plans (reference FFT::setSize :357 is a no-op then)
	signalsmith::RealFFT<float> r(3840);
	signalsmith::FFT<float> c(1024);
	const size_t before = ssfft_plans_created();
	CHECK(r.setSize(3840) == 1920, "RealFFT setSize return");
	CHECK(c.setSize(1024) == 1024, "FFT setSize return");
	CHECK(ssfft_plans_created() == before, "unchanged setSize made %zu new plans", ssfft_plans_created() - before);
	r.setSize(3842);
	CHECK(ssfft_plans_created() == before + 1, "changed setSize must plan once");
}

static void device_overloads() {
	const size_t n = 1920, batch = 64;
	vector<complex<float>> h(n * batch), back(n * batch), one(n);
	for (auto &v : h) v = complex<float>((float)urand(), (float)urand());
	complex<float> *d_in = nullptr, *d_out = nullptr;
	CHECK(cudaMalloc(reinterpret_cast<void **>(&d_in), h.size() * sizeof(h[0])) == cudaSuccess, "cudaMalloc");
	CHECK(cudaMalloc(reinterpret_cast<void **>(&d_out), h.size() * sizeof(h[0])) == cudaSuccess, "cudaMalloc");
	cudaMemcpy(d_in, h.data(), h.size() * sizeof(h[0]), cudaMemcpyHostToDevice);
	signalsmith::FFT<float> fft(n);
	fft.fft(signalsmith::device(d_in), signalsmith::device(d_out), batch);
	cudaMemcpy(back.data(), d_out, back.size() * sizeof(h[0]), cudaMemcpyDeviceToHost);
	for (size_t b = 0; b < batch; b += 21) {
		vector<complex<float>> x(h.begin() + b * n, h.begin() + (b + 1) * n), y(n);
		fft.fft(x, y);  // host path of the same object
		vector<complex<float>> d(back.begin() + b * n, back.begin() + (b + 1) * n);
		CHECK(close_enough(d, y, 1e-6), "device vs host batch %zu", b);
	}
	signalsmith::RealFFT<float> real(3840);
	float *d_real = reinterpret_cast<float *>(d_in);
	real.fft(signalsmith::device(d_real), signalsmith::device(d_out), 8);
	real.ifft(signalsmith::device(d_out), signalsmith::device(d_real), 8);
	CHECK(cudaDeviceSynchronize() == cudaSuccess, "sync");
	cudaFree(d_in);
	cudaFree(d_out);
}

int main(int argc, char **argv) {
	if (argc > 1) setsize_returns(argv[1]);
	individual_bins<double>(1e-6);
	individual_bins<float>(1e-6);
	linearity<double>(1e-6);
	linearity<float>(1e-6);
	inverse<double>(1, 1e-6);
	inverse<double>(-1, 1e-6);
	inverse<float>(-1, 1e-6);
	sizes();
	real_vs_complex<false>();
	real_vs_complex<true>();
	device_overloads();
	bool thrown = false;
	try {
		signalsmith::FFT<double> bad(64);
		signalsmith::RealFFT<double> r(1);  // RealFFT of size 1 has no bins: no plan, no work
		vector<double> x(1);
		vector<complex<double>> y(1);
		r.fft(x, y);
	} catch (const signalsmith::FFTError &) {
		thrown = true;
	}
	CHECK(!thrown, "size-1 RealFFT should be a no-op");
	std::printf("%s (%d failures)\n", failures ? "FAILED" : "all drop-in checks passed", failures);
	return failures ? 1 : 0;
}

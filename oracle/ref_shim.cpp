// oracle/ref_shim.cpp -- C-ABI wrapper around the UNMODIFIED reference header (TEST
// INFRASTRUCTURE ONLY).
//
// Compiled by oracle/Makefile (target `ref`) with `-I <reference checkout>`, so the reference's
// own signalsmith-fft.h is included from where it lies; nothing of it is copied here.  The
// resulting oracle/_ref/libssref.so exports the same entry points as liboracle.so with a
// `ref_` prefix.  It pins the C restatement (tests/test_oracle.py) and generates
// tests/golden/ (tests/golden/make_golden.py).  It only exists where the reference checkout
// does; nothing on the GPU path needs it.
#include <complex>
#include <cstddef>
#include <thread>
#include <vector>

#include "signalsmith-fft.h"

namespace {

template <typename V>
int run_complex(size_t n, int inverse, const V *in, V *out) {
	if (n == 0) return -1;
	signalsmith::FFT<V> fft(n);
	auto *ci = reinterpret_cast<const std::complex<V> *>(in);
	auto *co = reinterpret_cast<std::complex<V> *>(out);
	if (inverse) fft.ifft(ci, co);
	else fft.fft(ci, co);
	return 0;
}

template <typename V, bool modified>
int run_real(size_t n, int inverse, const V *in, V *out) {
	if (n / 2 == 0) return -1;
	typename std::conditional<modified, signalsmith::ModifiedRealFFT<V>, signalsmith::RealFFT<V>>::type fft(n);
	if (inverse) fft.ifft(reinterpret_cast<const std::complex<V> *>(in), out);
	else fft.fft(in, reinterpret_cast<std::complex<V> *>(out));
	return 0;
}

template <typename V>
int run_real_any(size_t n, int modified, int inverse, const V *in, V *out) {
	return modified ? run_real<V, true>(n, inverse, in, out) : run_real<V, false>(n, inverse, in, out);
}

// One instance per thread over a contiguous slice of the batch (instances are not thread-safe).
template <typename V>
int run_batch(int real, int modified, int inverse, size_t n, size_t batch, const V *in, V *out, int nthreads,
              size_t repeats) {
	if (nthreads < 1) nthreads = 1;
	size_t h2 = 2 * (n / 2);
	size_t in_dist = real ? (inverse ? h2 : n) : 2 * n;
	size_t out_dist = real ? (inverse ? n : h2) : 2 * n;
	auto worker = [&](size_t b0, size_t b1) {
		if (real) {
			if (modified) {
				signalsmith::ModifiedRealFFT<V> f(n);
				for (size_t r = 0; r < repeats; ++r)
					for (size_t b = b0; b < b1; ++b) {
						if (inverse)
							f.ifft(reinterpret_cast<const std::complex<V> *>(in + b * in_dist), out + b * out_dist);
						else f.fft(in + b * in_dist, reinterpret_cast<std::complex<V> *>(out + b * out_dist));
					}
			} else {
				signalsmith::RealFFT<V> f(n);
				for (size_t r = 0; r < repeats; ++r)
					for (size_t b = b0; b < b1; ++b) {
						if (inverse)
							f.ifft(reinterpret_cast<const std::complex<V> *>(in + b * in_dist), out + b * out_dist);
						else f.fft(in + b * in_dist, reinterpret_cast<std::complex<V> *>(out + b * out_dist));
					}
			}
		} else {
			signalsmith::FFT<V> f(n);
			for (size_t r = 0; r < repeats; ++r)
				for (size_t b = b0; b < b1; ++b) {
					auto *ci = reinterpret_cast<const std::complex<V> *>(in + b * in_dist);
					auto *co = reinterpret_cast<std::complex<V> *>(out + b * out_dist);
					if (inverse) f.ifft(ci, co);
					else f.fft(ci, co);
				}
		}
	};
	std::vector<std::thread> threads;
	for (int t = 1; t < nthreads; ++t)
		threads.emplace_back(worker, batch * t / nthreads, batch * (t + 1) / nthreads);
	worker(0, batch / nthreads);
	for (auto &th : threads) th.join();
	return 0;
}

// Return values of the size-setting members on a fresh object of class `cls` (0 FFT<double>,
// 1 RealFFT<double>, 2 ModifiedRealFFT<double>) made with size `first`: out[0] = setSize(n),
// out[1] = size() after it, out[2] = setSizeMinimum(n), out[3] = setSizeMaximum(n),
// out[4] = size() after that.
template <class T>
void setsize_returns(size_t first, size_t n, size_t *out) {
	T f(first);
	out[0] = f.setSize(n);
	out[1] = f.size();
	out[2] = f.setSizeMinimum(n);
	out[3] = f.setSizeMaximum(n);
	out[4] = f.size();
}
}  // namespace

extern "C" {
int ref_fft_f64(size_t n, int inverse, const double *in, double *out) { return run_complex<double>(n, inverse, in, out); }
int ref_fft_f32(size_t n, int inverse, const float *in, float *out) { return run_complex<float>(n, inverse, in, out); }
int ref_rfft_f64(size_t n, int modified, int inverse, const double *in, double *out) {
	return run_real_any<double>(n, modified, inverse, in, out);
}
int ref_rfft_f32(size_t n, int modified, int inverse, const float *in, float *out) {
	return run_real_any<float>(n, modified, inverse, in, out);
}
int ref_batch_f64(int real, int modified, int inverse, size_t n, size_t batch, const double *in, double *out,
                  int nthreads, size_t repeats) {
	return run_batch<double>(real, modified, inverse, n, batch, in, out, nthreads, repeats);
}
int ref_batch_f32(int real, int modified, int inverse, size_t n, size_t batch, const float *in, float *out,
                  int nthreads, size_t repeats) {
	return run_batch<float>(real, modified, inverse, n, batch, in, out, nthreads, repeats);
}
int ref_setsize_returns(int cls, size_t first, size_t n, size_t *out) {
	switch (cls) {
	case 0: setsize_returns<signalsmith::FFT<double>>(first, n, out); return 0;
	case 1: setsize_returns<signalsmith::RealFFT<double>>(first, n, out); return 0;
	case 2: setsize_returns<signalsmith::ModifiedRealFFT<double>>(first, n, out); return 0;
	}
	return -1;
}
size_t ref_size_minimum(size_t n) { return signalsmith::FFT<double>::sizeMinimum(n); }
size_t ref_size_maximum(size_t n) { return signalsmith::FFT<double>::sizeMaximum(n); }
size_t ref_real_size_minimum(size_t n) { return signalsmith::RealFFT<double>::sizeMinimum(n); }
size_t ref_real_size_maximum(size_t n) { return signalsmith::RealFFT<double>::sizeMaximum(n); }
}

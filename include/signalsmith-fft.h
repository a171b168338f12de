// signalsmith-fft.h -- drop-in GB300 replacement for the Signalsmith FFT header (v5 API).
//
// Same names, template parameters and behaviour as the reference header signalsmith-fft.h:
//   signalsmith::FFT<V>                     (reference :69-387)
//   signalsmith::RealFFT<V, optionFlags>    (reference :393-503)
//   signalsmith::FFTOptions::halfFreqShift  (reference :389-391)
//   signalsmith::ModifiedRealFFT<V>         (reference :505-508)
// with setSize / setSizeMinimum / setSizeMaximum / size / static sizeMinimum / sizeMaximum, and
// fft / ifft that accept any container or random-access iterator of std::complex<V> (reals for
// RealFFT), out of place, unnormalised, real spectra with {DC, Nyquist} packed into bin 0.
// The namespace is SIGNALSMITH_FFT_NAMESPACE (default `signalsmith`) and the include guard is
// the reference's, so this header is included instead of it, not beside it.
//
// The transforms run on the current CUDA device through libssfft.so's C ABI (ssfft.h), for
// V = float or double.  Extensions over the reference:
//   * device-pointer overloads: fft(signalsmith::device(d_in), signalsmith::device(d_out)
//     [, batch [, stream]]) run asynchronously on device memory, `batch` contiguous transforms;
//   * errors (no GPU, out of memory, unsupported size) throw signalsmith::FFTError instead of
//     the reference's undefined behaviour.
// Host-iterator calls are synchronous: input gathered into a host buffer, transformed by
// ssfft_exec_host (copies overlapped with compute), output scattered back.  Like the reference,
// one instance must not be used from two threads at once.
#ifndef SIGNALSMITH_FFT_V5
#define SIGNALSMITH_FFT_V5
#ifndef SIGNALSMITH_FFT_NAMESPACE
#define SIGNALSMITH_FFT_NAMESPACE signalsmith
#endif

#include <complex>
#include <cstddef>
#include <iterator>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "ssfft.h"

namespace SIGNALSMITH_FFT_NAMESPACE {

struct FFTError : std::runtime_error {
	ssfft_status status;
	FFTError(ssfft_status s, const std::string &what)
	    : std::runtime_error(what + ": " + ssfft_status_string(s) +
	                         (s == SSFFT_ERR_CUDA ? std::string(" (") + ssfft_last_cuda_error() + ")" : std::string())),
	      status(s) {}
};

// Tag for device memory: fft(device(d_in), device(d_out)).
template <typename T>
struct DevicePointer {
	T *ptr;
};
template <typename T>
DevicePointer<T> device(T *p) {
	return DevicePointer<T>{p};
}

namespace gpu_detail {

inline void check(ssfft_status s, const char *what) {
	if (s != SSFFT_SUCCESS) throw FFTError(s, what);
}

template <typename V>
struct DType;
template <>
struct DType<float> {
	static constexpr ssfft_dtype value = SSFFT_F32;
};
template <>
struct DType<double> {
	static constexpr ssfft_dtype value = SSFFT_F64;
};

// A container yields std::begin(c); anything else is taken as an iterator already (the
// reference's GetIterator, signalsmith-fft.h:55-67, has the same contract).
template <typename T, typename = void>
struct IterOf {
	static T get(T t) { return t; }
};
template <typename T>
struct IterOf<T, decltype((void)std::begin(std::declval<T &>()))> {
	static auto get(T &t) -> decltype(std::begin(t)) { return std::begin(t); }
};
template <typename T>
auto iter(T &&t) -> decltype(IterOf<typename std::remove_reference<T>::type>::get(t)) {
	return IterOf<typename std::remove_reference<T>::type>::get(t);
}

// Owning handle of one ssfft plan, re-created when the size, kind or batch changes.
class PlanHandle {
	ssfft_plan_t plan_ = nullptr;
	size_t n_ = 0, batch_ = 0;
	ssfft_kind kind_ = SSFFT_COMPLEX;
	ssfft_dtype dtype_ = SSFFT_F32;

public:
	PlanHandle() = default;
	PlanHandle(const PlanHandle &) = delete;
	PlanHandle &operator=(const PlanHandle &) = delete;
	~PlanHandle() { reset(); }
	void reset() {
		if (plan_) ssfft_plan_destroy(plan_);
		plan_ = nullptr;
		n_ = batch_ = 0;
	}
	ssfft_plan_t get(size_t n, ssfft_dtype dt, ssfft_kind kind, size_t batch) {
		if (plan_ && n == n_ && dt == dtype_ && kind == kind_ && batch <= batch_) return plan_;
		reset();
		check(ssfft_plan_create(&plan_, n, dt, kind, batch), "ssfft_plan_create");
		n_ = n;
		dtype_ = dt;
		kind_ = kind;
		batch_ = batch;
		return plan_;
	}
};

}  // namespace gpu_detail

template <typename V>
class FFT {
	static_assert(std::is_same<V, float>::value || std::is_same<V, double>::value,
	              "the GB300 FFT runs in float or double");
	using complex = std::complex<V>;
	size_t _size = 0;
	gpu_detail::PlanHandle host_plan, device_plan;
	std::vector<complex> stage_in, stage_out;

	template <bool inverse, typename In, typename Out>
	void run_host(In &&input, Out &&output) {
		if (_size == 0) return;
		auto in = gpu_detail::iter(input);
		auto out = gpu_detail::iter(output);
		for (size_t i = 0; i < _size; ++i) stage_in[i] = in[i];
		ssfft_plan_t p = host_plan.get(_size, gpu_detail::DType<V>::value, SSFFT_COMPLEX, 1);
		gpu_detail::check(ssfft_exec_host(p, inverse ? 1 : 0, stage_in.data(), stage_out.data()), "ssfft_exec_host");
		for (size_t i = 0; i < _size; ++i) out[i] = stage_out[i];
	}

public:
	static size_t sizeMinimum(size_t size) { return ssfft_size_minimum(size); }
	static size_t sizeMaximum(size_t size) { return ssfft_size_maximum(size); }
	// Extension (opt-in, new names): nearest 2^a 3^b 5^c sizes, which the reference's helpers
	// never pick but which run as fast here.
	static size_t sizeMinimumSmooth(size_t size) { return ssfft_size_minimum_smooth(size); }
	static size_t sizeMaximumSmooth(size_t size) { return ssfft_size_maximum_smooth(size); }

	FFT(size_t size, int fastDirection = 0) {
		if (fastDirection > 0) size = sizeMinimum(size);
		if (fastDirection < 0) size = sizeMaximum(size);
		setSize(size);
	}

	size_t setSize(size_t size) {
		if (size != _size) {
			_size = size;
			stage_in.assign(size, complex());
			stage_out.assign(size, complex());
			host_plan.reset();
			device_plan.reset();
			if (size) host_plan.get(size, gpu_detail::DType<V>::value, SSFFT_COMPLEX, 1);
		}
		return _size;
	}
	size_t setSizeMinimum(size_t size) { return setSize(sizeMinimum(size)); }
	size_t setSizeMaximum(size_t size) { return setSize(sizeMaximum(size)); }
	const size_t &size() const { return _size; }

	template <typename InputIterator, typename OutputIterator>
	void fft(InputIterator &&input, OutputIterator &&output) {
		run_host<false>(std::forward<InputIterator>(input), std::forward<OutputIterator>(output));
	}
	template <typename InputIterator, typename OutputIterator>
	void ifft(InputIterator &&input, OutputIterator &&output) {
		run_host<true>(std::forward<InputIterator>(input), std::forward<OutputIterator>(output));
	}

	// Device memory: `batch` transforms stored back to back, asynchronous on `stream`.
	void fft(DevicePointer<const complex> input, DevicePointer<complex> output, size_t batch = 1,
	         void *stream = nullptr) {
		run_device(false, input.ptr, output.ptr, batch, stream);
	}
	void ifft(DevicePointer<const complex> input, DevicePointer<complex> output, size_t batch = 1,
	          void *stream = nullptr) {
		run_device(true, input.ptr, output.ptr, batch, stream);
	}
	void fft(DevicePointer<complex> input, DevicePointer<complex> output, size_t batch = 1, void *stream = nullptr) {
		run_device(false, input.ptr, output.ptr, batch, stream);
	}
	void ifft(DevicePointer<complex> input, DevicePointer<complex> output, size_t batch = 1, void *stream = nullptr) {
		run_device(true, input.ptr, output.ptr, batch, stream);
	}

private:
	void run_device(bool inverse, const complex *in, complex *out, size_t batch, void *stream) {
		if (_size == 0 || batch == 0) return;
		ssfft_plan_t p = device_plan.get(_size, gpu_detail::DType<V>::value, SSFFT_COMPLEX, batch);
		gpu_detail::check(ssfft_exec_batch(p, inverse ? 1 : 0, in, out, batch, stream), "ssfft_exec_batch");
	}
};

struct FFTOptions {
	static constexpr int halfFreqShift = 1;
};

template <typename V, int optionFlags = 0>
class RealFFT {
	static_assert(std::is_same<V, float>::value || std::is_same<V, double>::value,
	              "the GB300 FFT runs in float or double");
	static constexpr bool modified = (optionFlags & FFTOptions::halfFreqShift) != 0;
	static constexpr ssfft_kind kind = modified ? SSFFT_REAL_HALFSHIFT : SSFFT_REAL;
	using complex = std::complex<V>;
	size_t _n = 0;  // real length the plan was made for
	gpu_detail::PlanHandle host_plan, device_plan;
	std::vector<V> stage_real;
	std::vector<complex> stage_bins;

public:
	// RealFFT::sizeMinimum / sizeMaximum (reference :403-408), quirks included.
	static size_t sizeMinimum(size_t size) { return ssfft_real_size_minimum(size); }
	static size_t sizeMaximum(size_t size) { return ssfft_real_size_maximum(size); }
	// Extension (opt-in, new names): nearest even sizes whose half is 2^a 3^b 5^c.
	static size_t sizeMinimumSmooth(size_t size) { return ssfft_real_size_minimum_smooth(size); }
	static size_t sizeMaximumSmooth(size_t size) { return ssfft_real_size_maximum_smooth(size); }

	RealFFT(size_t size, int fastDirection = 0) {
		if (fastDirection > 0) size = sizeMinimum(size);
		if (fastDirection < 0) size = sizeMaximum(size);
		setSize(size);
	}

	// Returns the size of the complex transform inside, size/2, as the reference does
	// (`return complexFft.setSize(size/2)`, :434); setSizeMinimum / setSizeMaximum return the
	// same (:436-441).  An unchanged size keeps the plans (the reference's FFT::setSize is a no-op
	// then, :357); the real length itself is the key, because the split twiddles depend on it
	// (:420-425), so 6 and 7 are different plans with the same half size.
	size_t setSize(size_t size) {
		if (size != _n) {
			_n = size;
			stage_real.assign(size, V());
			stage_bins.assign(size / 2, complex());
			host_plan.reset();
			device_plan.reset();
			if (size / 2) host_plan.get(size, gpu_detail::DType<V>::value, kind, 1);
		}
		return _n / 2;
	}
	size_t setSizeMinimum(size_t size) { return setSize(sizeMinimum(size)); }
	size_t setSizeMaximum(size_t size) { return setSize(sizeMaximum(size)); }
	size_t size() const { return 2 * (_n / 2); }

	// n reals in, n/2 complex bins out (bin 0 = {DC, Nyquist} unless half-shifted).
	template <typename InputIterator, typename OutputIterator>
	void fft(InputIterator &&input, OutputIterator &&output) {
		if (_n / 2 == 0) return;
		auto in = gpu_detail::iter(input);
		auto out = gpu_detail::iter(output);
		for (size_t i = 0; i < _n; ++i) stage_real[i] = in[i];
		ssfft_plan_t p = host_plan.get(_n, gpu_detail::DType<V>::value, kind, 1);
		gpu_detail::check(ssfft_exec_host(p, 0, stage_real.data(), stage_bins.data()), "ssfft_exec_host");
		for (size_t i = 0; i < _n / 2; ++i) out[i] = stage_bins[i];
	}
	// n/2 bins in, 2*(n/2) reals out, scaled by n (unnormalised).
	template <typename InputIterator, typename OutputIterator>
	void ifft(InputIterator &&input, OutputIterator &&output) {
		if (_n / 2 == 0) return;
		auto in = gpu_detail::iter(input);
		auto out = gpu_detail::iter(output);
		for (size_t i = 0; i < _n / 2; ++i) stage_bins[i] = in[i];
		ssfft_plan_t p = host_plan.get(_n, gpu_detail::DType<V>::value, kind, 1);
		gpu_detail::check(ssfft_exec_host(p, 1, stage_bins.data(), stage_real.data()), "ssfft_exec_host");
		for (size_t i = 0; i < 2 * (_n / 2); ++i) out[i] = stage_real[i];
	}

	// Device memory: `batch` frames back to back (n reals / n/2 bins each), asynchronous.
	void fft(DevicePointer<const V> input, DevicePointer<complex> output, size_t batch = 1, void *stream = nullptr) {
		run_device(false, input.ptr, output.ptr, batch, stream);
	}
	void fft(DevicePointer<V> input, DevicePointer<complex> output, size_t batch = 1, void *stream = nullptr) {
		run_device(false, input.ptr, output.ptr, batch, stream);
	}
	void ifft(DevicePointer<const complex> input, DevicePointer<V> output, size_t batch = 1, void *stream = nullptr) {
		run_device(true, input.ptr, output.ptr, batch, stream);
	}
	void ifft(DevicePointer<complex> input, DevicePointer<V> output, size_t batch = 1, void *stream = nullptr) {
		run_device(true, input.ptr, output.ptr, batch, stream);
	}

private:
	void run_device(bool inverse, const void *in, void *out, size_t batch, void *stream) {
		if (_n / 2 == 0 || batch == 0) return;
		ssfft_plan_t p = device_plan.get(_n, gpu_detail::DType<V>::value, kind, batch);
		gpu_detail::check(ssfft_exec_batch(p, inverse ? 1 : 0, in, out, batch, stream), "ssfft_exec_batch");
	}
};

template <typename V>
struct ModifiedRealFFT : public RealFFT<V, FFTOptions::halfFreqShift> {
	using RealFFT<V, FFTOptions::halfFreqShift>::RealFFT;
};

}  // namespace SIGNALSMITH_FFT_NAMESPACE

#undef SIGNALSMITH_FFT_NAMESPACE
#endif  // SIGNALSMITH_FFT_V5

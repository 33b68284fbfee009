// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// Compiles the reference's OWN CPU primitives (header-only C++20, included
// read-only from REF_DIR/src) into oracle/_ref/libugsdr_ref.so and exposes them
// through a flat C interface for the golden-vector generator
// (tests/golden/make_golden.py) and for cross-checking oracle/oracle.cpp.
// Nothing here is shipped or called by the product path.
//
// The reference does not build as shipped without Intel IPP (its FSE and
// Tracker need IPP-only overloads), so the acquisition loop below is a
// ~60-line restatement of FastSearchEngineBase::ProcessBpsk
// (src/acquisition/fse.hpp:242-276) that calls the reference's policies:
//   TableMixer::Translate            src/mixer/table_mixer.hpp:78-101
//   SequentialDft (r2c) + Conj       src/matched_filter/matched_filter.hpp:49-54
//   SequentialMatchedFilter          src/matched_filter/matched_filter.hpp:56-61
//   SequentialAbs / ReshapeAndSum    src/math/abs.hpp:24-32, reshape_and_sum.hpp:37-52
//   SequentialMaxIndex / MeanStdDev  src/math/max_index.hpp:31-42, mean_stddev.hpp:29-42
// FFTW itself is absent; oracle/shims/fftw3.h supplies its API (see there).
#include "prn_codes/codegen_wrapper.hpp"
#include "common.hpp"
#include "correlator/correlator.hpp"
#include "math/abs.hpp"
#include "math/conj.hpp"
#include "math/dft.hpp"
#include "math/max_index.hpp"
#include "math/mean_stddev.hpp"
#include "math/reshape_and_sum.hpp"
#include "matched_filter/matched_filter.hpp"
#include "mixer/table_mixer.hpp"
#include "resample/resampler.hpp"
#include "resample/upsampler.hpp"
#include "helpers/NtlabPackedSpan.hpp"
#include "antijamming/jse.hpp"
#include "math/stft.hpp"
#include "signal_parameters.hpp"

#include <complex>
#include <cstdint>
#include <cstring>
#include <span>
#include <utility>
#include <vector>

namespace {
	using ugsdr::Signal;

	template <Signal s>
	int CodeOf(int sv, float* out, int cap) {
		const auto& code = ugsdr::PrnGenerator<s>::template Get<float>(static_cast<std::size_t>(sv));
		const int len = static_cast<int>(code.size());
		if (out && cap >= len)
			std::memcpy(out, code.data(), sizeof(float) * code.size());
		return len;
	}

	template <typename T>
	std::vector<std::complex<T>> ToComplex(const T* p, std::size_t n) {
		std::vector<std::complex<T>> v(n);
		std::memcpy(v.data(), p, sizeof(T) * 2 * n);
		return v;
	}

	template <typename T>
	void FromComplex(const std::vector<std::complex<T>>& v, T* p) {
		std::memcpy(p, v.data(), sizeof(T) * 2 * v.size());
	}

	template <typename T>
	struct Peak {
		double level, sigma, code_offset, doppler;
		std::int64_t index;
		std::int64_t doppler_bin;
	};

	// ProcessBpsk (fse.hpp:242-276) generalised to K consecutive coherent blocks
	// of N samples each, the per-block GetOneMsPeak outputs (fse.hpp:201-220)
	// summed non-coherently; K = 1 is the reference loop as written.
	template <typename T>
	void Acquire(const T* signal_iq, std::size_t n_total, std::size_t n, std::size_t k_blocks,
		const T* code, double fs, double range, double step, double if_freq, double ratio,
		int reshape, int coherent, T* out_peak /*7 doubles packed as T? no: see below*/,
		double* rec, T* best_output) {
		using C = std::complex<T>;
		auto signal = ToComplex(signal_iq, n_total);
		std::vector<T> code_vec(code, code + n);
		// PrepareCodeSpectrum body (matched_filter.hpp:49-54): the templated
		// entry point rejects std::vector<float> (its Container constraint),
		// so the two calls it makes are issued directly.
		auto code_spectrum = ugsdr::SequentialDft::Transform(std::as_const(code_vec));
		ugsdr::SequentialConj::Transform(code_spectrum);

		const auto samples_per_ms = static_cast<std::size_t>(fs / 1e3);
		double best_level = 0.0, best_sigma = 1.0, best_code = 0.0, best_doppler = 0.0;
		std::int64_t best_index = 0, best_bin = -1, bin = 0;
		bool have = false;
		for (double doppler = -range; doppler <= range; doppler += step, ++bin) {
			// Mixer<TableMixer>::Translate(const T&) does not compile (no const
			// Process overload), so mix a copy in place: same arithmetic.
			auto translated = signal;
			ugsdr::TableMixer::Translate(translated, fs, -doppler);
			std::vector<T> acc;
			for (std::size_t b = 0; b < k_blocks; ++b) {
				std::vector<C> block(translated.begin() + b * n, translated.begin() + (b + 1) * n);
				ugsdr::SequentialMatchedFilter::FilterOptimized(block, code_spectrum);
				std::vector<T> one_ms;
				if (!reshape)
					one_ms = ugsdr::SequentialAbs::Transform(block);
				else if (coherent)
					one_ms = ugsdr::SequentialReshapeAndSum::Transform(ugsdr::SequentialAbs::Transform(block), samples_per_ms);
				else
					one_ms = ugsdr::SequentialAbs::Transform(ugsdr::SequentialReshapeAndSum::Transform(std::as_const(block), samples_per_ms));
				if (acc.empty())
					acc = std::move(one_ms);
				else
					for (std::size_t i = 0; i < acc.size(); ++i)
						acc[i] += one_ms[i];
			}
			auto mi = ugsdr::SequentialMaxIndex::Transform(acc);
			auto ms = ugsdr::SequentialMeanStdDev::Calculate(acc);
			const double level = mi.value;
			const double sigma = ms.sigma + ms.mean;
			// AcquisitionResult::operator<=> compares level only; `max_result < tmp`
			if (!have || best_level < level) {
				have = true;
				best_level = level;
				best_sigma = sigma;
				best_code = ratio * static_cast<double>(mi.index);
				best_doppler = doppler + if_freq;
				best_index = static_cast<std::int64_t>(mi.index);
				best_bin = bin;
				if (best_output)
					std::memcpy(best_output, acc.data(), sizeof(T) * acc.size());
			}
		}
		rec[0] = best_level;
		rec[1] = best_sigma;
		rec[2] = best_code;
		rec[3] = best_doppler;
		rec[4] = static_cast<double>(best_index);
		rec[5] = static_cast<double>(best_bin);
		rec[6] = best_level / best_sigma;
		(void)out_peak;
	}
}

extern "C" {

int ref_prn_code(int signal, int sv, float* out, int cap) {
	switch (static_cast<Signal>(signal)) {
	case Signal::GpsCoarseAcquisition_L1: return CodeOf<Signal::GpsCoarseAcquisition_L1>(sv, out, cap);
	case Signal::Gps_L5I: return CodeOf<Signal::Gps_L5I>(sv, out, cap);
	case Signal::Gps_L5Q: return CodeOf<Signal::Gps_L5Q>(sv, out, cap);
	case Signal::GlonassCivilFdma_L1: return CodeOf<Signal::GlonassCivilFdma_L1>(sv, out, cap);
	case Signal::Galileo_E1b: return CodeOf<Signal::Galileo_E1b>(sv, out, cap);
	case Signal::Galileo_E1c: return CodeOf<Signal::Galileo_E1c>(sv, out, cap);
	case Signal::SbasCoarseAcquisition_L1: return CodeOf<Signal::SbasCoarseAcquisition_L1>(sv, out, cap);
	case Signal::QzssCoarseAcquisition_L1: return CodeOf<Signal::QzssCoarseAcquisition_L1>(sv, out, cap);
	case Signal::BeiDou_B1I: return CodeOf<Signal::BeiDou_B1I>(sv, out, cap);
	case Signal::NavIC_L5: return CodeOf<Signal::NavIC_L5>(sv, out, cap);
	default: return -1;
	}
}

// RepeatCodeNTimes (common.hpp:78-85) then SequentialUpsampler (upsampler.hpp:30-37)
void ref_repeat_upsample(const float* code, int len, int repeats, float* out, std::size_t samples) {
	std::vector<float> v(code, code + len);
	auto up = ugsdr::SequentialUpsampler::Transform(ugsdr::RepeatCodeNTimes(v, static_cast<std::size_t>(repeats)), samples);
	std::memcpy(out, up.data(), sizeof(float) * samples);
}

// Mixer<TableMixer>::Translate(T&, fs, f, phase) in place (mixer.hpp:33-42)
void ref_table_mixer_f32(float* iq, std::size_t n, double fs, double f, double phase) {
	auto v = ToComplex(iq, n);
	ugsdr::TableMixer::Translate(v, fs, f, phase);
	FromComplex(v, iq);
}
void ref_table_mixer_f64(double* iq, std::size_t n, double fs, double f, double phase) {
	auto v = ToComplex(iq, n);
	ugsdr::TableMixer::Translate(v, fs, f, phase);
	FromComplex(v, iq);
}

// SequentialDft::Transform(const complex vector, inverse) (dft.hpp:114-135, 217-220)
void ref_dft_c2c_f32(const float* in, float* out, std::size_t n, int inverse) {
	const auto v = ToComplex(in, n);
	auto r = ugsdr::SequentialDft::Transform(v, inverse != 0);
	FromComplex(r, out);
}
// SequentialDft::Transform(const real vector) r2c (dft.hpp:222-225)
void ref_dft_r2c_f32(const float* in, float* out, std::size_t n) {
	const std::vector<float> v(in, in + n);
	auto r = ugsdr::SequentialDft::Transform(v);
	FromComplex(r, out);
}
// code spectrum = conj(r2c(code)) (matched_filter.hpp:49-54)
void ref_prepare_code_spectrum_f32(const float* code, std::size_t n, float* out) {
	const std::vector<float> v(code, code + n);
	auto spec = ugsdr::SequentialDft::Transform(v);
	ugsdr::SequentialConj::Transform(spec);
	FromComplex(spec, out);
}
void ref_filter_optimized_f32(float* iq, std::size_t n, const float* spectrum) {
	auto v = ToComplex(iq, n);
	const auto s = ToComplex(spectrum, n);
	ugsdr::SequentialMatchedFilter::FilterOptimized(v, s);
	FromComplex(v, iq);
}
void ref_abs_f32(const float* iq, std::size_t n, float* out) {
	const auto v = ToComplex(iq, n);
	auto r = ugsdr::SequentialAbs::Transform(v);
	std::memcpy(out, r.data(), sizeof(float) * n);
}
int ref_reshape_sum_f32(const float* in, std::size_t n, std::size_t block, float* out) {
	try {
		const std::vector<float> v(in, in + n);
		auto r = ugsdr::SequentialReshapeAndSum::Transform(v, block);
		std::memcpy(out, r.data(), sizeof(float) * r.size());
		return 0;
	}
	catch (...) {
		return -1;
	}
}
void ref_max_index_f32(const float* in, std::size_t n, float* value, std::size_t* index) {
	const std::vector<float> v(in, in + n);
	auto r = ugsdr::SequentialMaxIndex::Transform(v);
	*value = r.value;
	*index = r.index;
}
void ref_mean_std_f32(const float* in, std::size_t n, float* mean, float* sigma) {
	const std::vector<float> v(in, in + n);
	auto r = ugsdr::SequentialMeanStdDev::Calculate(v);
	*mean = r.mean;
	*sigma = r.sigma;
}
// FindPreambleGps / FindPreambleGlonass's filter (measurements/observable.hpp:
// 206-215, 263-272) through the reference's own primitives: the navigation
// symbols sign(prompt I) as complex, the preamble symbols (restated from
// observable.hpp:92-94, 143-146: Observable does not compile without IPP)
// upsampled by SequentialUpsampler and resized to the prompt's length,
// SequentialMatchedFilter::Filter, SequentialAbs.  out: n magnitudes.
void ref_preamble_filter_f32(const float* prompt_i, std::size_t n, int message, float* out) {
	static const float gps[8] = {1, -1, -1, -1, 1, -1, 1, 1};
	static const float glo[40] = {-1, -1, -1, -1, -1, 1, 1, 1, -1, -1, 1, -1, -1, -1, 1, -1, 1, -1, 1, 1,
		1, 1, -1, 1, 1, -1, 1, -1, -1, 1, 1, -1, 1, -1, 1, -1, 1, -1, -1, 1};
	const float* sym = message == 1 ? glo : gps;
	const std::size_t n_sym = message == 1 ? 40 : 8, up = message == 1 ? 10 : 20;
	std::vector<std::complex<float>> preamble(sym, sym + n_sym);
	ugsdr::SequentialUpsampler::Transform(preamble, preamble.size() * up);
	preamble.resize(n);
	std::vector<std::complex<float>> bits(n);
	for (std::size_t i = 0; i < n; ++i)
		bits[i] = prompt_i[i] > 0 ? 1.f : -1.f;
	const auto filtered = ugsdr::SequentialMatchedFilter::Filter(std::as_const(bits), preamble);
	const auto y = ugsdr::SequentialAbs::Transform(filtered);
	std::memcpy(out, y.data(), sizeof(float) * n);
}
// SequentialResampler (resampler.hpp:39-46) on complex samples; returns output length
std::size_t ref_resample_c32(const float* iq, std::size_t n, float* out, std::size_t cap, std::size_t new_fs, std::size_t old_fs) {
	auto v = ToComplex(iq, n);
	ugsdr::SequentialResampler::Transform(v, new_fs, old_fs);
	if (out && cap >= v.size())
		FromComplex(v, out);
	return v.size();
}
// SequentialCorrelator (correlator.hpp:27-34)
void ref_correlate_f32(const float* iq, const float* code, std::size_t n, float* out) {
	const auto sig = ToComplex(iq, n);
	const std::vector<float> c(code, code + n);
	auto r = ugsdr::SequentialCorrelator::Correlate(std::span(sig), std::span(c));
	out[0] = r.real();
	out[1] = r.imag();
}

// rec: level, sigma(=std+mean), code_offset, doppler(+IF), index, doppler_bin, snr
void ref_acquire_f32(const float* iq, std::size_t n_total, std::size_t n, std::size_t k_blocks, const float* code,
	double fs, double range, double step, double if_freq, double ratio, int reshape, int coherent,
	double* rec, float* best_output) {
	Acquire<float>(iq, n_total, n, k_blocks, code, fs, range, step, if_freq, ratio, reshape, coherent, nullptr, rec, best_output);
}
void ref_acquire_f64(const double* iq, std::size_t n_total, std::size_t n, std::size_t k_blocks, const double* code,
	double fs, double range, double step, double if_freq, double ratio, int reshape, int coherent,
	double* rec, double* best_output) {
	Acquire<double>(iq, n_total, n, k_blocks, code, fs, range, step, if_freq, ratio, reshape, coherent, nullptr, rec, best_output);
}


// Packed front-end formats (golden vectors for the GPU decoders).
// BbpDdc file through the reference's own reader: SignalParametersBase::
// GetSeveralMs (signal_parameters.hpp:262-273) -> OpenFile's epoch framing
// (78-85), VerifyHeaders (48-57) and PackedSpan (helpers/BbpPackedSpan.hpp).
// Returns the number of decoded samples (ms * fs / 1e3) or -1 on error.
long ref_bbp_read(const char* path, double central, double fs, std::size_t ms, float* out_iq) {
	try {
		auto sp = ugsdr::SignalParametersBase<float>(path, ugsdr::FileType::BbpDdc, central, fs);
		// PackedSpan::Iterator::operator- (helpers/BbpPackedSpan.hpp:63-67) is
		// off by one, so the reader's std::copy (signal_parameters.hpp:244)
		// stops two samples past each epoch: harmless between epochs (the next
		// one overwrites them), past the end of the last one.  The slack here
		// keeps those two writes inside this vector.
		const std::size_t n = ms * static_cast<std::size_t>(fs / 1e3);
		std::vector<std::complex<float>> v(n + 64);
		sp.GetSeveralMs(0, ms, v);
		std::memcpy(out_iq, v.data(), n * sizeof(std::complex<float>));
		return static_cast<long>(n);
	}
	catch (...) {
		return -1;
	}
}

// NT1065 grabber bytes through NtlabPackedSpan<offset> (helpers/NtlabPackedSpan.hpp),
// channel 0..3 = First..Fourth (bit offsets 6, 4, 2, 0).
void ref_nt1065_decode(const unsigned char* bytes, std::size_t n, int channel, float* out_iq) {
	auto* dst = reinterpret_cast<std::complex<float>*>(out_iq);
	const auto* src = reinterpret_cast<const std::byte*>(bytes);
	switch (channel) {
	case 0: { auto s = ugsdr::NtlabPackedSpan<6, float>(src, n); std::copy(s.begin(), s.end(), dst); break; }
	case 1: { auto s = ugsdr::NtlabPackedSpan<4, float>(src, n); std::copy(s.begin(), s.end(), dst); break; }
	case 2: { auto s = ugsdr::NtlabPackedSpan<2, float>(src, n); std::copy(s.begin(), s.end(), dst); break; }
	default: { auto s = ugsdr::NtlabPackedSpan<0, float>(src, n); std::copy(s.begin(), s.end(), dst); break; }
	}
}

// ShortTimeFourierTransform<SequentialStft>::Transform(src) with the default
// 128-sample window and 96-sample overlap (math/stft.hpp:19-21, 42-61):
// returns the column count; columns are written when cap allows.
long ref_stft_f32(const float* iq, std::size_t n, float* out, std::size_t cap_columns) {
	const auto v = ToComplex(iq, n);
	const auto cols = ugsdr::ShortTimeFourierTransform<ugsdr::SequentialStft>::Transform(v);
	if (out && cols.size() <= cap_columns)
		for (std::size_t i = 0; i < cols.size(); ++i)
			std::memcpy(out + 2 * i * cols[i].size(), cols[i].data(), sizeof(float) * 2 * cols[i].size());
	return static_cast<long>(cols.size());
}

// the container-of-containers overload: OverlapAndAdd (math/stft.hpp:63-75)
void ref_istft_f32(const float* cols_iq, std::size_t n_columns, float* out) {
	std::vector<std::vector<std::complex<float>>> cols(n_columns);
	for (std::size_t i = 0; i < n_columns; ++i)
		cols[i] = ToComplex(cols_iq + 2 * i * 128, 128);
	const auto r = ugsdr::ShortTimeFourierTransform<ugsdr::SequentialStft>::Transform(cols);
	FromComplex(r, out);
}

// JammingSuppressionEngine<complex<float>>(fs).Process(src_dst) in place
// (antijamming/jse.hpp:89-102); the detections (jamming_detection.hpp:29-48)
// go out as type / bin / frequency / J/N; returns their count.
int ref_jamming_process_f32(float* iq, std::size_t n, double fs, int* types, long* bins, double* freqs, double* jn,
	int cap) {
	auto v = ToComplex(iq, n);
	ugsdr::JammingSuppressionEngine<std::complex<float>> engine(fs);
	engine.Process(v);
	FromComplex(v, iq);
	const auto& det = engine.GetDetectionResults();
	const int count = static_cast<int>(det.size());
	for (int i = 0; i < count && i < cap; ++i) {
		types[i] = static_cast<int>(det[i].interference_type);
		bins[i] = static_cast<long>(det[i].frequency_bin);
		freqs[i] = det[i].frequency;
		jn[i] = det[i].jammer_to_noise;
	}
	return count;
}
}

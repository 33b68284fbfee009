// ORACLE — CPU restatement of the ugsdr acquisition-and-correlation path.
// TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
// the checker, and by bench.py's cpu_baseline / --impl reference arm.  The
// product library (ugsdr_gb300/csrc) never links or calls it.
//
// Parity is pinned: tests/test_oracle.py checks every function here against
// golden vectors produced by the reference's own primitives
// (oracle/ref_harness.cpp compiled from the reference sources into
// oracle/_ref/, fixtures in tests/golden/).
//
// Each function is instantiated for float (the reference's CPU path runs in
// float: FseConfig with UnderlyingType = float) and double (the FP64 oracle
// the magnitude tolerances are stated against).  FFTs are the project DFT in
// oracle/fft64.hpp, computed in double and rounded to T, with FFTW's
// conventions as the reference's SequentialDft uses them.
#include "fft64.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <type_traits>
#include <vector>

namespace oracle {
	namespace {
		constexpr double kPi = 3.14159265358979323846;  // == std::numbers::pi

		// Fft64 plans cached per (size, sign): the reference plans per call with
		// FFTW_ESTIMATE (math/dft.hpp:117-120); the cache only removes the
		// twiddle-table rebuild, the transform arithmetic is unchanged.
		std::mutex plan_mutex;
		std::map<std::pair<std::size_t, int>, std::shared_ptr<Fft64>> plans;

		std::shared_ptr<Fft64> Plan(std::size_t n, int sign) {
			std::lock_guard<std::mutex> lock(plan_mutex);
			auto& slot = plans[{n, sign}];
			if (!slot)
				slot = std::make_shared<Fft64>(n, sign);
			return slot;
		}

		// Fft64 keeps per-call state only on the stack, so one plan serves all threads.
		void Transform(const cd* in, cd* out, std::size_t n, int sign) {
			Plan(n, sign)->Execute(in, out);
		}

		// The CPU baseline's float transform (FftT<float>: the same algorithm in
		// float, like FFTW's float plans the reference calls); set per worker
		// thread by orc_fse_baseline_f32 only, so the checker stays in double.
		thread_local bool tl_float_fft = false;
		std::map<std::pair<std::size_t, int>, std::shared_ptr<Fft32>> plans32;

		std::shared_ptr<Fft32> Plan32(std::size_t n, int sign) {
			std::lock_guard<std::mutex> lock(plan_mutex);
			auto& slot = plans32[{n, sign}];
			if (!slot)
				slot = std::make_shared<Fft32>(n, sign);
			return slot;
		}
	}

	// ---------------------------------------------------------------- mixer
	// TableMixer (mixer/table_mixer.hpp:27-58, 78-101) behind Mixer::Translate
	// (mixer/mixer.hpp:21-25, 33-42): 64-entry phase LUT (table of 80 sines,
	// cos = table[i + 16]), 32-bit NCO with adder = floor(2^32 f / fs)
	// (mixer/nco.hpp:17-20), index = top 6 bits, complex multiply in T.
	template <typename T>
	void TableMix(std::complex<T>* x, std::size_t n, double fs, double f, double phase) {
		phase = std::fmod(phase, 2 * kPi);
		if (phase < 0)
			phase += 2 * kPi;
		if (std::abs(f) == 0.0)
			return;
		if (f < 0)
			f = fs + f;
		constexpr std::size_t table_size = 80;
		const double table_step = 5 * kPi / table_size / 2;
		T table[table_size];
		for (std::size_t i = 0; i < table_size; ++i)
			table[i] = static_cast<T>(std::sin(static_cast<double>(i) * table_step));
		const std::uint64_t adder = static_cast<std::uint64_t>(4294967296.0 * f / fs);
		std::uint32_t holder = static_cast<std::uint32_t>(static_cast<std::uint64_t>(4294967296.0 * phase / (2 * kPi)));
		for (std::size_t i = 0; i < n; ++i) {
			const std::uint32_t idx = holder >> 26;
			holder = static_cast<std::uint32_t>(holder + adder);
			const T c = table[idx + 16], s = table[idx];
			const T a = x[i].real(), b = x[i].imag();
			// (a + ib)(c + is) evaluated as the reference's complex<T> multiply
			const volatile T re = a * c;
			const volatile T re2 = b * s;
			const volatile T im = a * s;
			const volatile T im2 = b * c;
			x[i] = std::complex<T>(re - re2, im + im2);
		}
	}

	// ------------------------------------------------------------- DFT / MF
	// SequentialDft with FFTW (math/dft.hpp:114-135): forward unnormalised;
	// inverse scaled by 1/N then 2 (dft.hpp:124-129).
	template <typename T>
	void DftC2c(const std::complex<T>* in, std::complex<T>* out, std::size_t n, bool inverse) {
		if constexpr (std::is_same_v<T, float>) {
			if (tl_float_fft) {
				Plan32(n, inverse ? +1 : -1)->Execute(in, out);
				if (inverse)
					for (std::size_t i = 0; i < n; ++i) {
						out[i] /= static_cast<T>(n);
						out[i] *= static_cast<T>(2);
					}
				return;
			}
		}
		std::vector<cd> a(n), b(n);
		for (std::size_t i = 0; i < n; ++i)
			a[i] = cd(in[i].real(), in[i].imag());
		Transform(a.data(), b.data(), n, inverse ? +1 : -1);
		for (std::size_t i = 0; i < n; ++i)
			out[i] = std::complex<T>(static_cast<T>(b[i].real()), static_cast<T>(b[i].imag()));
		if (inverse)
			for (std::size_t i = 0; i < n; ++i) {
				out[i] /= static_cast<T>(n);
				out[i] *= static_cast<T>(2);
			}
	}

	// r2c: bins 0..n/2 filled, n/2+1..n-1 left zero (dft.hpp:37-46, 184-192)
	template <typename T>
	void DftR2c(const T* in, std::complex<T>* out, std::size_t n) {
		std::vector<cd> a(n), b(n);
		for (std::size_t i = 0; i < n; ++i)
			a[i] = cd(in[i], 0.0);
		Transform(a.data(), b.data(), n, -1);
		for (std::size_t i = 0; i < n; ++i)
			out[i] = i <= n / 2 ? std::complex<T>(static_cast<T>(b[i].real()), static_cast<T>(b[i].imag())) : std::complex<T>{};
	}

	// spectrum_mode 0 = one-sided (FFTW path), 1 = two-sided (IPP/ArrayFire paths,
	// matched_filter/ipp_matched_filter.hpp:73-79): full conj spectrum, 1/N scale.
	template <typename T>
	void PrepareCodeSpectrum(const T* code, std::complex<T>* out, std::size_t n, int spectrum_mode) {
		if (spectrum_mode == 0) {
			DftR2c(code, out, n);
		}
		else {
			std::vector<cd> a(n), b(n);
			for (std::size_t i = 0; i < n; ++i)
				a[i] = cd(code[i], 0.0);
			Transform(a.data(), b.data(), n, -1);
			for (std::size_t i = 0; i < n; ++i)
				out[i] = std::complex<T>(static_cast<T>(b[i].real()), static_cast<T>(b[i].imag()));
		}
		for (std::size_t i = 0; i < n; ++i)
			out[i] = std::conj(out[i]);  // SequentialConj (math/conj.hpp:28-32)
	}

	// SequentialMatchedFilter::ProcessOptimized (matched_filter.hpp:56-61)
	template <typename T>
	void FilterOptimized(std::complex<T>* x, const std::complex<T>* spectrum, std::size_t n, int spectrum_mode) {
		std::vector<std::complex<T>> f(n);
		DftC2c(x, f.data(), n, false);
		for (std::size_t i = 0; i < n; ++i)
			f[i] *= spectrum[i];
		if (spectrum_mode == 0) {
			DftC2c(f.data(), x, n, true);
		}
		else {
			std::vector<cd> a(n), b(n);
			for (std::size_t i = 0; i < n; ++i)
				a[i] = cd(f[i].real(), f[i].imag());
			Transform(a.data(), b.data(), n, +1);
			for (std::size_t i = 0; i < n; ++i)
				x[i] = std::complex<T>(static_cast<T>(b[i].real() / n), static_cast<T>(b[i].imag() / n));
		}
	}

	// ------------------------------------------------------------ reductions
	template <typename T>
	void Abs(const std::complex<T>* x, T* out, std::size_t n) {  // math/abs.hpp:24-32
		for (std::size_t i = 0; i < n; ++i)
			out[i] = std::abs(x[i]);
	}

	// ReshapeAndSum (math/reshape_and_sum.hpp:15-18, 73-81): fold into `block`
	template <typename V>
	int ReshapeSum(V* v, std::size_t n, std::size_t block) {
		if (block == 0 || n % block != 0)
			return -1;
		for (std::size_t i = 1; i < n / block; ++i)
			for (std::size_t j = 0; j < block; ++j)
				v[j] += v[j + i * block];
		return 0;
	}

	template <typename T>
	std::size_t MaxIndex(const T* v, std::size_t n) {  // math/max_index.hpp:31-42: first maximum
		return static_cast<std::size_t>(std::max_element(v, v + n) - v);
	}

	template <typename T>
	void MeanStd(const T* v, std::size_t n, T* mean, T* sigma) {  // math/mean_stddev.hpp:29-42
		if (n < 2) {
			*mean = 0;
			*sigma = 0;
			return;
		}
		T q{}, m{};
		for (std::size_t i = 0; i < n; ++i) {
			q += v[i] * v[i];
			m += v[i];
		}
		const T val = (q - m * m / n) / (n - 1);
		*mean = m / n;
		*sigma = std::sqrt(val);
	}

	// ------------------------------------------------------------ resampling
	// RepeatCodeNTimes (common.hpp:78-85) + SequentialUpsampler (resample/upsampler.hpp:30-37)
	template <typename V>
	void Upsample(const V* src, std::size_t len, V* dst, std::size_t samples) {
		for (std::size_t i = 0; i < samples; ++i)
			dst[i] = src[(i * len / samples) % len];
	}

	// SequentialResampler (resample/resampler.hpp:80-87) + Accumulator
	// (resample/decimator.hpp:144-160): ZOH to lcm, boxcar mean of lcm/new_fs.
	// The reference names div's (quot, rem) as [rem, quot]; a non-zero remainder
	// pads to (quot + 1) * ratio with zeros.  Output length returned.
	template <typename T>
	std::size_t Resample(const std::complex<T>* src, std::size_t n, std::complex<T>* dst, std::size_t new_fs, std::size_t old_fs) {
		const std::size_t lcm = std::lcm(new_fs, old_fs);
		const std::size_t up = lcm * n / old_fs;
		const std::size_t ratio = lcm / new_fs;
		if (ratio == 1) {
			for (std::size_t i = 0; i < up; ++i)
				dst[i] = src[(i * n / up) % n];
			return up;
		}
		const std::size_t quot = up / ratio, rem = up % ratio;
		const std::size_t padded = rem ? (quot + 1) * ratio : up;
		const std::size_t out_n = padded / ratio;
		for (std::size_t k = 0; k < out_n; ++k) {
			std::complex<T> acc{};
			for (std::size_t j = 0; j < ratio; ++j) {
				const std::size_t i = k * ratio + j;
				if (i < up)
					acc += src[(i * n / up) % n];
			}
			dst[k] = acc / static_cast<T>(ratio);
		}
		return out_n;
	}

	// ----------------------------------------------------------- acquisition
	struct AcqRecord {
		double level, sigma, code_offset, doppler, index, doppler_bin, snr, mean, std;
	};

	// FastSearchEngineBase::ProcessBpsk (acquisition/fse.hpp:242-276) with the
	// per-block GetOneMsPeak output (fse.hpp:201-220) summed over K consecutive
	// coherent blocks of n samples (K = 1: the reference loop as written).
	// stat 0 = |y| (reference), 1 = |y|^2.  All Doppler bins are reported in
	// grid[bin] (level, index, mean, sigma) when grid != nullptr.
	template <typename T>
	void Acquire(const std::complex<T>* signal, std::size_t n_total, std::size_t n, std::size_t k_blocks,
		const T* code, double fs, double range, double step, double if_freq, double ratio,
		int reshape, int coherent, int stat, int spectrum_mode, AcqRecord* rec, double* grid, T* best_output) {
		std::vector<std::complex<T>> spectrum(n);
		PrepareCodeSpectrum(code, spectrum.data(), n, spectrum_mode);
		const std::size_t spm = static_cast<std::size_t>(fs / 1e3);
		const std::size_t m = reshape ? spm : n;
		std::vector<std::complex<T>> mixed(n_total), block(n);
		std::vector<T> acc(m), one(n);
		bool have = false;
		AcqRecord best{};
		std::int64_t bin = 0;
		for (double doppler = -range; doppler <= range; doppler += step, ++bin) {
			std::copy(signal, signal + n_total, mixed.begin());
			TableMix(mixed.data(), n_total, fs, -doppler, 0.0);
			std::fill(acc.begin(), acc.end(), T{});
			for (std::size_t b = 0; b < k_blocks; ++b) {
				std::copy(mixed.begin() + b * n, mixed.begin() + (b + 1) * n, block.begin());
				FilterOptimized(block.data(), spectrum.data(), n, spectrum_mode);
				if (reshape && !coherent) {
					ReshapeSum(block.data(), n, spm);
					for (std::size_t i = 0; i < m; ++i)
						one[i] = stat ? std::norm(block[i]) : std::abs(block[i]);
				}
				else {
					for (std::size_t i = 0; i < n; ++i)
						one[i] = stat ? std::norm(block[i]) : std::abs(block[i]);
					if (reshape)
						ReshapeSum(one.data(), n, spm);
				}
				for (std::size_t i = 0; i < m; ++i)
					acc[i] += one[i];
			}
			const std::size_t idx = MaxIndex(acc.data(), m);
			T mean{}, sd{};
			MeanStd(acc.data(), m, &mean, &sd);
			const double level = acc[idx];
			if (grid) {
				grid[4 * bin + 0] = level;
				grid[4 * bin + 1] = static_cast<double>(idx);
				grid[4 * bin + 2] = mean;
				grid[4 * bin + 3] = sd;
			}
			if (!have || best.level < level) {  // first strictly greater wins (fse.hpp:265)
				have = true;
				best.level = level;
				best.sigma = static_cast<double>(sd) + static_cast<double>(mean);
				best.code_offset = ratio * static_cast<double>(idx);
				best.doppler = doppler + if_freq;
				best.index = static_cast<double>(idx);
				best.doppler_bin = static_cast<double>(bin);
				best.mean = mean;
				best.std = sd;
				if (best_output)
					std::copy(acc.begin(), acc.end(), best_output);
			}
		}
		best.snr = best.level / best.sigma;
		*rec = best;
	}

	// ------------------------------------------------------------- tracking
	// AddWithPhase (tracking/tracking_parameters.hpp:89-98)
	template <typename T>
	std::complex<T> AddWithPhase(std::complex<T> lhs, std::complex<T> rhs, double relative_phase) {
		if (relative_phase < 0.5)
			std::swap(lhs, rhs);
		const auto wl = lhs.real() / relative_phase;
		const auto wr = rhs.real() / (1.0 - relative_phase);
		if (std::abs(wl + wr) > std::abs(wl))
			return lhs + rhs;
		return lhs - rhs;
	}

	// CorrelateSplit (tracking/tracking_parameters.hpp:472-493): one tap at a
	// fractional code phase as two dot products split at the period boundary.
	template <typename T>
	std::complex<T> CorrelateSplit(const std::complex<T>* sig, const T* full_code, std::size_t samples_per_ms,
		double code_period_ms, double phase) {
		const double period = static_cast<double>(samples_per_ms) * code_period_ms;
		while (phase < 0)
			phase += period;
		if (phase > period)
			phase = std::fmod(phase, period);
		const std::size_t first_len = static_cast<std::size_t>(std::ceil(phase)) % samples_per_ms;
		const std::size_t second_len = samples_per_ms - first_len;
		const std::size_t first_phase = static_cast<std::size_t>(std::ceil(2 * period - phase));
		const std::size_t second_phase = first_phase + first_len;
		std::complex<T> a{}, b{};
		for (std::size_t i = 0; i < first_len; ++i)
			a += sig[i] * full_code[first_phase + i];
		for (std::size_t i = 0; i < second_len; ++i)
			b += sig[first_len + i] * full_code[second_phase + i];
		return AddWithPhase(a, b, std::fmod(phase, static_cast<double>(samples_per_ms)) / samples_per_ms);
	}

	// ------------------------------------------------ interference mitigation
	// SequentialStft::SplitIntoColumns (math/stft.hpp:34-61): column i =
	// x[i hop, i hop + w) times the periodic Hann window (double, stored as T)
	// through std::multiplies<complex<T>>, forward DFT.
	template <typename T>
	std::vector<std::vector<std::complex<T>>> Stft(const std::complex<T>* x, std::size_t n, std::size_t w, std::size_t overlap) {
		const std::size_t hop = w - overlap;
		const std::size_t cols = (n - overlap) / hop;
		std::vector<T> win(w);
		for (std::size_t i = 0; i < w; ++i)
			win[i] = static_cast<T>(0.5 * (1 - std::cos(2.0 * kPi * static_cast<double>(i) / static_cast<double>(w))));
		std::vector<std::vector<std::complex<T>>> dst(cols, std::vector<std::complex<T>>(w));
		for (std::size_t c = 0; c < cols; ++c) {
			std::vector<std::complex<T>> v(w);
			for (std::size_t i = 0; i < w; ++i)
				v[i] = x[c * hop + i] * std::complex<T>(win[i]);
			DftC2c(v.data(), dst[c].data(), w, false);
		}
		return dst;
	}

	// OverlapAndAdd (math/stft.hpp:63-75): inverse DFTs (2/w scaled) summed at i hop
	template <typename T>
	std::vector<std::complex<T>> OverlapAdd(const std::vector<std::vector<std::complex<T>>>& cols, std::size_t w, std::size_t overlap) {
		const std::size_t hop = w - overlap;
		std::vector<std::complex<T>> dst(w + (cols.size() - 1) * hop);
		std::vector<std::complex<T>> inv(w);
		for (std::size_t i = 0; i < cols.size(); ++i) {
			DftC2c(cols[i].data(), inv.data(), w, true);
			for (std::size_t j = 0; j < w; ++j)
				dst[i * hop + j] += inv[j];
		}
		return dst;
	}

	struct JamCandidate {
		std::size_t bin;
		double frequency;
		double jn;
	};
	struct JamDetection {
		int type;  // 1 narrowband, 2 wideband
		std::size_t bin;
		double frequency;
		double jn;
	};

	// JammingDetector::IntermediateDetection (antijamming/jamming_detection.hpp:
	// 113-128) with its NullRegion (101-110): 8 rounds of first max then +-3
	// bins nulled, J/N against the sigma of what is left, J/N < 6 erased.
	template <typename T>
	std::vector<std::vector<JamCandidate>> JamIntermediate(const std::vector<std::vector<std::complex<T>>>& stft, double fs) {
		std::vector<std::vector<JamCandidate>> out(stft.size());
		for (std::size_t c = 0; c < stft.size(); ++c) {
			const std::size_t w = stft[c].size();
			std::vector<T> mag(w);
			for (std::size_t k = 0; k < w; ++k)
				mag[k] = std::abs(stft[c][k]);
			auto& cand = out[c];
			for (int r = 0; r < 8; ++r) {
				const std::size_t index = MaxIndex(mag.data(), w);
				cand.push_back({index, static_cast<double>(index) * fs / static_cast<double>(w), static_cast<double>(mag[index])});
				const std::size_t start = (index - 3 + w) % w;
				std::size_t finish = (index + 3 + w) % w;
				if (finish < start)
					finish += w;
				for (std::size_t i = start; i <= finish; ++i)
					mag[i % w] = 0;
			}
			T mean{}, sd{};
			MeanStd(mag.data(), w, &mean, &sd);
			for (auto& el : cand)
				el.jn /= sd;
			cand.erase(std::remove_if(cand.begin(), cand.end(), [](const JamCandidate& v) { return v.jn < 6.0; }), cand.end());
		}
		return out;
	}

	// AnalyzeStftData (jamming_detection.hpp:130-189)
	std::vector<JamDetection> JamAnalyze(const std::vector<std::vector<JamCandidate>>& inter) {
		std::vector<JamDetection> dst;
		std::size_t mean_jammers = 0;
		for (auto& el : inter)
			mean_jammers += el.size();
		mean_jammers /= inter.size();
		for (std::size_t i = 0; i < mean_jammers; ++i) {
			std::map<double, std::pair<double, JamCandidate>> occ;
			double quantity = 0;
			for (auto& el : inter) {
				if (el.size() <= i)
					continue;
				auto& slot = occ[el[i].frequency];
				slot.first += 1;
				slot.second.frequency = el[i].frequency;
				slot.second.bin = el[i].bin;
				slot.second.jn += el[i].jn;
				++quantity;
			}
			for (auto& kv : occ) {
				kv.second.first /= quantity;
				kv.second.second.jn /= quantity;
			}
			std::size_t cnt_wideband = 0;
			const JamCandidate* wide = &occ.begin()->second.second;
			for (auto& kv : occ) {
				const double probability = kv.second.first;
				if (probability >= 0.9) {
					dst.push_back({1, kv.second.second.bin, kv.second.second.frequency, kv.second.second.jn});
					break;
				}
				if (probability >= 0.9 / static_cast<double>(occ.size())) {
					++cnt_wideband;
					wide = &kv.second.second;
				}
			}
			if (cnt_wideband >= static_cast<std::size_t>(occ.size() * 0.9))
				dst.push_back({2, wide->bin, wide->frequency, wide->jn});
		}
		return dst;
	}

	// JammingSuppressionEngine::Process (antijamming/jse.hpp:89-102) in place
	template <typename T>
	std::vector<JamDetection> JamProcess(std::complex<T>* x, std::size_t n, double fs, bool suppress) {
		auto stft = Stft(x, n, 128, 96);
		const auto det = JamAnalyze(JamIntermediate(stft, fs));
		if (!suppress || det.empty())
			return det;
		const bool wideband = std::any_of(det.begin(), det.end(), [](const JamDetection& d) { return d.type == 2; });
		if (!wideband) {
			// FilterInFreqencyDomain (jse.hpp:61-68) with NullRegion (50-59)
			std::vector<std::complex<T>> spec(n);
			DftC2c(x, spec.data(), n, false);
			for (auto& d : det) {
				const auto idx = static_cast<std::size_t>(d.frequency / fs * static_cast<double>(n));
				std::ptrdiff_t start = static_cast<std::ptrdiff_t>(idx) - 128;
				std::ptrdiff_t finish = static_cast<std::ptrdiff_t>(idx) + 128;
				start += static_cast<std::ptrdiff_t>(n);
				if (finish < start)
					finish += static_cast<std::ptrdiff_t>(n);
				for (std::ptrdiff_t i = start; i <= finish; ++i)
					spec[static_cast<std::size_t>(i) % n] = 0;
			}
			DftC2c(spec.data(), x, n, true);
			return det;
		}
		// FilterWideband (jse.hpp:70-87)
		for (auto& col : stft)
			for (auto& el : col)
				if (std::abs(el) >= 20.0)
					el = 0;
		auto y = OverlapAdd(stft, 128, 96);
		y.resize(n);
		std::copy(y.begin(), y.end(), x);
		return det;
	}
}

using namespace oracle;

extern "C" {

#define ORC_BOTH(decl_f, decl_d) decl_f decl_d

void orc_table_mixer_f32(float* iq, std::size_t n, double fs, double f, double phase) {
	TableMix(reinterpret_cast<std::complex<float>*>(iq), n, fs, f, phase);
}
void orc_table_mixer_f64(double* iq, std::size_t n, double fs, double f, double phase) {
	TableMix(reinterpret_cast<std::complex<double>*>(iq), n, fs, f, phase);
}
void orc_dft_c2c_f64(const double* in, double* out, std::size_t n, int inverse) {
	DftC2c(reinterpret_cast<const std::complex<double>*>(in), reinterpret_cast<std::complex<double>*>(out), n, inverse != 0);
}
void orc_dft_c2c_f32(const float* in, float* out, std::size_t n, int inverse) {
	DftC2c(reinterpret_cast<const std::complex<float>*>(in), reinterpret_cast<std::complex<float>*>(out), n, inverse != 0);
}
void orc_dft_r2c_f32(const float* in, float* out, std::size_t n) {
	DftR2c(in, reinterpret_cast<std::complex<float>*>(out), n);
}
void orc_prepare_code_spectrum_f32(const float* code, std::size_t n, int mode, float* out) {
	PrepareCodeSpectrum(code, reinterpret_cast<std::complex<float>*>(out), n, mode);
}
void orc_prepare_code_spectrum_f64(const double* code, std::size_t n, int mode, double* out) {
	PrepareCodeSpectrum(code, reinterpret_cast<std::complex<double>*>(out), n, mode);
}
void orc_filter_optimized_f32(float* iq, std::size_t n, const float* spectrum, int mode) {
	FilterOptimized(reinterpret_cast<std::complex<float>*>(iq), reinterpret_cast<const std::complex<float>*>(spectrum), n, mode);
}
void orc_filter_optimized_f64(double* iq, std::size_t n, const double* spectrum, int mode) {
	FilterOptimized(reinterpret_cast<std::complex<double>*>(iq), reinterpret_cast<const std::complex<double>*>(spectrum), n, mode);
}
void orc_abs_f32(const float* iq, std::size_t n, float* out) {
	Abs(reinterpret_cast<const std::complex<float>*>(iq), out, n);
}
int orc_reshape_sum_f32(float* v, std::size_t n, std::size_t block) { return ReshapeSum(v, n, block); }
int orc_reshape_sum_c32(float* iq, std::size_t n, std::size_t block) {
	return ReshapeSum(reinterpret_cast<std::complex<float>*>(iq), n, block);
}
std::size_t orc_max_index_f32(const float* v, std::size_t n) { return MaxIndex(v, n); }
void orc_mean_std_f32(const float* v, std::size_t n, float* mean, float* sigma) { MeanStd(v, n, mean, sigma); }
void orc_mean_std_f64(const double* v, std::size_t n, double* mean, double* sigma) { MeanStd(v, n, mean, sigma); }
void orc_upsample_f32(const float* src, std::size_t len, float* dst, std::size_t samples) { Upsample(src, len, dst, samples); }
std::size_t orc_resample_c32(const float* iq, std::size_t n, float* out, std::size_t new_fs, std::size_t old_fs) {
	return Resample(reinterpret_cast<const std::complex<float>*>(iq), n, reinterpret_cast<std::complex<float>*>(out), new_fs, old_fs);
}
void orc_correlate_f32(const float* iq, const float* code, std::size_t n, float* out) {
	std::complex<float> acc{};
	const auto* s = reinterpret_cast<const std::complex<float>*>(iq);
	for (std::size_t i = 0; i < n; ++i)
		acc += s[i] * code[i];  // std::inner_product (correlator/correlator.hpp:27-34)
	out[0] = acc.real();
	out[1] = acc.imag();
}
void orc_correlate_split_f32(const float* iq, const float* full_code, std::size_t samples_per_ms, double code_period_ms,
	double phase, float* out) {
	auto r = CorrelateSplit(reinterpret_cast<const std::complex<float>*>(iq), full_code, samples_per_ms, code_period_ms, phase);
	out[0] = r.real();
	out[1] = r.imag();
}

// rec[9]: level, sigma(=std+mean), code_offset, doppler(+IF), index, doppler_bin, snr, mean, std
void orc_acquire_f32(const float* iq, std::size_t n_total, std::size_t n, std::size_t k_blocks, const float* code,
	double fs, double range, double step, double if_freq, double ratio, int reshape, int coherent, int stat,
	int spectrum_mode, double* rec, double* grid, float* best_output) {
	AcqRecord r{};
	Acquire(reinterpret_cast<const std::complex<float>*>(iq), n_total, n, k_blocks, code, fs, range, step, if_freq, ratio,
		reshape, coherent, stat, spectrum_mode, &r, grid, best_output);
	std::memcpy(rec, &r, sizeof(r));
}
void orc_acquire_f64(const double* iq, std::size_t n_total, std::size_t n, std::size_t k_blocks, const double* code,
	double fs, double range, double step, double if_freq, double ratio, int reshape, int coherent, int stat,
	int spectrum_mode, double* rec, double* grid, double* best_output) {
	AcqRecord r{};
	Acquire(reinterpret_cast<const std::complex<double>*>(iq), n_total, n, k_blocks, code, fs, range, step, if_freq, ratio,
		reshape, coherent, stat, spectrum_mode, &r, grid, best_output);
	std::memcpy(rec, &r, sizeof(r));
}

// Many PRNs over the same signal on `threads` host threads (the reference runs
// its PRN loop under std::execution::par_unseq, fse.hpp:294).  codes: n_codes x n.
void orc_acquire_many_f32(const float* iq, std::size_t n_total, std::size_t n, std::size_t k_blocks, const float* codes,
	std::size_t n_codes, double fs, double range, double step, double if_freq, double ratio, int reshape, int coherent,
	int stat, int spectrum_mode, int threads, double* recs /* n_codes x 9 */) {
	std::atomic<std::size_t> next{0};
	auto worker = [&]() {
		for (std::size_t c; (c = next.fetch_add(1)) < n_codes;) {
			AcqRecord r{};
			Acquire(reinterpret_cast<const std::complex<float>*>(iq), n_total, n, k_blocks, codes + c * n, fs, range, step,
				if_freq, ratio, reshape, coherent, stat, spectrum_mode, &r, nullptr, static_cast<float*>(nullptr));
			std::memcpy(recs + 9 * c, &r, sizeof(r));
		}
	};
	if (threads <= 1) {
		worker();
		return;
	}
	std::vector<std::thread> pool;
	for (int t = 0; t < threads; ++t)
		pool.emplace_back(worker);
	for (auto& t : pool)
		t.join();
}


// The CPU baseline: orc_acquire_many_f32 with every per-block transform in
// float (FftT<float>), the reference's FFTW float path restated; plans are
// cached per size (the reference plans per call with FFTW_ESTIMATE).
void orc_fse_baseline_f32(const float* iq, std::size_t n_total, std::size_t n, std::size_t k_blocks, const float* codes,
	std::size_t n_codes, double fs, double range, double step, int threads, double* recs /* n_codes x 9 */) {
	std::atomic<std::size_t> next{0};
	auto worker = [&]() {
		tl_float_fft = true;
		for (std::size_t c; (c = next.fetch_add(1)) < n_codes;) {
			AcqRecord r{};
			Acquire(reinterpret_cast<const std::complex<float>*>(iq), n_total, n, k_blocks, codes + c * n, fs, range, step,
				0.0, 1.0, 0, 1, 0, 0, &r, nullptr, static_cast<float*>(nullptr));
			std::memcpy(recs + 9 * c, &r, sizeof(r));
		}
		tl_float_fft = false;
	};
	if (threads <= 1) {
		worker();
		return;
	}
	std::vector<std::thread> pool;
	for (int t = 0; t < threads; ++t)
		pool.emplace_back(worker);
	for (auto& t : pool)
		t.join();
}

// SequentialStft split: returns the column count, columns to out when non-null
std::size_t orc_stft_f32(const float* iq, std::size_t n, int w, int overlap, float* out) {
	const auto cols = Stft(reinterpret_cast<const std::complex<float>*>(iq), n, static_cast<std::size_t>(w), static_cast<std::size_t>(overlap));
	if (out)
		for (std::size_t c = 0; c < cols.size(); ++c)
			std::memcpy(out + 2 * c * w, cols[c].data(), sizeof(float) * 2 * w);
	return cols.size();
}
// OverlapAndAdd of n_cols columns of w complex samples
void orc_istft_f32(const float* cols_iq, std::size_t n_cols, int w, int overlap, float* out) {
	std::vector<std::vector<std::complex<float>>> cols(n_cols, std::vector<std::complex<float>>(w));
	for (std::size_t c = 0; c < n_cols; ++c)
		std::memcpy(cols[c].data(), cols_iq + 2 * c * w, sizeof(float) * 2 * w);
	const auto y = OverlapAdd(cols, static_cast<std::size_t>(w), static_cast<std::size_t>(overlap));
	std::memcpy(out, y.data(), sizeof(float) * 2 * y.size());
}
// JammingDetector::Process (suppress = 0) or JammingSuppressionEngine::Process
// (suppress = 1, iq modified in place); returns the detection count
int orc_jamming_process_f32(float* iq, std::size_t n, double fs, int suppress, int* types, long* bins, double* freqs,
	double* jn, int cap) {
	const auto det = JamProcess(reinterpret_cast<std::complex<float>*>(iq), n, fs, suppress != 0);
	for (int i = 0; i < cap && i < static_cast<int>(det.size()); ++i) {
		types[i] = det[i].type;
		bins[i] = static_cast<long>(det[i].bin);
		freqs[i] = det[i].frequency;
		jn[i] = det[i].jn;
	}
	return static_cast<int>(det.size());
}
}

// ugsdr_cuda_policies.hpp - Cuda* policy classes for ugsdr's CRTP interfaces.
//
// Drop this header into the reference tree as src/cuda/ugsdr_cuda_policies.hpp
// (next to src/mixer, src/matched_filter, ...), link libugsdr_cuda.so, and
//   using Config = ugsdr::ParametricCudaFseConfig<8192000>;
//   ugsdr::FastSearchEngineBase<Config, ugsdr::DefaultChannelConfig, float> fse(dfe, 5e3, 200);
// compiles unchanged: every class derives from the reference interface it
// replaces, so the FseConfig static_asserts (src/acquisition/fse.hpp:59-66)
// hold.  Each policy forwards to one C entry point of ugsdr_cuda.h; a
// failure status is rethrown as std::runtime_error, as the CPU policies throw.
// Computation is float on the GPU; double instantiations convert.
//
// UGSDR_REF_SRC may point at the reference's src/ directory when the header
// is used from elsewhere (default: the parent directory of this header).
#pragma once

#include "ugsdr_cuda.h"
#include "ugsdr_cuda_engine.hpp"

#ifndef UGSDR_REF_SRC
#define UGSDR_REF_SRC ..
#endif
#define UGSDR_STR2(x) #x
#define UGSDR_STR(x) UGSDR_STR2(x)
#include UGSDR_STR(UGSDR_REF_SRC/acquisition/fse.hpp)
#include UGSDR_STR(UGSDR_REF_SRC/correlator/correlator.hpp)
#include UGSDR_STR(UGSDR_REF_SRC/math/dft.hpp)
#include UGSDR_STR(UGSDR_REF_SRC/math/stft.hpp)
#include UGSDR_STR(UGSDR_REF_SRC/antijamming/jamming_detection.hpp)

#include <complex>
#include <span>
#include <stdexcept>
#include <string>
#include <vector>

namespace ugsdr {
	namespace cuda_detail {
		// one context per host thread: the reference calls its policies from
		// std::execution::par_unseq lambdas (fse.hpp:294, tracker.hpp:192)
		inline ugsdr_ctx* Context() {
			struct Holder {
				ugsdr_ctx* ctx = nullptr;
				Holder() {
					if (ugsdr_ctx_create(0, &ctx) != UGSDR_OK)
						throw std::runtime_error("ugsdr_ctx_create failed (no CUDA device?)");
				}
				~Holder() { ugsdr_ctx_destroy(ctx); }
			};
			static thread_local Holder holder;
			return holder.ctx;
		}

		inline void Check(int status) {
			if (status != UGSDR_OK)
				throw std::runtime_error(std::string("ugsdr_cuda: ") + ugsdr_last_error(Context()));
		}

		template <typename T>
		std::vector<std::complex<float>> ToF(const std::vector<std::complex<T>>& v) {
			if constexpr (std::is_same_v<T, float>)
				return v;
			else
				return std::vector<std::complex<float>>(v.begin(), v.end());
		}
		template <typename T>
		std::vector<float> ToF(const std::vector<T>& v) {
			if constexpr (std::is_same_v<T, float>)
				return v;
			else
				return std::vector<float>(v.begin(), v.end());
		}
		template <typename T, typename U>
		void Assign(std::vector<T>& dst, const std::vector<U>& src) {
			dst.assign(src.begin(), src.end());
		}
		inline float* F(std::vector<std::complex<float>>& v) { return reinterpret_cast<float*>(v.data()); }
		inline const float* F(const std::vector<std::complex<float>>& v) { return reinterpret_cast<const float*>(v.data()); }
	}

	// Mixer<TableMixer> arithmetic (table_mixer.hpp:78-101) on the GPU
	class CudaMixer final : public Mixer<CudaMixer> {
	protected:
		friend class Mixer<CudaMixer>;
		template <typename T>
		static void Process(std::vector<std::complex<T>>& src_dst, double fs, double f, double phase = 0) {
			auto v = cuda_detail::ToF(src_dst);
			cuda_detail::Check(ugsdr_mix(cuda_detail::Context(), cuda_detail::F(v), v.size(), fs, f, phase));
			cuda_detail::Assign(src_dst, v);
		}
		template <typename T>
		static auto Process(const std::vector<std::complex<T>>& src, double fs, double f, double phase = 0) {
			auto dst = src;
			Process(dst, fs, f, phase);
			return dst;
		}
	public:
		CudaMixer(double fs, double f, double phase) : Mixer<CudaMixer>(fs, f, phase) {}
	};

	class CudaDft final : public DiscreteFourierTransform<CudaDft> {
	protected:
		friend class DiscreteFourierTransform<CudaDft>;
		template <typename T>
		static auto Process(const std::vector<std::complex<T>>& src, bool is_inverse = false) {
			auto v = cuda_detail::ToF(src);
			std::vector<std::complex<float>> out(v.size());
			cuda_detail::Check(ugsdr_dft(cuda_detail::Context(), cuda_detail::F(v), cuda_detail::F(out), v.size(), is_inverse));
			std::vector<std::complex<T>> r;
			cuda_detail::Assign(r, out);
			return r;
		}
		template <typename T>
		static void Process(std::vector<std::complex<T>>& src_dst, bool is_inverse = false) {
			const auto& src = src_dst;
			src_dst = Process(src, is_inverse);
		}
	};

	// FFTW-path semantics (one-sided code spectrum, 2/N inverse scale)
	class CudaMatchedFilter final : public MatchedFilter<CudaMatchedFilter> {
	protected:
		friend class MatchedFilter<CudaMatchedFilter>;
		template <typename T>
		static auto Prepare(const std::vector<T>& impulse_response) {
			auto code = cuda_detail::ToF(impulse_response);
			std::vector<std::complex<float>> spec(code.size());
			cuda_detail::Check(ugsdr_matched_filter_prepare(cuda_detail::Context(), code.data(), code.size(),
				UGSDR_SPECTRUM_ONE_SIDED, cuda_detail::F(spec)));
			std::vector<std::complex<T>> r;
			cuda_detail::Assign(r, spec);
			return r;
		}
		template <typename T1, typename T2>
		static void ProcessOptimized(T1& src_dst, const T2& spectrum) {
			auto v = cuda_detail::ToF(src_dst);
			auto s = cuda_detail::ToF(spectrum);
			cuda_detail::Check(ugsdr_matched_filter(cuda_detail::Context(), cuda_detail::F(v), v.size(), cuda_detail::F(s),
				UGSDR_SPECTRUM_ONE_SIDED));
			cuda_detail::Assign(src_dst, v);
		}
		template <typename T1, typename T2>
		static void Process(T1& src_dst, const T2& impulse_response) {
			ProcessOptimized(src_dst, Prepare(impulse_response));
		}
	};

	class CudaAbs final : public Abs<CudaAbs> {
	protected:
		friend class Abs<CudaAbs>;
		template <typename T>
		static auto Process(const std::vector<std::complex<T>>& src) {
			auto v = cuda_detail::ToF(src);
			std::vector<float> out(v.size());
			cuda_detail::Check(ugsdr_abs(cuda_detail::Context(), cuda_detail::F(v), v.size(), out.data()));
			std::vector<T> r;
			cuda_detail::Assign(r, out);
			return r;
		}
	};

	class CudaReshapeAndSum final : public ReshapeAndSum<CudaReshapeAndSum> {
	protected:
		friend class ReshapeAndSum<CudaReshapeAndSum>;
		template <typename T>
		static void Process(std::vector<T>& src, std::size_t block) {
			constexpr bool cplx = is_complex_v<T>;
			auto v = cuda_detail::ToF(src);
			decltype(v) out(block);
			cuda_detail::Check(ugsdr_reshape_sum(cuda_detail::Context(), reinterpret_cast<const float*>(v.data()), v.size(),
				block, cplx, reinterpret_cast<float*>(out.data())));
			cuda_detail::Assign(src, out);
		}
		template <typename T>
		static auto Process(const std::vector<T>& src, std::size_t block) {
			auto dst = src;
			Process(dst, block);
			return dst;
		}
	};

	class CudaMaxIndex final : public MaxIndex<CudaMaxIndex> {
	protected:
		friend class MaxIndex<CudaMaxIndex>;
		template <typename T>
		static Result<T> Process(const std::vector<T>& src) {
			auto v = cuda_detail::ToF(src);
			float value = 0;
			std::size_t index = 0;
			cuda_detail::Check(ugsdr_max_index(cuda_detail::Context(), v.data(), v.size(), &value, &index));
			return Result<T>{static_cast<T>(value), index};
		}
	};

	class CudaMeanStdDev final : public MeanStdDev<CudaMeanStdDev> {
	protected:
		friend class MeanStdDev<CudaMeanStdDev>;
		template <typename T>
		static auto Process(const std::vector<T>& src) {
			auto v = cuda_detail::ToF(src);
			float mean = 0, sigma = 0;
			cuda_detail::Check(ugsdr_mean_stddev(cuda_detail::Context(), v.data(), v.size(), &mean, &sigma));
			return Result<T>{static_cast<T>(mean), static_cast<T>(sigma)};
		}
	};

	class CudaUpsampler final : public Upsampler<CudaUpsampler> {
	protected:
		friend class Upsampler<CudaUpsampler>;
		template <typename T>
		static void Process(std::vector<T>& src_dst, std::size_t samples) {
			constexpr bool cplx = is_complex_v<T>;
			auto v = cuda_detail::ToF(src_dst);
			decltype(v) out(samples);
			cuda_detail::Check(ugsdr_upsample(cuda_detail::Context(), reinterpret_cast<const float*>(v.data()), v.size(), cplx,
				reinterpret_cast<float*>(out.data()), samples));
			cuda_detail::Assign(src_dst, out);
		}
	};

	class CudaResampler final : public Resampler<CudaResampler> {
	protected:
		friend class Resampler<CudaResampler>;
		template <typename T>
		static void Process(std::vector<std::complex<T>>& src_dst, std::size_t new_fs, std::size_t old_fs) {
			auto v = cuda_detail::ToF(src_dst);
			std::size_t n_out = 0;
			auto* ctx = cuda_detail::Context();
			cuda_detail::Check(ugsdr_resample(ctx, cuda_detail::F(v), v.size(), new_fs, old_fs, nullptr, 0, &n_out));
			std::vector<std::complex<float>> out(n_out);
			cuda_detail::Check(ugsdr_resample(ctx, cuda_detail::F(v), v.size(), new_fs, old_fs, cuda_detail::F(out), n_out, &n_out));
			cuda_detail::Assign(src_dst, out);
		}
		template <typename T>
		static auto Process(const std::vector<std::complex<T>>& src, std::size_t new_fs, std::size_t old_fs) {
			auto dst = src;
			Process(dst, new_fs, old_fs);
			return dst;
		}
	};

	class CudaCorrelator final : public Correlator<CudaCorrelator> {
	protected:
		friend class Correlator<CudaCorrelator>;
		template <typename UnderlyingType, typename T>
		static auto Process(const std::span<const std::complex<UnderlyingType>>& signal, const std::span<const T>& code) {
			if (signal.size() != code.size())
				throw std::runtime_error("Size mismatch");
			std::vector<std::complex<float>> s(signal.begin(), signal.end());
			std::vector<float> c(code.begin(), code.end());
			float out[2];
			cuda_detail::Check(ugsdr_correlate(cuda_detail::Context(), cuda_detail::F(s), c.data(), c.size(), out));
			return std::complex<UnderlyingType>(out[0], out[1]);
		}
	};

	// SequentialStft (math/stft.hpp:33-88): both Transform overloads
	class CudaStft final : public ShortTimeFourierTransform<CudaStft> {
	protected:
		friend class ShortTimeFourierTransform<CudaStft>;
		template <typename T>
		static auto Process(const std::vector<T>& src, std::size_t window_length, std::size_t overlap_length) {
			using Dst = std::conditional_t<is_complex_v<T>, T, std::complex<T>>;
			std::vector<std::complex<float>> x(src.begin(), src.end());
			std::size_t cols = 0;
			auto* ctx = cuda_detail::Context();
			const int w = static_cast<int>(window_length), ov = static_cast<int>(overlap_length);
			cuda_detail::Check(ugsdr_stft(ctx, cuda_detail::F(x), x.size(), w, ov, nullptr, &cols));
			std::vector<std::complex<float>> flat(cols * window_length);
			cuda_detail::Check(ugsdr_stft(ctx, cuda_detail::F(x), x.size(), w, ov, cuda_detail::F(flat), &cols));
			std::vector<std::vector<Dst>> dst(cols);
			for (std::size_t c = 0; c < cols; ++c)
				dst[c].assign(flat.begin() + c * window_length, flat.begin() + (c + 1) * window_length);
			return dst;
		}
		template <typename T>
		static auto Process(const std::vector<std::vector<T>>& src, std::size_t window_length, std::size_t overlap_length) {
			std::vector<std::complex<float>> flat;
			flat.reserve(src.size() * window_length);
			for (const auto& col : src)
				flat.insert(flat.end(), col.begin(), col.end());
			std::vector<std::complex<float>> out(window_length + (src.size() - 1) * (window_length - overlap_length));
			cuda_detail::Check(ugsdr_istft(cuda_detail::Context(), cuda_detail::F(flat), src.size(), static_cast<int>(window_length),
				static_cast<int>(overlap_length), cuda_detail::F(out)));
			return std::vector<T>(out.begin(), out.end());
		}
	};

	// JammingSuppressionEngine<T> (antijamming/jse.hpp:24-107) on the GPU: the
	// same constructor, Process(src_dst) in place and GetDetectionResults.
	// The front end holds the engine as a member, not a policy
	// (dfe/dfe.hpp:113): a GPU build swaps that member's type.
	template <typename T>
	class CudaJammingSuppressionEngine {
	public:
		using DetectionResult = typename JammingDetector<std::complex<underlying_t<T>>>::DetectionResult;

		explicit CudaJammingSuppressionEngine(double sampling_rate) : fs(sampling_rate) {}

		void Process(std::vector<T>& src_dst) {
			auto x = cuda_detail::ToF(src_dst);
			ugsdr_jamming_detection det[16];
			int n = 0;
			cuda_detail::Check(ugsdr_jamming_suppress(cuda_detail::Context(), cuda_detail::F(x), x.size(), fs, 0, det, 16, &n));
			if constexpr (std::is_same_v<T, std::complex<float>>)
				src_dst.swap(x);
			else
				cuda_detail::Assign(src_dst, x);
			results.clear();
			for (int i = 0; i < n && i < 16; ++i)
				results.emplace_back(static_cast<typename DetectionResult::InterferenceType>(det[i].type),
					static_cast<std::size_t>(det[i].frequency_bin), det[i].frequency, det[i].jammer_to_noise);
		}

		const auto& GetDetectionResults() const { return results; }

	private:
		double fs = 0.0;
		std::vector<DetectionResult> results;
	};

	// FastSearchEngineBase's call surface (fse.hpp:450-507) over the batched
	// engine: constructed on the reference's DigitalFrontend with the Doppler
	// range and step, Process() reads the same 4 ms (GetSeveralEpochs) and
	// returns the reference's AcquisitionResult<T> sorted by Sv.  The GPS L1
	// C/A, L5I/L5Q, GLONASS L1OF and Galileo E1B subbands the frontend has are
	// searched (the systems cuda::CudaFastSearchEngine covers); unlike the
	// per-op Cuda* policies inside FastSearchEngineBase, every search of a call
	// goes to the GPU in one ugsdr_acquire_batch.
	template <ChannelConfigConcept ChConfig = DefaultChannelConfig, typename T = float>
	class CudaFastSearchEngineFor {
	public:
		CudaFastSearchEngineFor(DigitalFrontend<ChConfig, T>& dfe, double range, double step,
			double acquisition_sampling_rate = 8192000.0, int device = 0)
			: digital_frontend(dfe), engine({}, range, step, acquisition_sampling_rate, device) {}

		std::vector<AcquisitionResult<T>> Process(bool plot_results = false, std::size_t ms_offset = 0) {
			(void)plot_results;
			auto& epoch = digital_frontend.GetSeveralEpochs(ms_offset, cuda::CudaFastSearchEngine::ms_to_process);
			const std::pair<Signal, int> signals[] = {{Signal::GpsCoarseAcquisition_L1, UGSDR_GPS_L1CA}, {Signal::Gps_L5I, UGSDR_GPS_L5I},
				{Signal::Gps_L5Q, UGSDR_GPS_L5Q}, {Signal::GlonassCivilFdma_L1, UGSDR_GLONASS_L1OF}, {Signal::Galileo_E1b, UGSDR_GALILEO_E1B}};
			std::vector<std::vector<std::complex<float>>> buffers;
			std::vector<cuda::Subband> subbands;
			for (const auto& [sig, id] : signals) {
				if (!digital_frontend.HasSignal(sig))
					continue;
				buffers.push_back(cuda_detail::ToF(epoch.GetSubband(sig)));
				cuda::Subband s;
				s.signal = id;
				s.samples = buffers.back().data();
				s.sample_type = UGSDR_SAMPLES_CF32;
				s.n_samples = buffers.back().size();
				s.sampling_rate = digital_frontend.GetSamplingRate(sig);
				s.central_frequency = digital_frontend.GetCentralFrequency(sig);
				subbands.push_back(s);
			}
			engine.SetSubbands(subbands);
			const auto found = engine.Process(false, 0);
			std::vector<AcquisitionResult<T>> dst;
			for (const auto& r : found) {
				AcquisitionResult<T> a;
				a.sv_number.id = r.sv_number.id;
				a.sv_number.system = static_cast<System>(r.sv_number.system);
				a.sv_number.signal = static_cast<Signal>(r.sv_number.signal);
				a.doppler = r.doppler;
				a.code_offset = r.code_offset;
				a.level = r.level;
				a.sigma = r.sigma;
				a.intermediate_frequency = r.intermediate_frequency;
				dst.push_back(std::move(a));
			}
			return dst;
		}

	private:
		DigitalFrontend<ChConfig, T>& digital_frontend;
		cuda::CudaFastSearchEngine engine;
	};

	// FseConfig bundle (fse.hpp:36-67, 98-109) on the GPU policies
	template <auto acquisition_sampling_rate>
	using ParametricCudaFseConfig = FseConfig<
		acquisition_sampling_rate,
		CudaMixer,
		CudaUpsampler,
		CudaMatchedFilter,
		CudaAbs,
		CudaReshapeAndSum,
		CudaMaxIndex,
		CudaMeanStdDev,
		CudaResampler>;
}

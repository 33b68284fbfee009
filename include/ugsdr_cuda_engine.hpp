// ugsdr_cuda_engine.hpp - the fast search engine of ugsdr on the GPU.
//
// CudaFastSearchEngine has the call shape of ugsdr::FastSearchEngineBase
// (src/acquisition/fse.hpp:450-507): construct it with the capture, the
// Doppler range and step, call Process(plot_results, ms_offset) and get the
// acquired satellites sorted by Sv.  It does what the reference's per-system
// drivers do, with every search of a call in one ugsdr_acquire_batch:
//   GPS L1 C/A  AcquireGoldCodesL1 (fse.hpp:278-300): IF removal at the input
//               rate, AdjustSamplingRate (222-240), 32 codes of 4 ms folded
//               to 1 ms after |.| (GetOneMsPeak, 201-220); when no L1 C/A
//               satellite passes, L5I then L5Q (ProcessGps, 327-335:
//               AcquireL5, 302-325, at 20.46 MHz, folded before |.|)
//   GLONASS     ProcessGlonass (337-354): one search per letter
//               k = -7..5 with IF -(fc - (1602 MHz + k 562.5 kHz)), the
//               shared 511-chip code
//   Galileo E1B ProcessGalileo (356-396): 4 ms codes without folding, the
//               four per-ms sign permutations, the best of the four kept
// A satellite is kept when level / sigma > 3.3 (fse.hpp:272) - for Galileo,
// its best permutation.  Results carry the reference's fields; output_peak
// stays empty (the batched engine returns each search's peak record, not the
// folded correlation; the reference fills it only to plot it).
//
// No reference headers are needed; ugsdr_cuda_policies.hpp adds a
// constructor from the reference's DigitalFrontend.  Code spectra are built
// once per (signal, sv, length, permutation) and stay on the device between
// calls.  Errors are thrown as std::runtime_error.
#pragma once

#include "ugsdr_cuda.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

namespace ugsdr {
	namespace cuda {
		// ugsdr::System (src/common.hpp:68-76), the systems this engine searches
		enum class System : std::uint32_t { Gps = 0, Glonass = 1, Galileo = 2 };

		// ugsdr::Sv (src/common.hpp:147-150, ordering 282-288): id, system and
		// signal (an ugsdr_signal value, the reference's Signal numbering)
		struct Sv {
			std::int32_t id = 0;
			System system = System::Gps;
			std::uint32_t signal = UGSDR_GPS_L1CA;
			bool operator<(const Sv& rhs) const {
				if (system != rhs.system)
					return static_cast<std::uint32_t>(system) < static_cast<std::uint32_t>(rhs.system);
				if (signal != rhs.signal)
					return signal < rhs.signal;
				return id < rhs.id;
			}
		};

		// ugsdr::AcquisitionResult (src/acquisition/acquisition_result.hpp:11-27)
		template <typename T>
		struct AcquisitionResult {
			Sv sv_number;
			double doppler = 0;
			double code_offset = 0;
			double level = 0;
			double sigma = 1.0;
			double intermediate_frequency = 0;
			std::vector<T> output_peak;
			double GetSnr() const { return level / sigma; }
			bool operator<(const AcquisitionResult& rhs) const { return level < rhs.level; }
		};

		// One subband of the capture, as DigitalFrontend::GetSeveralEpochs(...)
		// .GetSubband(signal) hands it to the reference engine, with the
		// channel's sampling rate and central frequency.  `samples` holds at
		// least (ms_offset + 4) ms of sample_type samples (host memory unless
		// samples_on_device).
		struct Subband {
			int signal = UGSDR_GPS_L1CA;  // UGSDR_GPS_L1CA / _L5I / _L5Q, UGSDR_GLONASS_L1OF, UGSDR_GALILEO_E1B
			const void* samples = nullptr;
			int sample_type = UGSDR_SAMPLES_CF32;
			int samples_on_device = 0;
			std::size_t n_samples = 0;
			double sampling_rate = 0;
			double central_frequency = 0;
		};

		class CudaFastSearchEngine {
		public:
			static constexpr std::size_t ms_to_process = 4;
			static constexpr double peak_threshold = 3.3;
			static constexpr double acquisition_sampling_rate_L5 = 20.46e6;

			CudaFastSearchEngine(std::vector<Subband> subbands, double range, double step,
				double acquisition_sampling_rate = 8192000.0, int device = 0)
				: subbands_(std::move(subbands)), range_(range), step_(step), acq_rate_(acquisition_sampling_rate) {
				if (ugsdr_ctx_create(device, &ctx_) != UGSDR_OK)
					throw std::runtime_error("ugsdr_ctx_create failed (no CUDA device?)");
			}
			CudaFastSearchEngine(const CudaFastSearchEngine&) = delete;
			CudaFastSearchEngine& operator=(const CudaFastSearchEngine&) = delete;
			~CudaFastSearchEngine() {
				for (const auto& kv : handles_)
					ugsdr_code_release(ctx_, kv.second);
				ugsdr_ctx_destroy(ctx_);
			}

			ugsdr_ctx* Context() const { return ctx_; }

			// the capture a later Process() reads (code spectra stay cached)
			void SetSubbands(std::vector<Subband> subbands) { subbands_ = std::move(subbands); }

			// FastSearchEngineBase::AdjustSamplingRate (fse.hpp:222-240): the
			// divisor of the rate with whole kHz closest to the target, or the
			// signal's own rate when the search runs out of candidates
			static double AdjustSamplingRate(double signal_sampling_rate, double target_sampling_rate) {
				double new_rate = signal_sampling_rate;
				const auto limit = static_cast<std::size_t>(2 * signal_sampling_rate / target_sampling_rate);
				for (std::size_t i = 1; i < limit; ++i) {
					const double candidate = signal_sampling_rate / static_cast<double>(i);
					if (std::fmod(candidate / 1e3, 1) != 0.0)
						continue;
					if (std::abs(target_sampling_rate - candidate) > std::abs(target_sampling_rate - new_rate))
						return new_rate;
					new_rate = candidate;
				}
				return signal_sampling_rate;
			}

			std::vector<AcquisitionResult<float>> Process(bool plot_results = false, std::size_t ms_offset = 0) {
				(void)plot_results;  // the Windows viewer is not part of this backend
				std::vector<AcquisitionResult<float>> dst;
				std::vector<Search> searches;
				if (const Subband* s = Find(UGSDR_GPS_L1CA))
					AddGoldL1(*s, ms_offset, searches);
				if (const Subband* s = Find(UGSDR_GLONASS_L1OF))
					AddGlonass(*s, ms_offset, searches);
				if (const Subband* s = Find(UGSDR_GALILEO_E1B))
					AddGalileo(*s, ms_offset, searches);
				Run(searches, dst);
				// ProcessGps: L5I, then L5Q, only while no GPS satellite was kept
				for (const int l5 : {UGSDR_GPS_L5I, UGSDR_GPS_L5Q}) {
					const bool have_gps =
						std::any_of(dst.begin(), dst.end(), [](const auto& r) { return r.sv_number.system == System::Gps; });
					const Subband* s = Find(l5);
					if (have_gps || !s)
						continue;
					std::vector<Search> l5_searches;
					AddL5(*s, l5, ms_offset, l5_searches);
					Run(l5_searches, dst);
				}
				std::sort(dst.begin(), dst.end(), [](const auto& lhs, const auto& rhs) { return lhs.sv_number < rhs.sv_number; });
				return dst;
			}

		private:
			// one search = one ugsdr_acq_job; the satellite of each code slot
			struct Search {
				ugsdr_acq_job job{};
				std::vector<int> codes;
				std::vector<Sv> sv;
				bool galileo = false;  // four permutation slots per satellite, best kept
			};

			std::vector<Subband> subbands_;
			double range_, step_, acq_rate_;
			ugsdr_ctx* ctx_ = nullptr;
			std::map<std::tuple<int, int, std::size_t, std::uint32_t>, int> handles_;

			const Subband* Find(int signal) const {
				for (const auto& s : subbands_)
					if (s.signal == signal && s.samples && s.n_samples)
						return &s;
				return nullptr;
			}

			void Check(int status) const {
				if (status != UGSDR_OK)
					throw std::runtime_error(std::string("ugsdr_cuda: ") + ugsdr_last_error(ctx_));
			}

			// conj(FFT) of RepeatCodeNTimes(code, repeats) upsampled to n samples,
			// segment signs from sign_mask; cached for later calls
			int Code(int signal, int sv, std::size_t repeats, std::size_t n, std::uint32_t sign_mask, std::size_t sign_segment) {
				const auto key = std::make_tuple(signal, sv, n, sign_mask);
				if (auto it = handles_.find(key); it != handles_.end())
					return it->second;
				std::size_t len = 0;
				std::vector<float> chips(16384);
				Check(ugsdr_prn_code(signal, sv, chips.data(), chips.size(), &len));
				int h = -1;
				Check(ugsdr_code_put(ctx_, chips.data(), len, repeats, n, sign_mask, sign_segment, UGSDR_SPECTRUM_ONE_SIDED, &h));
				handles_[key] = h;
				return h;
			}

			// the 4 ms window at ms_offset of a subband, translated by -IF at the
			// input rate and resampled to the acquisition rate on the device
			ugsdr_acq_job BaseJob(const Subband& s, std::size_t ms_offset, double intermediate_frequency, double new_rate) const {
				std::size_t bytes_per_ms = 0;
				const auto spm = static_cast<std::size_t>(s.sampling_rate / 1e3);
				Check(ugsdr_sample_bytes(s.sample_type, s.sampling_rate, spm, &bytes_per_ms));
				if (s.n_samples < (ms_offset + ms_to_process) * spm)
					throw std::runtime_error("ugsdr_cuda: the subband holds fewer than ms_offset + 4 ms of samples");
				ugsdr_acq_job j{};
				j.samples = static_cast<const char*>(s.samples) + ms_offset * bytes_per_ms;
				j.sample_type = s.sample_type;
				j.samples_on_device = s.samples_on_device;
				j.n_samples = ms_to_process * spm;
				j.sampling_rate = new_rate;
				j.input_sampling_rate = new_rate != s.sampling_rate ? s.sampling_rate : 0.0;
				j.intermediate_frequency = intermediate_frequency;
				j.frontend_frequency = -intermediate_frequency;  // Translate(signal, fs, -IF)
				j.code_offset_ratio = s.sampling_rate / new_rate;
				j.block_samples = static_cast<std::size_t>(ms_to_process * new_rate / 1e3);
				j.n_blocks = 1;
				j.doppler_range = range_;
				j.doppler_step = step_;
				j.statistic = UGSDR_STAT_ABS;
				j.spectrum_mode = UGSDR_SPECTRUM_ONE_SIDED;
				return j;
			}

			void AddGoldL1(const Subband& s, std::size_t ms_offset, std::vector<Search>& out) {
				const double f_if = -(s.central_frequency - 1575.42e6);
				const double new_rate = AdjustSamplingRate(s.sampling_rate, acq_rate_);
				Search q;
				q.job = BaseJob(s, ms_offset, f_if, new_rate);
				q.job.fold_samples = static_cast<std::size_t>(new_rate / 1e3);
				q.job.fold_coherent = 1;  // |.| then fold (GetOneMsPeak<true, true>)
				for (int sv = 0; sv < 32; ++sv) {
					q.codes.push_back(Code(UGSDR_GPS_L1CA, sv, ms_to_process, q.job.block_samples, 0, 0));
					q.sv.push_back(Sv{sv, System::Gps, UGSDR_GPS_L1CA});
				}
				out.push_back(std::move(q));
			}

			void AddL5(const Subband& s, int signal, std::size_t ms_offset, std::vector<Search>& out) {
				const double f_if = -(s.central_frequency - 1176.45e6);
				const double new_rate = AdjustSamplingRate(s.sampling_rate, acquisition_sampling_rate_L5);
				Search q;
				q.job = BaseJob(s, ms_offset, f_if, new_rate);
				q.job.fold_samples = static_cast<std::size_t>(new_rate / 1e3);
				q.job.fold_coherent = 0;  // fold, then |.| (GetOneMsPeak<true, false>)
				for (int sv = 0; sv < 32; ++sv) {
					q.codes.push_back(Code(signal, sv, ms_to_process, q.job.block_samples, 0, 0));
					q.sv.push_back(Sv{sv, System::Gps, static_cast<std::uint32_t>(signal)});
				}
				out.push_back(std::move(q));
			}

			void AddGlonass(const Subband& s, std::size_t ms_offset, std::vector<Search>& out) {
				const double new_rate = AdjustSamplingRate(s.sampling_rate, acq_rate_);
				for (int k = -7; k < 6; ++k) {  // gln_min_frequency .. gln_max_frequency - 1 (fse.hpp:163-168)
					const double f_if = -(s.central_frequency - (1602e6 + k * 0.5625e6));
					Search q;
					q.job = BaseJob(s, ms_offset, f_if, new_rate);
					q.job.fold_samples = static_cast<std::size_t>(new_rate / 1e3);
					q.job.fold_coherent = 1;
					q.codes.push_back(Code(UGSDR_GLONASS_L1OF, 0, ms_to_process, q.job.block_samples, 0, 0));
					q.sv.push_back(Sv{k, System::Glonass, UGSDR_GLONASS_L1OF});
					out.push_back(std::move(q));
				}
			}

			void AddGalileo(const Subband& s, std::size_t ms_offset, std::vector<Search>& out) {
				const double f_if = -(s.central_frequency - 1575.42e6);
				const double new_rate = AdjustSamplingRate(s.sampling_rate, acq_rate_);
				Search q;
				q.job = BaseJob(s, ms_offset, f_if, new_rate);
				q.galileo = true;  // no fold (ProcessBpsk<false>)
				const auto spm = static_cast<std::size_t>(new_rate / 1e3);
				// sign permutations {1,1,1,1}, {1,1,1,-1}, {1,1,-1,-1}, {1,-1,-1,-1} (fse.hpp:374-388)
				const std::uint32_t masks[4] = {0u, 0x8u, 0xCu, 0xEu};
				for (int sv = 0; sv < 50; ++sv)
					for (const std::uint32_t m : masks) {
						q.codes.push_back(Code(UGSDR_GALILEO_E1B, sv, 1, q.job.block_samples, m, spm));
						q.sv.push_back(Sv{sv, System::Galileo, UGSDR_GALILEO_E1B});
					}
				out.push_back(std::move(q));
			}

			void Run(std::vector<Search>& searches, std::vector<AcquisitionResult<float>>& dst) {
				if (searches.empty())
					return;
				std::vector<ugsdr_acq_job> jobs;
				std::vector<std::vector<ugsdr_acq_result>> results(searches.size());
				std::vector<ugsdr_acq_result*> ptrs;
				for (std::size_t i = 0; i < searches.size(); ++i) {
					searches[i].job.codes = searches[i].codes.data();
					searches[i].job.n_codes = static_cast<int>(searches[i].codes.size());
					jobs.push_back(searches[i].job);
					results[i].resize(searches[i].codes.size());
					ptrs.push_back(results[i].data());
				}
				Check(ugsdr_acquire_batch(ctx_, jobs.data(), static_cast<int>(jobs.size()), ptrs.data()));
				for (std::size_t i = 0; i < searches.size(); ++i) {
					const Search& q = searches[i];
					const std::size_t per = q.galileo ? 4 : 1;
					for (std::size_t c = 0; c < q.codes.size(); c += per) {
						// the best permutation: std::max_element keeps the first maximum
						std::size_t best = c;
						for (std::size_t k = c + 1; k < c + per; ++k)
							if (results[i][best].level < results[i][k].level)
								best = k;
						const ugsdr_acq_result& r = results[i][best];
						AcquisitionResult<float> a;
						a.sv_number = q.sv[c];
						a.doppler = r.doppler;
						a.code_offset = r.code_offset;
						a.level = r.level;
						a.sigma = r.sigma;
						a.intermediate_frequency = q.job.intermediate_frequency;
						if (a.GetSnr() > peak_threshold)
							dst.push_back(std::move(a));
					}
				}
			}
		};
	}
}

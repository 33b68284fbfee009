// Tracking correlator bank: many channels, many 1 ms epochs, one launch.
//
// Per channel and epoch (Tracker::TrackSingleSatellite, src/tracking/
// tracker.hpp:156-177, with GetEpl 119-139):
//   1. carrier wipe-off: TableMixer arithmetic (64-entry LUT, non-contracted
//      complex<float> product, table_mixer.hpp:78-101) driven by a 64-bit NCO
//      whose phase is the channel's 64-bit fixed-point carrier phase;
//   2. five taps VE, E, P, L, VL, each CorrelateSplit (tracking_parameters.hpp:
//      472-493): the dot product of the epoch with the 3-period upsampled code
//      from index ceil(2 P - phase), split at sample ceil(phase) mod spm into
//      two sums combined by AddWithPhase (89-98);
//   3. Pll(prompt), Dll(early, late) in FP64 (495-528).
// One CTA owns one channel for the whole launch: all threads sweep the epoch's
// samples (coalesced; every channel reads the same epoch, so it stays in L2),
// each thread keeping an exact incremental code-chip index per tap (no
// per-sample division), then thread 0 runs the FP64 loop update.
#include "internal.hpp"
#include "acq_kernels.cuh"

#include <cmath>
#include <cstring>

namespace ugsdr_gpu {
	namespace {
		constexpr int kTrackThreads = 256;
		constexpr double kTwo64 = 18446744073709551616.0;
		constexpr double kPi = 3.14159265358979323846;

		struct TrackState {
			// static
			int code, len, period_ms, pad;
			double base;            // base code frequency
			// dynamic (FP64 loop state; carrier phase as cycles * 2^64)
			double code_phase, carrier_freq, carrier_phase_error, code_nco, code_error, code_freq;
			double prev_re, prev_im;
			unsigned long long phase_fx;
			long long epoch;
		};

		struct TrackOut {
			float taps[5][2];
			double carrier_frequency, carrier_phase, code_phase, code_frequency, phase_error, code_error;
		};
		static_assert(sizeof(TrackOut) == sizeof(ugsdr_track_output), "output layout");

		struct TrackParams {
			const void* samples;
			size_t spm;             // samples per epoch (fs / 1e3)
			int n_epochs;
			int n_channels;
			double fs;
			double offsets[5];      // chips: VE, E, P, L, VL
			double k1_pll, k2_pll, k3_pll, k1_dll, k2_dll;
			const float* chips;     // [code][len_max]
			int len_max;
			const float* lut;
			TrackState* states;
			TrackOut* out;          // [epoch][channel] or null
		};

		__device__ __forceinline__ unsigned long long frac_to_fx(double cycles) {
			double f = cycles - floor(cycles);
			double v = f * kTwo64;
			if (v >= kTwo64)
				v = 0.0;
			return static_cast<unsigned long long>(v);
		}

		// AddWithPhase (tracking_parameters.hpp:89-98)
		__device__ void add_with_phase(double lr, double li, double rr, double ri, double rel, double& o_re, double& o_im) {
			if (rel < 0.5) {
				double t = lr; lr = rr; rr = t;
				t = li; li = ri; ri = t;
			}
			const double wl = lr / rel;
			const double wr = rr / (1.0 - rel);
			if (fabs(wl + wr) > fabs(wl)) {
				o_re = lr + rr;
				o_im = li + ri;
			}
			else {
				o_re = lr - rr;
				o_im = li - ri;
			}
		}

		template <int ST>
		__global__ void __launch_bounds__(kTrackThreads) track_bank_kernel(TrackParams p) {
			extern __shared__ float s_chips[];
			__shared__ float s_lut[80];
			__shared__ float s_red[kTrackThreads / 32][20];
			__shared__ unsigned long long s_holder0, s_adder;
			__shared__ int s_mix;
			__shared__ unsigned long long s_first_phase[5];
			__shared__ int s_first_len[5];
			__shared__ double s_rel[5];

			TrackState* st = p.states + blockIdx.x;
			const int len = st->len;
			const float* chips = p.chips + static_cast<size_t>(st->code) * p.len_max;
			for (int i = threadIdx.x; i < len; i += blockDim.x)
				s_chips[i] = chips[i];
			if (threadIdx.x < 80)
				s_lut[threadIdx.x] = p.lut[threadIdx.x];

			const size_t spm = p.spm;
			const int period_ms = st->period_ms;
			const double period = static_cast<double>(spm) * period_ms;
			const unsigned long long L3 = 3ull * static_cast<unsigned long long>(len);
			const unsigned long long S3 = static_cast<unsigned long long>(3 * period_ms * p.fs / 1e3);
			// per-thread chip stride over blockDim samples: blockDim * L3 = dchip * S3 + drem
			const unsigned long long dnum = static_cast<unsigned long long>(blockDim.x) * L3;
			const int dchip = static_cast<int>((dnum / S3) % static_cast<unsigned long long>(len));
			const unsigned int drem = static_cast<unsigned int>(dnum % S3);
			const double spc = p.fs / st->base;
			__syncthreads();

			for (int ep = 0; ep < p.n_epochs; ++ep) {
				if (threadIdx.x == 0) {
					// GetEpl: Translate(signal, fs, -carrier_frequency, -carrier_phase)
					double f = -st->carrier_freq;
					s_mix = fabs(f) != 0.0;
					if (f < 0)
						f = p.fs + f;
					double av = kTwo64 * f / p.fs;
					if (av >= kTwo64)
						av = 0.0;
					s_adder = static_cast<unsigned long long>(av);
					s_holder0 = 0ull - st->phase_fx;
					const double ph = st->code_phase - p.fs / 1e3 * static_cast<double>(st->epoch % period_ms);
					for (int t = 0; t < 5; ++t) {
						double q = ph + spc * p.offsets[t];
						while (q < 0)
							q += period;
						if (q > period)
							q = fmod(q, period);
						s_first_len[t] = static_cast<int>(static_cast<unsigned long long>(ceil(q)) % spm);
						s_first_phase[t] = static_cast<unsigned long long>(ceil(2 * period - q));
						s_rel[t] = fmod(q, static_cast<double>(spm)) / static_cast<double>(spm);
					}
				}
				__syncthreads();
				// chip trackers: sample i uses full-code index q = first_phase + i,
				// chip = (q * L3 / S3) mod len, advanced exactly by (dchip, drem) per step
				int chip[5];
				unsigned int rem[5];
				int first_len[5];
				for (int t = 0; t < 5; ++t) {
					const unsigned long long num = (s_first_phase[t] + threadIdx.x) * L3;
					chip[t] = static_cast<int>((num / S3) % static_cast<unsigned long long>(len));
					rem[t] = static_cast<unsigned int>(num % S3);
					first_len[t] = s_first_len[t];
				}
				float acc[20];
#pragma unroll
				for (int k = 0; k < 20; ++k)
					acc[k] = 0.f;
				const unsigned long long adder = s_adder;
				unsigned long long holder = s_holder0 + static_cast<unsigned long long>(threadIdx.x) * adder;
				const unsigned long long hstep = static_cast<unsigned long long>(blockDim.x) * adder;
				const bool mix = s_mix;
				const size_t base = static_cast<size_t>(ep) * spm;
				for (int i = threadIdx.x; i < static_cast<int>(spm); i += blockDim.x) {
					float2 x = load_sample<ST>(p.samples, base + i);
					if (mix) {
						const uint32_t idx = static_cast<uint32_t>(holder >> 58);
						const float c = s_lut[idx + 16], s = s_lut[idx];
						x = c2(__fsub_rn(__fmul_rn(x.x, c), __fmul_rn(x.y, s)), __fadd_rn(__fmul_rn(x.x, s), __fmul_rn(x.y, c)));
					}
					holder += hstep;
#pragma unroll
					for (int t = 0; t < 5; ++t) {
						const float cv = s_chips[chip[t]];
						const int slot = 4 * t + (i < first_len[t] ? 0 : 2);
						acc[slot] += x.x * cv;
						acc[slot + 1] += x.y * cv;
						rem[t] += drem;
						int adv = dchip;
						if (rem[t] >= S3) {
							rem[t] -= static_cast<unsigned int>(S3);
							++adv;
						}
						chip[t] += adv;
						if (chip[t] >= len)
							chip[t] -= len;
					}
				}
				// block reduction of the 20 partial sums
#pragma unroll
				for (int k = 0; k < 20; ++k) {
					float v = acc[k];
					for (int o = 16; o > 0; o >>= 1)
						v += __shfl_down_sync(0xffffffffu, v, o);
					if ((threadIdx.x & 31) == 0)
						s_red[threadIdx.x >> 5][k] = v;
				}
				__syncthreads();
				if (threadIdx.x == 0) {
					double sums[20];
					for (int k = 0; k < 20; ++k) {
						double v = 0;
						for (int w = 0; w < static_cast<int>(blockDim.x / 32); ++w)
							v += s_red[w][k];
						sums[k] = v;
					}
					double tap_re[5], tap_im[5];
					for (int t = 0; t < 5; ++t)
						add_with_phase(sums[4 * t], sums[4 * t + 1], sums[4 * t + 2], sums[4 * t + 3], s_rel[t], tap_re[t], tap_im[t]);
					// UpdatePhase (tracking_parameters.hpp:163-165) with the pre-update frequency
					st->phase_fx += frac_to_fx(st->carrier_freq / 1000.0);
					// Pll(prompt) (tracking_parameters.hpp:495-511)
					const double pr = static_cast<float>(tap_re[2]), pi = static_cast<float>(tap_im[2]);
					const double err = pr != 0.0 ? atan(pi / pr) / (kPi * 2.0) : 0.0;
					const double cross = pr * st->prev_im - st->prev_re * pi;
					const double dot = fabs(pr * st->prev_re + st->prev_im * pi);
					const double ferr = atan2(cross, dot) / kPi;
					st->carrier_freq += p.k1_pll * err - p.k2_pll * st->carrier_phase_error - p.k3_pll * ferr;
					st->carrier_phase_error = err;
					st->phase_fx += static_cast<unsigned long long>(llrint(err / 4.0 * kTwo64));
					st->prev_re = pr;
					st->prev_im = pi;
					// Dll(early, late) (tracking_parameters.hpp:513-528)
					const double er = static_cast<float>(tap_re[1]), ei = static_cast<float>(tap_im[1]);
					const double lr = static_cast<float>(tap_re[3]), li = static_cast<float>(tap_im[3]);
					const double ea = hypot(er, ei), la = hypot(lr, li);
					double ce = 0.0;
					if (ea + la != 0)
						ce = (ea - la) / (ea + la);
					st->code_nco += (p.k1_dll * (ce - st->code_error) + p.k2_dll * ce) * (st->base / 1.023e6);
					st->code_error = ce;
					st->code_freq = st->base - st->code_nco;
					st->code_phase -= p.fs / 1000 / 2 * (st->code_freq / st->base - 1);
					if (p.out) {
						TrackOut o;
						for (int t = 0; t < 5; ++t) {
							o.taps[t][0] = static_cast<float>(tap_re[t]);
							o.taps[t][1] = static_cast<float>(tap_im[t]);
						}
						o.carrier_frequency = st->carrier_freq;
						o.carrier_phase = static_cast<double>(st->phase_fx) / kTwo64 * 2 * kPi;
						o.code_phase = st->code_phase;
						o.code_frequency = st->code_freq;
						o.phase_error = err;
						o.code_error = ce;
						p.out[static_cast<size_t>(ep) * p.n_channels + blockIdx.x] = o;
					}
					++st->epoch;
				}
				__syncthreads();
			}
		}
	}
}

using namespace ugsdr_gpu;

struct ugsdr_track_bank {
	ugsdr_ctx* ctx = nullptr;
	int n_channels = 0;
	int len_max = 0;
	double fs = 0;
	size_t spm = 0;
	double offsets[5] = {};
	double k1_pll = 0, k2_pll = 0, k3_pll = 0, k1_dll = 0, k2_dll = 0;
	DevBuf chips, states, samples, out;
};

extern "C" {

int ugsdr_track_create(ugsdr_ctx* ctx, const ugsdr_track_config* cfg, const ugsdr_track_channel* channels, int n_channels,
	const float* codes, const int* code_lens, int n_codes, int code_len_max, ugsdr_track_bank** bank) {
	if (!ctx || !bank)
		return UGSDR_E_INVALID;
	*bank = nullptr;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		require(cfg && channels && codes && code_lens && n_channels > 0 && n_codes > 0 && code_len_max > 0, "null or empty bank description");
		require(std::fabs(cfg->integration_time - 1e-3) < 1e-12, "integration_time must be 0.001 s (one epoch)");
		require(code_len_max * sizeof(float) <= 48 * 1024, "codes longer than 12288 chips are not supported");
		auto b = std::make_unique<ugsdr_track_bank>();
		b->ctx = ctx;
		b->n_channels = n_channels;
		b->len_max = code_len_max;
		b->fs = channels[0].sampling_rate;
		require(b->fs > 0 && std::fmod(b->fs, 1e3) == 0.0, "sampling rate must be a whole number of kHz");
		b->spm = static_cast<size_t>(b->fs / 1e3);
		const double el = cfg->early_late_spacing, vel = cfg->very_early_late_spacing;
		const double offs[5] = {vel, el, 0.0, -el, -vel};
		std::memcpy(b->offsets, offs, sizeof(offs));
		// loop constants (tracking_parameters.hpp:72-87), bandwidths as parameters
		const double T = cfg->integration_time;
		const double bp = cfg->pll_bandwidth, bf = cfg->fll_bandwidth, bd = cfg->dll_bandwidth;
		b->k1_pll = T * (bp / 0.53 * (bp / 0.53)) + 1.414 * (bp / 0.53);
		b->k2_pll = 1.414 * (bp / 0.53);
		b->k3_pll = T * (bf / 0.25);
		const double zeta = 1.0, gain = 0.1;
		const double wn = bd * 8.0 * zeta / (4.0 * zeta * zeta + 1.0);
		require(wn > 0, "dll_bandwidth must be positive");
		const double tau1 = gain / (wn * wn), tau2 = 2.0 * zeta / wn;
		b->k1_dll = tau2 / tau1;
		b->k2_dll = T / tau1;

		std::vector<TrackState> st(n_channels);
		for (int c = 0; c < n_channels; ++c) {
			const auto& ch = channels[c];
			require(ch.code >= 0 && ch.code < n_codes, "channel code index out of range");
			require(ch.sampling_rate == b->fs, "all channels of a bank share one sampling rate");
			require(ch.code_frequency > 0 && ch.code_length > 0 && ch.code_frequency < b->fs, "bad code rate");
			const int len = code_lens[ch.code];
			require(len > 0 && len <= code_len_max && static_cast<double>(len) == ch.code_length, "code length mismatch");
			const double period = ch.code_length / ch.code_frequency * 1000.0;
			const int period_ms = static_cast<int>(std::lround(period));
			require(period_ms >= 1 && std::fabs(period - period_ms) < 1e-9, "code period must be a whole number of ms");
			TrackState s{};
			s.code = ch.code;
			s.len = len;
			s.period_ms = period_ms;
			s.base = ch.code_frequency;
			s.code_phase = ch.code_phase;
			s.carrier_freq = ch.carrier_frequency;
			s.code_freq = ch.code_frequency;
			const double cyc = ch.carrier_phase / (2 * kPi);
			double fr = (cyc - std::floor(cyc)) * kTwo64;
			s.phase_fx = fr >= kTwo64 ? 0ull : static_cast<unsigned long long>(fr);
			st[c] = s;
		}
		b->chips.reserve(sizeof(float) * static_cast<size_t>(n_codes) * code_len_max);
		b->states.reserve(sizeof(TrackState) * n_channels);
		UG_CUDA(cudaMemcpy(b->chips.ptr, codes, sizeof(float) * static_cast<size_t>(n_codes) * code_len_max, cudaMemcpyHostToDevice));
		UG_CUDA(cudaMemcpy(b->states.ptr, st.data(), sizeof(TrackState) * n_channels, cudaMemcpyHostToDevice));
		*bank = b.release();
	});
}

int ugsdr_track_run(ugsdr_track_bank* bank, const void* samples, int sample_type, int samples_on_device, size_t samples_per_epoch,
	int n_epochs, ugsdr_track_output* outputs) {
	if (!bank)
		return UGSDR_E_INVALID;
	ugsdr_ctx* ctx = bank->ctx;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		require(samples && n_epochs > 0, "null samples or no epochs");
		require(samples_per_epoch == bank->spm, "samples_per_epoch must be sampling_rate / 1000");
		require(sample_type >= 0 && sample_type <= 3, "unknown sample type");
		const size_t per = sample_type == UGSDR_SAMPLES_CF32 ? 8 : sample_type == UGSDR_SAMPLES_CI8 ? 2 : sample_type == UGSDR_SAMPLES_CI16 ? 4 : 1;
		const size_t n = bank->spm * static_cast<size_t>(n_epochs);
		const void* dev = samples;
		if (!samples_on_device) {
			bank->samples.reserve(per * n);
			UG_CUDA(cudaMemcpyAsync(bank->samples.ptr, samples, per * n, cudaMemcpyHostToDevice, ctx->stream));
			dev = bank->samples.ptr;
		}
		TrackParams p{};
		p.samples = dev;
		p.spm = bank->spm;
		p.n_epochs = n_epochs;
		p.n_channels = bank->n_channels;
		p.fs = bank->fs;
		std::memcpy(p.offsets, bank->offsets, sizeof(p.offsets));
		p.k1_pll = bank->k1_pll;
		p.k2_pll = bank->k2_pll;
		p.k3_pll = bank->k3_pll;
		p.k1_dll = bank->k1_dll;
		p.k2_dll = bank->k2_dll;
		p.chips = bank->chips.as<float>();
		p.len_max = bank->len_max;
		p.lut = get_lut(ctx);
		p.states = bank->states.as<TrackState>();
		if (outputs) {
			bank->out.reserve(sizeof(TrackOut) * static_cast<size_t>(n_epochs) * bank->n_channels);
			p.out = bank->out.as<TrackOut>();
		}
		const size_t smem = sizeof(float) * bank->len_max;
		{
			KernelTimer timer(ctx, "track_bank");
			switch (sample_type) {
			case UGSDR_SAMPLES_CF32:
				track_bank_kernel<UGSDR_SAMPLES_CF32><<<bank->n_channels, kTrackThreads, smem, ctx->stream>>>(p);
				break;
			case UGSDR_SAMPLES_CI8:
				track_bank_kernel<UGSDR_SAMPLES_CI8><<<bank->n_channels, kTrackThreads, smem, ctx->stream>>>(p);
				break;
			case UGSDR_SAMPLES_CI16:
				track_bank_kernel<UGSDR_SAMPLES_CI16><<<bank->n_channels, kTrackThreads, smem, ctx->stream>>>(p);
				break;
			default:
				track_bank_kernel<UGSDR_SAMPLES_RI8><<<bank->n_channels, kTrackThreads, smem, ctx->stream>>>(p);
				break;
			}
		}
		note_launch(ctx);
		if (outputs)
			UG_CUDA(cudaMemcpyAsync(outputs, p.out, sizeof(TrackOut) * static_cast<size_t>(n_epochs) * bank->n_channels,
				cudaMemcpyDeviceToHost, ctx->stream));
		UG_CUDA(cudaStreamSynchronize(ctx->stream));
	});
}

int ugsdr_track_destroy(ugsdr_track_bank* bank) {
	if (!bank)
		return UGSDR_E_INVALID;
	{
		std::lock_guard<std::mutex> lock(bank->ctx->mutex);
		cudaStreamSynchronize(bank->ctx->stream);
	}
	delete bank;
	return UGSDR_OK;
}
}

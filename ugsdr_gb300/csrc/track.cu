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
#include "packed.cuh"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <type_traits>
#include <vector>

namespace ugsdr_gpu {
	namespace {
		constexpr int kTrackThreads = 256;
		constexpr int kWinChunk = 4096;   // samples per chunk at most (a multiple of 4 x kTrackThreads)
		constexpr int kWinPad = 128;      // window margin: taps within +-kWinPad samples of the prompt
		constexpr int kWinFloats = kWinChunk + 2 * kWinPad + 8;  // one window: margins + 16-byte rounding
		constexpr int kCopyChunkEpochs = 1000;  // host-buffer runs: epochs per overlapped copy
		constexpr int kStageBytes = 16384;  // one staged sample chunk (two buffers, double-buffered)
		constexpr double kMaxRate = 131.072e6;  // 32 chunks of 4096 samples per epoch

		template <int ST>
		constexpr int sample_size() {
			return ST == UGSDR_SAMPLES_CF32 ? 8 : ST == UGSDR_SAMPLES_CI16 ? 4 : ST == UGSDR_SAMPLES_CI8 ? 2 : 1;
		}
		// samples per chunk: the window's 4096, or fewer so a chunk fits one stage buffer
		template <int ST>
		constexpr int chunk_samples() {
			return kStageBytes / sample_size<ST>() < kWinChunk ? kStageBytes / sample_size<ST>() : kWinChunk;
		}

		template <int G>
		__device__ __forceinline__ void cp_async_g(void* smem, const void* gmem) {
			const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(smem));
			asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(gmem), "n"(G));
		}
		__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
		__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }
		constexpr double kTwo64 = 18446744073709551616.0;
		constexpr double kPi = 3.14159265358979323846;

		struct TrackState {
			// static
			int code, len, period_ms, pad;
			long long rep;          // the channel's replica table: offset in floats
			double base;            // base code frequency
			// dynamic (FP64 loop state; carrier phase as cycles * 2^64)
			double code_phase, carrier_freq, carrier_phase_error, code_nco, code_error, code_freq;
			double prev_re, prev_im;
			unsigned long long phase_fx;
			long long epoch;
			double phase_rad;       // nco_mode 1: the reference's carrier phase, rad
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
			const float* replicas;  // replica tables (TrackState::rep)
			const float* lut;
			TrackState* states;
			TrackOut* out;          // [epoch][channel] or null
			int stage_g;            // cp.async size (16/8/4) when staged: it divides the epoch and chunk byte offsets and the base alignment
			int nco_mode;           // 0: 64-bit fixed-point carrier NCO; 1: the reference's per-epoch TableMixer NCO
		};

		__device__ __forceinline__ unsigned long long frac_to_fx(double cycles) {
			double f = cycles - floor(cycles);
			double v = f * kTwo64;
			if (v >= kTwo64)
				v = 0.0;
			return static_cast<unsigned long long>(v);
		}

		// Loop state of one channel, held in registers of warp 0's lane 0 for the
		// whole launch (loaded from / stored back to TrackState).
		struct LoopState {
			double code_phase, carrier_freq, carrier_phase_error, code_nco, code_error, code_freq;
			float prev_re, prev_im;
			unsigned long long phase_fx;
			long long epoch;
			double phase_rad;
		};

		// q - floor(q / m) m for q >= 0 and integer m, by a reciprocal and an
		// exact correction: equals fmod(q, m).
		__device__ __forceinline__ double mod_pos(double q, double m, double inv_m) {
			double r = q - floor(q * inv_m) * m;
			if (r < 0)
				r += m;
			else if (r >= m)
				r -= m;
			return r;
		}

		// correlation of four samples per thread: every tap's sample on the left
		// of its CorrelateSplit split (kLeft), every one on the right (kRight), or
		// per tap and with the chunk's bounds checked (kMixed)
		enum { kLeft = 0, kRight = 1, kMixed = 2 };

		template <int ST, bool STAGED>
		__global__ void __launch_bounds__(kTrackThreads, 2) track_bank_kernel(TrackParams p) {
			// The epoch is correlated in chunks of CH samples.  Chunk k's replica
			// window is one contiguous slice of the channel's replica table (the
			// code over three periods at the sampling rate, kWinPad samples of
			// margin on each side), copied by cp.async into one of two shared
			// windows one chunk ahead; every tap reads it at its own offset.
			// STAGED: the chunk's samples are copied the same way into one of two
			// stage buffers — the samples do not depend on the loop state, so they
			// run one chunk ahead across epochs too, while the first window of an
			// epoch waits for the loop update that places it.
			constexpr int CH = chunk_samples<ST>();
			constexpr int SB = sample_size<ST>();
			extern __shared__ __align__(16) unsigned char s_dyn[];  // 2 windows, then (STAGED) 2 stage buffers
			float* const s_win = reinterpret_cast<float*>(s_dyn);
			unsigned char* const s_stage = s_dyn + 2 * kWinFloats * sizeof(float);
			__shared__ float s_lut[80];
			__shared__ float s_red[kTrackThreads / 32][20];
			__shared__ float s_sum[20];
			__shared__ unsigned long long s_holder0, s_adder;
			__shared__ int s_mix;
			__shared__ int s_first_len[5], s_off[5], s_split_lo, s_split_hi;
			__shared__ double s_rel[5];
			__shared__ long long s_wstart;  // replica-table index of chunk 0's window

			TrackState* st = p.states + blockIdx.x;
			const float* rep = p.replicas + st->rep;
			for (int i = threadIdx.x; i < 80; i += blockDim.x)
				s_lut[i] = p.lut[i];

			const int spm = static_cast<int>(p.spm);
			const int period_ms = st->period_ms;
			const double period = static_cast<double>(spm) * period_ms;
			const double inv_period = 1.0 / period, inv_spm = 1.0 / static_cast<double>(spm);
			const long long P = static_cast<long long>(spm) * period_ms;
			const int n_chunks = (spm + CH - 1) / CH;
			const double spc = p.fs / st->base;
			const double base_freq = st->base, inv_base = 1.0 / st->base, dll_scale = st->base / 1.023e6;
			// the loop update's constant quotients, formed once (the same values
			// the reference's expressions give): FP64 divisions are the slowest
			// operations of the per-epoch serial update on warp 0
			const double fs_ms = p.fs / 1e3, half_fs_ms = p.fs / 1000 / 2, two64_over_fs = kTwo64 / p.fs;
			const int lane = threadIdx.x & 31;
			// epoch % period_ms of the next tap set-up, advanced by one per epoch
			// (no 64-bit modulo on the serial path)
			int ep_mod = static_cast<int>(st->epoch % period_ms);
			const bool warp0 = threadIdx.x < 32;

			LoopState ls{};
			if (threadIdx.x == 0)
				ls = LoopState{st->code_phase, st->carrier_freq, st->carrier_phase_error, st->code_nco, st->code_error,
					st->code_freq, static_cast<float>(st->prev_re), static_cast<float>(st->prev_im), st->phase_fx, st->epoch,
					st->phase_rad};

			// carrier NCO of GetEpl's Translate(signal, fs, -f, -phase), lane 0
			auto nco_setup = [&](bool first) {
				double f = -ls.carrier_freq;
				s_mix = fabs(f) != 0.0;
				if (f < 0)
					f = p.fs + f;
				if (p.nco_mode == 1) {
					// Mixer::Translate's NCO (mixer.hpp:21-42, nco.hpp:17-20): phase
					// reduced to [0, 2 pi), 32-bit holder and adder; carried in the
					// upper half of the 64-bit accumulator, whose top 6 bits are then
					// the 32-bit NCO's index and whose wrap is its wrap
					double ph = fmod(-ls.phase_rad, 2 * kPi);
					if (ph < 0)
						ph = __dadd_rn(ph, 2 * kPi);
					const unsigned long long a32 = static_cast<unsigned long long>(__ddiv_rn(__dmul_rn(4294967296.0, f), p.fs));
					const unsigned long long h32 =
						static_cast<unsigned long long>(__ddiv_rn(__dmul_rn(4294967296.0, ph), 2 * kPi)) & 0xFFFFFFFFull;
					s_adder = a32 << 32;
					s_holder0 = h32 << 32;
					return;
				}
				// the increment in NumericallyControlledOscillator's order (2^64 f) / fs
				// (nco.hpp:17-20) for the channel's starting frequency, so a sample
				// whose phase lands exactly on a LUT boundary (a rational f / fs, as
				// a caller's round starting Doppler gives) picks the same entry as the
				// host restatement; after a loop update (f from the FP64 filter) as
				// f times the quotient 2^64 / fs formed once per launch
				double av = first ? kTwo64 * f / p.fs : f * two64_over_fs;
				if (av >= kTwo64)
					av = 0.0;
				s_adder = static_cast<unsigned long long>(av);
				s_holder0 = 0ull - ls.phase_fx;
			};
			// CorrelateSplit set-up of the five taps from the code phase, lanes 0-4
			// of warp 0 (one tap each): split point, weight, replica offset.
			auto tap_setup = [&]() {
				const double code_phase = __shfl_sync(0xffffffffu, ls.code_phase, 0);
				long long fp = 0;
				int fl = 0;
				if (lane < 5) {
					const double ph = code_phase - fs_ms * static_cast<double>(ep_mod);
					double q = ph + spc * p.offsets[lane];
					while (q < 0)
						q += period;
					if (q > period)
						q = mod_pos(q, period, inv_period);
					fl = static_cast<int>(static_cast<unsigned int>(ceil(q)) % static_cast<unsigned int>(spm));
					s_first_len[lane] = fl;
					fp = static_cast<long long>(ceil(2 * period - q));
					s_rel[lane] = mod_pos(q, static_cast<double>(spm), inv_spm) * inv_spm;
				}
				const long long fp2 = __shfl_sync(0xffffffffu, fp, 2);
				// the taps' split points span [lo, hi): outside it every tap is on one side
				int lo = lane < 5 ? fl : spm, hi = lane < 5 ? fl : 0;
#pragma unroll
				for (int o = 4; o > 0; o >>= 1) {
					lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
					hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
				}
				if (lane < 5) {
					long long d = fp - fp2;  // reduced to the prompt's code period
					while (d > P / 2)
						d -= P;
					while (d <= -P / 2)
						d += P;
					s_off[lane] = static_cast<int>(d) + kWinPad;
					if (lane == 2) {
						// window entry j of the chunk at c0 is full-code index
						// fp2 - kWinPad + c0 + j, replica-table index fp2 + c0 + j
						s_wstart = fp2;
						s_split_lo = lo;
						s_split_hi = hi;
					}
				}
			};
			// chunk k's window (n_c + 2 kWinPad entries from table index x0) into
			// window buf: 16-byte copies from x0 rounded down to 4 entries (the
			// table is padded for the rounded-up end)
			auto fetch_window = [&](int buf, long long x0, int n_c) {
				const long long a0 = x0 & ~3ll;
				const int n_copy = (static_cast<int>(x0 - a0) + n_c + 2 * kWinPad + 3) & ~3;
				float* dst = s_win + buf * kWinFloats;
				const float* src = rep + a0;
				for (int o = 4 * threadIdx.x; o < n_copy; o += 4 * blockDim.x)
					cp_async_g<16>(dst + o, src + o);
			};
			// samples of global chunk gi = epoch * n_chunks + chunk into stage buffer gi & 1
			const int total_chunks = p.n_epochs * n_chunks;
			auto stage = [&](int gi) {
				const int e = gi / n_chunks;
				const int c = (gi - e * n_chunks) * CH;
				const int bytes = min(CH, spm - c) * SB;
				const char* src = static_cast<const char*>(p.samples) + (static_cast<size_t>(e) * spm + c) * SB;
				unsigned char* dst = s_stage + (gi & 1) * kStageBytes;
				if (p.stage_g == 16) {
					for (int o = threadIdx.x * 16; o < bytes; o += blockDim.x * 16)
						cp_async_g<16>(dst + o, src + o);
				}
				else if (p.stage_g == 8) {
					for (int o = threadIdx.x * 8; o < bytes; o += blockDim.x * 8)
						cp_async_g<8>(dst + o, src + o);
				}
				else {
					for (int o = threadIdx.x * 4; o < bytes; o += blockDim.x * 4)
						cp_async_g<4>(dst + o, src + o);
				}
			};
			if (warp0) {
				if (lane == 0)
					nco_setup(ls.epoch == 0);  // the channel's first epoch (not every launch: runs split differently agree)
				tap_setup();
			}
			if constexpr (STAGED)
				stage(0);
			__syncthreads();  // s_wstart of epoch 0
			fetch_window(0, s_wstart, min(CH, spm));
			cp_async_commit();

			for (int ep = 0; ep < p.n_epochs; ++ep) {
				int off[5];
#pragma unroll
				for (int t = 0; t < 5; ++t)
					off[t] = s_off[t];
				const long long wstart = s_wstart;
				const int split_lo = s_split_lo, split_hi = s_split_hi;
				float acc[20];
#pragma unroll
				for (int k = 0; k < 20; ++k)
					acc[k] = 0.f;
				const unsigned long long adder = s_adder;
				unsigned long long holder = s_holder0 + static_cast<unsigned long long>(threadIdx.x) * adder;
				const unsigned long long hstep = static_cast<unsigned long long>(blockDim.x) * adder;
				const bool mix = s_mix;
				const size_t base = static_cast<size_t>(ep) * spm;
				for (int k = 0; k < n_chunks; ++k) {
					const int c0 = k * CH;
					const int n_c = min(CH, spm - c0);
					const int gi = ep * n_chunks + k;
					cp_async_wait_all();  // this chunk's window and samples (issued one chunk earlier)
					__syncthreads();      // ... for every thread; the other buffers were last read by chunk gi - 1
					if (k + 1 < n_chunks) {
						fetch_window((gi + 1) & 1, wstart + c0 + CH, min(CH, spm - c0 - CH));
						if constexpr (STAGED)
							stage(gi + 1);
						cp_async_commit();
					}
					else if (STAGED && gi + 1 < total_chunks) {
						stage(gi + 1);  // the next epoch's first samples; its window follows the loop update
						cp_async_commit();
					}
					const void* stage_buf = s_stage + (gi & 1) * kStageBytes;
					const float* win = s_win + (gi & 1) * kWinFloats + static_cast<int>((wstart + c0) & 3ll);
					const int lo = split_lo - c0, hi = split_hi - c0;  // chunk-relative split span
					auto correlate4 = [&](int i0, auto mode_tag) {
						constexpr int MODE = decltype(mode_tag)::value;
						float2 xs[4];
#pragma unroll
						for (int u = 0; u < 4; ++u) {
							const int i = i0 + u * kTrackThreads;
							if (MODE == kMixed && i >= n_c) {
								xs[u] = c2(0.f, 0.f);
								continue;
							}
							if constexpr (STAGED)
								xs[u] = load_sample<ST>(stage_buf, i);
							else
								xs[u] = load_sample<ST>(p.samples, base + c0 + i);
						}
#pragma unroll
						for (int u = 0; u < 4; ++u) {
							const int i = i0 + u * kTrackThreads;
							if (MODE == kMixed && i >= n_c)
								break;
							float2 x = xs[u];
							if (mix) {
								const uint32_t idx = static_cast<uint32_t>(holder >> 58);
								const float c = s_lut[idx + 16], s = s_lut[idx];
								x = c2(__fsub_rn(__fmul_rn(x.x, c), __fmul_rn(x.y, s)), __fadd_rn(__fmul_rn(x.x, s), __fmul_rn(x.y, c)));
							}
							holder += hstep;
#pragma unroll
							for (int t = 0; t < 5; ++t) {
								const float cv = win[i + off[t]];
								// the two CorrelateSplit partial sums
								bool left = MODE == kLeft;
								if constexpr (MODE == kMixed)
									left = c0 + i < s_first_len[t];
								if (left) {
									acc[4 * t] += x.x * cv;
									acc[4 * t + 1] += x.y * cv;
								}
								else {
									acc[4 * t + 2] += x.x * cv;
									acc[4 * t + 3] += x.y * cv;
								}
							}
						}
					};
					for (int i0 = threadIdx.x; i0 < n_c; i0 += 4 * kTrackThreads) {
						const int i3 = i0 + 3 * kTrackThreads;  // the thread's last sample of the four
						if (i3 < n_c && i3 < lo)
							correlate4(i0, std::integral_constant<int, kLeft>{});
						else if (i3 < n_c && i0 >= hi)
							correlate4(i0, std::integral_constant<int, kRight>{});
						else
							correlate4(i0, std::integral_constant<int, kMixed>{});
					}
				}
				// block reduction of the 20 partial sums
#pragma unroll
				for (int k = 0; k < 20; ++k) {
					float v = acc[k];
#pragma unroll
					for (int o = 16; o > 0; o >>= 1)
						v += __shfl_down_sync(0xffffffffu, v, o);
					if (lane == 0)
						s_red[threadIdx.x >> 5][k] = v;
				}
				__syncthreads();
				if (warp0) {
					if (lane < 20) {
						float v = 0.f;
						for (int w = 0; w < kTrackThreads / 32; ++w)
							v += s_red[w][lane];
						s_sum[lane] = v;
					}
					__syncwarp();
					// AddWithPhase per tap (lanes 0-4): the reference's comparison
					// |l / rel + r / (1 - rel)| > |l / rel| multiplied through by
					// rel (1 - rel) > 0; taps rounded to float as the reference's
					float tap_re = 0.f, tap_im = 0.f;
					if (lane < 5) {
						float lr = s_sum[4 * lane], li = s_sum[4 * lane + 1], rr = s_sum[4 * lane + 2], ri = s_sum[4 * lane + 3];
						const double rel = s_rel[lane];
						if (rel < 0.5) {
							float t0 = lr; lr = rr; rr = t0;
							t0 = li; li = ri; ri = t0;
						}
						const double a = static_cast<double>(lr) * (1.0 - rel);
						const bool plus = fabs(a + static_cast<double>(rr) * rel) > fabs(a);
						// lhs +- rhs of complex<float>: float sums, as the reference adds
						tap_re = plus ? __fadd_rn(lr, rr) : __fsub_rn(lr, rr);
						tap_im = plus ? __fadd_rn(li, ri) : __fsub_rn(li, ri);
					}
					float taps_re[5], taps_im[5];
#pragma unroll
					for (int t = 0; t < 5; ++t) {
						taps_re[t] = __shfl_sync(0xffffffffu, tap_re, t);
						taps_im[t] = __shfl_sync(0xffffffffu, tap_im, t);
					}
					const float pr = taps_re[2], pi = taps_im[2];
					const float ppr = __shfl_sync(0xffffffffu, ls.prev_re, 0), ppi = __shfl_sync(0xffffffffu, ls.prev_im, 0);
					// discriminators in the reference's float types, side by side:
					// lane 0 PLL atan(imag / real), 1 FLL atan2(cross, dot), 2 |E|, 3 |L|
					float part = 0.f;
					double part_d = 0.0;  // nco_mode 1: the reference's double atan of the float ratio
					if (lane == 0) {
						if (p.nco_mode == 1)
							part_d = pr != 0.f ? atan(static_cast<double>(__fdiv_rn(pi, pr))) : 0.0;
						else
							part = pr != 0.f ? atanf(__fdiv_rn(pi, pr)) : 0.f;
					}
					else if (lane == 1) {
						const float cross = __fsub_rn(__fmul_rn(pr, ppi), __fmul_rn(ppr, pi));
						const float dot = fabsf(__fadd_rn(__fmul_rn(pr, ppr), __fmul_rn(ppi, pi)));
						part = atan2f(cross, dot);
					}
					else if (lane == 2) {
						part = hypotf(taps_re[1], taps_im[1]);
					}
					else if (lane == 3) {
						part = hypotf(taps_re[3], taps_im[3]);
					}
					const float ferr_f = __shfl_sync(0xffffffffu, part, 1);
					const float ea = __shfl_sync(0xffffffffu, part, 2);
					const float la = __shfl_sync(0xffffffffu, part, 3);
					if (lane == 0) {
						// the reference divides by 2 pi and pi (nco_mode 1 keeps the
						// quotients); the 64-bit NCO mode multiplies by the reciprocals
						const double err = p.nco_mode == 1 ? part_d / (kPi * 2.0) : static_cast<double>(part) * (0.5 / kPi);
						const double ferr = p.nco_mode == 1 ? static_cast<double>(ferr_f) / kPi : static_cast<double>(ferr_f) * (1.0 / kPi);
						// UpdatePhase (tracking_parameters.hpp:163-165) with the pre-update frequency
						ls.phase_fx += frac_to_fx(ls.carrier_freq * 1e-3);
						if (p.nco_mode == 1)  // the radian phase: the reference NCO mode's carrier phase
							ls.phase_rad = __dadd_rn(ls.phase_rad, __ddiv_rn(__dmul_rn(2 * kPi, ls.carrier_freq), 1000.0));
						// Pll(prompt) (tracking_parameters.hpp:495-511), loop filter in FP64
						// in the reference's operation order, nothing contracted
						ls.carrier_freq = __dadd_rn(ls.carrier_freq, __dsub_rn(__dsub_rn(__dmul_rn(p.k1_pll, err),
							__dmul_rn(p.k2_pll, ls.carrier_phase_error)), __dmul_rn(p.k3_pll, ferr)));
						ls.carrier_phase_error = err;
						ls.phase_fx += static_cast<unsigned long long>(llrint(err * (kTwo64 / 4.0)));
						if (p.nco_mode == 1)
							ls.phase_rad = __dadd_rn(ls.phase_rad, __ddiv_rn(__dmul_rn(err, kPi), 2.0));
						ls.prev_re = pr;
						ls.prev_im = pi;
						// Dll(early, late) (tracking_parameters.hpp:513-528)
						double ce = 0.0;
						if (ea + la != 0.f)
							ce = __fdiv_rn(__fsub_rn(ea, la), __fadd_rn(ea, la));
						ls.code_nco = __dadd_rn(ls.code_nco, __dmul_rn(__dadd_rn(__dmul_rn(p.k1_dll, __dsub_rn(ce, ls.code_error)),
							__dmul_rn(p.k2_dll, ce)), dll_scale));
						ls.code_error = ce;
						ls.code_freq = __dsub_rn(base_freq, ls.code_nco);
						// code_freq / base as the reference divides it (nco_mode 1), by the
						// reciprocal otherwise (one FP64 division less on the epoch's serial path)
						const double ratio = p.nco_mode == 1 ? __ddiv_rn(ls.code_freq, base_freq) : __dmul_rn(ls.code_freq, inv_base);
						ls.code_phase = __dsub_rn(ls.code_phase, __dmul_rn(half_fs_ms, __dsub_rn(ratio, 1.0)));
						if (p.out) {
							TrackOut o;
							for (int t = 0; t < 5; ++t) {
								o.taps[t][0] = taps_re[t];
								o.taps[t][1] = taps_im[t];
							}
							o.carrier_frequency = ls.carrier_freq;
							o.carrier_phase = p.nco_mode == 1 ? ls.phase_rad : static_cast<double>(ls.phase_fx) / kTwo64 * 2 * kPi;
							o.code_phase = ls.code_phase;
							o.code_frequency = ls.code_freq;
							o.phase_error = err;
							o.code_error = ce;
							p.out[static_cast<size_t>(ep) * p.n_channels + blockIdx.x] = o;
						}
						++ls.epoch;
						nco_setup(false);
					}
					__syncwarp();
					ep_mod = ep_mod + 1 == period_ms ? 0 : ep_mod + 1;
					if (ep + 1 < p.n_epochs)
						tap_setup();
				}
				__syncthreads();  // the next epoch's NCO and taps
				if (ep + 1 < p.n_epochs) {
					fetch_window(((ep + 1) * n_chunks) & 1, s_wstart, min(CH, spm));
					cp_async_commit();
				}
			}
			if (threadIdx.x == 0) {
				st->code_phase = ls.code_phase;
				st->carrier_freq = ls.carrier_freq;
				st->carrier_phase_error = ls.carrier_phase_error;
				st->code_nco = ls.code_nco;
				st->code_error = ls.code_error;
				st->code_freq = ls.code_freq;
				st->prev_re = ls.prev_re;
				st->prev_im = ls.prev_im;
				st->phase_fx = ls.phase_fx;
				st->epoch = ls.epoch;
			}
		}
	}
}

using namespace ugsdr_gpu;

struct ugsdr_track_bank {
	ugsdr_ctx* ctx = nullptr;
	int n_channels = 0;
	double fs = 0;
	size_t spm = 0;
	double offsets[5] = {};
	double k1_pll = 0, k2_pll = 0, k3_pll = 0, k1_dll = 0, k2_dll = 0;
	int nco_mode = 0;
	DevBuf replicas, states;
};

namespace {
	// Enqueues n_epochs of the bank on the context stream; `dev_out` (device,
	// or null) receives n_epochs x n_channels outputs.
	void track_enqueue(ugsdr_track_bank* bank, const void* samples, int sample_type, int samples_on_device,
		size_t samples_per_epoch, int n_epochs, TrackOut* dev_out) {
		ugsdr_ctx* ctx = bank->ctx;
		require(samples && n_epochs > 0, "null samples or no epochs");
		require(samples_per_epoch == bank->spm, "samples_per_epoch must be sampling_rate / 1000");
		require(sample_type >= 0 && sample_type <= UGSDR_SAMPLES_NT1065_4, "unknown sample type");
		const size_t n = bank->spm * static_cast<size_t>(n_epochs);
		const size_t bytes = capture_bytes(sample_type, bank->fs, n);
		const void* dev = samples;
		if (!samples_on_device) {
			ctx->track_samples.reserve(bytes);
			UG_CUDA(cudaMemcpyAsync(ctx->track_samples.ptr, samples, bytes, cudaMemcpyHostToDevice, ctx->stream));
			dev = ctx->track_samples.ptr;
		}
		if (is_packed(sample_type)) {
			// packed captures (BBP DDC, NT1065) are decoded to complex float first
			PackedLayout l;
			l.spm = static_cast<uint32_t>(bank->spm);
			l.epoch_bytes = static_cast<uint32_t>(bbp_epoch_bytes(bank->fs));
			ctx->track_unpacked.reserve(sizeof(float2) * n);
			const int blocks = static_cast<int>(std::min<size_t>((n + 255) / 256, static_cast<size_t>(ctx->sm_count) * 8));
			unpack_kernel<<<blocks, 256, 0, ctx->stream>>>(dev, sample_type, l, n, ctx->track_unpacked.as<float2>());
			note_launch(ctx);
			dev = ctx->track_unpacked.ptr;
			sample_type = UGSDR_SAMPLES_CF32;
		}
		const size_t per = capture_bytes(sample_type, bank->fs, n) / n;  // bytes per sample the kernel reads
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
		p.nco_mode = bank->nco_mode;
		p.replicas = bank->replicas.as<float>();
		p.lut = get_lut(ctx);
		p.states = bank->states.as<TrackState>();
		p.out = dev_out;
		// stage the samples through shared memory when a 16/8/4-byte cp.async
		// divides the epoch size and the base address (chunks are 32 KiB or 8192
		// samples, multiples of 16 bytes)
		const uintptr_t addr = reinterpret_cast<uintptr_t>(dev);
		p.stage_g = 0;
		for (int g : {16, 8, 4})
			if ((per * bank->spm) % g == 0 && addr % g == 0) {
				p.stage_g = g;
				break;
			}
		const dim3 grid(bank->n_channels), block(kTrackThreads);
		const size_t smem_win = 2 * sizeof(float) * kWinFloats;
		const size_t smem = smem_win + (p.stage_g ? 2 * kStageBytes : 0);
		KernelTimer timer(ctx, "track_bank");
		auto launch = [&](auto staged_kernel, auto direct_kernel) {
			auto kernel = p.stage_g ? staged_kernel : direct_kernel;
			UG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
			kernel<<<grid, block, smem, ctx->stream>>>(p);
		};
		switch (sample_type) {
		case UGSDR_SAMPLES_CF32:
			launch(track_bank_kernel<UGSDR_SAMPLES_CF32, true>, track_bank_kernel<UGSDR_SAMPLES_CF32, false>);
			break;
		case UGSDR_SAMPLES_CI8:
			launch(track_bank_kernel<UGSDR_SAMPLES_CI8, true>, track_bank_kernel<UGSDR_SAMPLES_CI8, false>);
			break;
		case UGSDR_SAMPLES_CI16:
			launch(track_bank_kernel<UGSDR_SAMPLES_CI16, true>, track_bank_kernel<UGSDR_SAMPLES_CI16, false>);
			break;
		default:
			launch(track_bank_kernel<UGSDR_SAMPLES_RI8, true>, track_bank_kernel<UGSDR_SAMPLES_RI8, false>);
			break;
		}
		note_launch(ctx);
	}
}

namespace ugsdr_gpu {
	void track_bank_shape(const ugsdr_track_bank* bank, ugsdr_ctx** ctx, int* n_channels, size_t* spm, double* fs) {
		*ctx = bank->ctx;
		*n_channels = bank->n_channels;
		*spm = bank->spm;
		*fs = bank->fs;
	}

	// The serving path: n_epochs of device samples on `stream` (the caller
	// holds the context lock), outputs to device memory.
	void track_enqueue_on(ugsdr_track_bank* bank, const void* dev_samples, int sample_type, int n_epochs,
		ugsdr_track_output* dev_out, cudaStream_t stream) {
		ugsdr_ctx* ctx = bank->ctx;
		const cudaStream_t saved = ctx->stream;
		ctx->stream = stream;
		try {
			track_enqueue(bank, dev_samples, sample_type, 1, bank->spm, n_epochs, reinterpret_cast<TrackOut*>(dev_out));
		}
		catch (...) {
			ctx->stream = saved;
			throw;
		}
		ctx->stream = saved;
	}
}

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
		require(code_len_max <= (1 << 20), "codes longer than 2^20 chips are not supported");
		auto b = std::make_unique<ugsdr_track_bank>();
		b->ctx = ctx;
		b->n_channels = n_channels;
		b->fs = channels[0].sampling_rate;
		require(b->fs > 0 && std::fmod(b->fs, 1e3) == 0.0, "sampling rate must be a whole number of kHz");
		b->spm = static_cast<size_t>(b->fs / 1e3);
		require(b->spm >= 2 * kWinPad && b->fs <= kMaxRate, "sampling rate must be between 256 kHz and 131.072 MHz");
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
		require(cfg->nco_mode == 0 || cfg->nco_mode == 1, "nco_mode must be 0 or 1");
		b->nco_mode = cfg->nco_mode;

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
			// every tap within kWinPad - 2 samples of the prompt (replica window margin)
			require((std::fmax(std::fabs(el), std::fabs(vel)) * b->fs / ch.code_frequency) + 2 <= kWinPad,
				"tap spacing too wide for the sampling rate (more than 126 samples from the prompt)");
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
			s.phase_rad = ch.carrier_phase;
			st[c] = s;
		}
		// replica tables, one per (code, period): the code repeated over three
		// periods and upsampled as Codes::FillCodesImpl does (tracker.hpp:40-50:
		// full-code index q takes chip floor(q L3 / S3) mod len, L3 = 3 len,
		// S3 = 3 P), stored from q = -kWinPad to 3 P + kWinPad + 16 (periodic
		// beyond the three periods), each table 16-byte aligned
		std::vector<float> tables;
		std::map<std::pair<int, int>, long long> where;
		for (auto& s : st) {
			const auto key = std::make_pair(s.code, s.period_ms);
			auto it = where.find(key);
			if (it == where.end()) {
				const unsigned long long P = b->spm * static_cast<unsigned long long>(s.period_ms);
				const unsigned long long L3 = 3ull * static_cast<unsigned long long>(s.len), S3 = 3 * P;
				const size_t n_tab = (3 * P + 2 * kWinPad + 16 + 3) / 4 * 4;
				const long long at = static_cast<long long>(tables.size());
				tables.resize(tables.size() + n_tab);
				const float* chips = codes + static_cast<size_t>(s.code) * code_len_max;
				for (size_t x = 0; x < n_tab; ++x) {
					long long q = static_cast<long long>(x) - kWinPad;
					q %= static_cast<long long>(S3);
					if (q < 0)
						q += static_cast<long long>(S3);
					const unsigned long long chip = (static_cast<unsigned long long>(q) * L3 / S3) % static_cast<unsigned long long>(s.len);
					tables[static_cast<size_t>(at) + x] = chips[chip];
				}
				it = where.emplace(key, at).first;
			}
			s.rep = it->second;
		}
		b->replicas.reserve(sizeof(float) * tables.size());
		b->states.reserve(sizeof(TrackState) * n_channels);
		UG_CUDA(cudaMemcpy(b->replicas.ptr, tables.data(), sizeof(float) * tables.size(), cudaMemcpyHostToDevice));
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
		TrackOut* dev_out = nullptr;
		const size_t out_per_epoch = sizeof(TrackOut) * bank->n_channels;
		if (outputs) {
			ctx->track_out.reserve(out_per_epoch * static_cast<size_t>(n_epochs));
			dev_out = ctx->track_out.as<TrackOut>();
		}
		if (samples_on_device || n_epochs <= kCopyChunkEpochs) {
			track_enqueue(bank, samples, sample_type, samples_on_device, samples_per_epoch, n_epochs, dev_out);
			if (outputs)
				UG_CUDA(cudaMemcpyAsync(outputs, dev_out, out_per_epoch * static_cast<size_t>(n_epochs), cudaMemcpyDeviceToHost,
					ctx->stream));
			UG_CUDA(cudaStreamSynchronize(ctx->stream));
			return;
		}
		// host capture: chunks of kCopyChunkEpochs epochs through two staging
		// slots, the copy of chunk c + 1 (copy stream) overlapping the bank's
		// run over chunk c (context stream); each chunk's outputs are copied
		// back as soon as its run ends
		require(samples_per_epoch == bank->spm, "samples_per_epoch must be sampling_rate / 1000");
		require(sample_type >= 0 && sample_type <= UGSDR_SAMPLES_NT1065_4, "unknown sample type");
		if (!ctx->copy_stream) {
			UG_CUDA(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking));
			for (int i = 0; i < 2; ++i) {
				UG_CUDA(cudaEventCreateWithFlags(&ctx->slot_copied[i], cudaEventDisableTiming));
				UG_CUDA(cudaEventCreateWithFlags(&ctx->slot_used[i], cudaEventDisableTiming));
			}
		}
		const size_t chunk_bytes = capture_bytes(sample_type, bank->fs, bank->spm * static_cast<size_t>(kCopyChunkEpochs));
		ctx->track_samples.reserve(2 * chunk_bytes);
		const char* src = static_cast<const char*>(samples);
		const int n_chunks = (n_epochs + kCopyChunkEpochs - 1) / kCopyChunkEpochs;
		auto epochs_of = [&](int c) { return std::min(kCopyChunkEpochs, n_epochs - c * kCopyChunkEpochs); };
		auto slot_ptr = [&](int c) { return ctx->track_samples.as<char>() + (c & 1) * chunk_bytes; };
		auto copy_in = [&](int c) {
			if (c >= 2)  // the run over chunk c - 2 has read the slot
				UG_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->slot_used[c & 1], 0));
			const size_t bytes = capture_bytes(sample_type, bank->fs, bank->spm * static_cast<size_t>(epochs_of(c)));
			UG_CUDA(cudaMemcpyAsync(slot_ptr(c), src + static_cast<size_t>(c) * chunk_bytes, bytes, cudaMemcpyHostToDevice,
				ctx->copy_stream));
			UG_CUDA(cudaEventRecord(ctx->slot_copied[c & 1], ctx->copy_stream));
		};
		copy_in(0);
		for (int c = 0; c < n_chunks; ++c) {
			const int e0 = c * kCopyChunkEpochs;
			const int ne = epochs_of(c);
			UG_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->slot_copied[c & 1], 0));
			TrackOut* out_c = dev_out ? dev_out + static_cast<size_t>(e0) * bank->n_channels : nullptr;
			track_enqueue(bank, slot_ptr(c), sample_type, 1, samples_per_epoch, ne, out_c);
			UG_CUDA(cudaEventRecord(ctx->slot_used[c & 1], ctx->stream));
			// the next chunk's copy goes ahead of this chunk's outputs on the
			// copy stream, so it overlaps this run
			if (c + 1 < n_chunks)
				copy_in(c + 1);
			if (outputs) {
				UG_CUDA(cudaStreamWaitEvent(ctx->copy_stream, ctx->slot_used[c & 1], 0));
				UG_CUDA(cudaMemcpyAsync(reinterpret_cast<char*>(outputs) + out_per_epoch * static_cast<size_t>(e0), out_c,
					out_per_epoch * static_cast<size_t>(ne), cudaMemcpyDeviceToHost, ctx->copy_stream));
			}
		}
		UG_CUDA(cudaStreamSynchronize(ctx->copy_stream));
		UG_CUDA(cudaStreamSynchronize(ctx->stream));
	});
}

int ugsdr_track_run_device(ugsdr_track_bank* bank, const void* samples, int sample_type, size_t samples_per_epoch,
	int n_epochs, ugsdr_track_output* outputs) {
	if (!bank)
		return UGSDR_E_INVALID;
	ugsdr_ctx* ctx = bank->ctx;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		track_enqueue(bank, samples, sample_type, 1, samples_per_epoch, n_epochs, reinterpret_cast<TrackOut*>(outputs));
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

// Tracking outputs -> measurements on the device (src/measurements/
// observable.hpp), for every channel of a tracking bank at once, reading the
// bank's n_epochs x n_channels output array where the bank left it.
//
//   preamble_kernel   FindPreambleGps / FindPreambleGlonass's candidate
//                     search (observable.hpp:204-220, 260-277): the sign of
//                     the prompt I per epoch, circularly correlated with the
//                     preamble upsampled to 1 ms, epochs above the threshold
//                     listed in order.  One CTA per channel over tiles of
//                     epochs; the correlation is a sum of per-symbol box sums
//                     of the signs, exact in integers.
//   obs_sigma_kernel  CalculateSnr's sigma (observable.hpp:55-72): the
//                     reference's SequentialMeanStdDev over the prompt Q in
//                     float, in epoch order (mean_stddev.hpp:29-42), one warp
//                     per channel.
//   obs_segsum_kernel the per-epoch carrier-phase increments summed per
//   obs_emit_kernel   segment of epochs, then per epoch the unwrapped phase
//                     (segment prefix + warp scan, snapped to the bank's
//                     wrapped 64-bit phase), pseudorange, pseudophase,
//                     Doppler and SNR (the Observable constructor, 75-88).
#include "internal.hpp"

#include <cmath>
#include <vector>

namespace ugsdr_gpu {
	namespace {
		constexpr int kObsThreads = 256;
		constexpr int kObsWarps = kObsThreads / 32;
		constexpr int kPreambleTile = 1024;    // epochs per CTA pass
		constexpr int kSegment = 1024;         // epochs per warp of the phase scan
		constexpr int kMaxPreambleSymbols = 40;
		constexpr int kMaxPreambleLen = 400;   // symbols x upsampling, GLONASS
		constexpr double kTwoPi = 6.283185307179586476925286766559;
		constexpr double kInvTwoPi = 1.0 / kTwoPi;

		// Preambles as +-1 symbols per 20 ms (GPS) or 10 ms (GLONASS):
		// GetPreambleGps (observable.hpp:92-94), the LNAV preamble 10001011;
		// GetPreambleGlonass (143-146), the 30-chip time mark followed by ten
		// meander symbols.  Thresholds on |matched filter| from 219 and 276.
		__constant__ signed char kGpsPreamble[8] = {1, -1, -1, -1, 1, -1, 1, 1};
		__constant__ signed char kGloPreamble[40] = {
			-1, -1, -1, -1, -1, 1, 1, 1, -1, -1, 1, -1, -1, -1, 1, -1, 1, -1, 1, 1,
			1, 1, -1, 1, 1, -1, 1, -1, -1, 1, 1, -1, 1, -1, 1, -1, 1, -1, -1, 1};

		struct PreambleParams {
			const ugsdr_track_output* out;  // [epoch][channel]
			int n_epochs, n_channels;
			const int* messages;            // per channel, ugsdr_nav_message
			int* counts;                    // per channel
			int* indexes;                   // [channel][cap]
			int cap;
		};

		__global__ void __launch_bounds__(kObsThreads) preamble_kernel(PreambleParams p) {
			__shared__ int win[kPreambleTile + kMaxPreambleLen];
			__shared__ int box[kPreambleTile + kMaxPreambleLen];
			__shared__ int sym[kMaxPreambleSymbols];
			__shared__ int warp_hits[kObsWarps];
			const int c = blockIdx.x;
			const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
			const bool glonass = p.messages[c] == UGSDR_NAV_GLONASS;
			const int n_sym = glonass ? 40 : 8;
			const int up = glonass ? 10 : 20;
			const int threshold = glonass ? 370 : 153;
			const int n = p.n_epochs;
			// the preamble is cut to the prompt's length (preamble.resize(size))
			const int len = min(n_sym * up, n);
			const int full = len / up, rem = len % up;
			const int span = kPreambleTile + len;
			for (int s = threadIdx.x; s < n_sym; s += kObsThreads)
				sym[s] = glonass ? kGloPreamble[s] : kGpsPreamble[s];
			int found = 0;  // candidates so far, the same in every thread
			for (int k0 = 0; k0 < n; k0 += kPreambleTile) {
				__syncthreads();  // the previous tile's readers are done
				for (int t = threadIdx.x; t < span; t += kObsThreads) {
					const int e = (k0 + t) % n;  // the filter is circular
					win[t] = p.out[static_cast<size_t>(e) * p.n_channels + c].taps[2][0] > 0.f ? 1 : -1;
				}
				__syncthreads();
				for (int t = threadIdx.x; t + up <= span; t += kObsThreads) {
					int b = 0;
					for (int j = 0; j < up; ++j)
						b += win[t + j];
					box[t] = b;
				}
				__syncthreads();
				for (int r = 0; r < kPreambleTile / kObsThreads; ++r) {
					const int t = r * kObsThreads + threadIdx.x;
					const int k = k0 + t;
					bool hit = false;
					if (k < n) {
						// y[k] = 2 sum_m x[(k + m) mod n] p[m] (the 2/N inverse
						// of the reference's FFT matched filter)
						int s = 0;
						for (int q = 0; q < full; ++q)
							s += sym[q] * box[t + q * up];
						if (rem) {
							int b = 0;
							for (int j = 0; j < rem; ++j)
								b += win[t + full * up + j];
							s += sym[full] * b;
						}
						hit = 2 * abs(s) > threshold;
					}
					const unsigned mask = __ballot_sync(0xffffffffu, hit);
					if (lane == 0)
						warp_hits[warp] = __popc(mask);
					__syncthreads();
					int before = found, total = found;
					for (int w = 0; w < kObsWarps; ++w) {
						before += w < warp ? warp_hits[w] : 0;
						total += warp_hits[w];
					}
					if (hit) {
						const int pos = before + __popc(mask & ((1u << lane) - 1u));
						if (pos < p.cap)
							p.indexes[static_cast<size_t>(c) * p.cap + pos] = k;
					}
					found = total;
					__syncthreads();  // warp_hits is rewritten next round
				}
			}
			if (threadIdx.x == 0)
				p.counts[c] = found;
		}

		// per channel, precomputed on the host
		struct ObsChannel {
			double samples_to_ms;   // 1000 / sampling_rate
			double windup;          // intermediate_frequency / 1e3
			double intermediate_frequency;
			double phase0;          // carrier phase before epoch 0, cycles
			double frequency0;      // carrier frequency before epoch 0, Hz
			double correction;      // range_correction_ms
			long long position;     // preamble_position
		};

		struct ObsParams {
			const ugsdr_track_output* out;  // [epoch][channel]
			int n_epochs, n_channels, n_segments;
			const ObsChannel* ch;
			float* sigma;                   // per channel
			double* segsum;                 // [channel][segment]
			ugsdr_observable* obs;          // [epoch][channel]
		};

		__device__ __forceinline__ const ugsdr_track_output& rec(const ObsParams& p, int e, int c) {
			return p.out[static_cast<size_t>(e) * p.n_channels + c];
		}

		// cycles the loop advanced the carrier phase at epoch e: UpdatePhase
		// with the frequency before the epoch's update (2 pi f / 1000 rad),
		// then Pll's phase_error * pi / 2 rad (tracking_parameters.hpp:163-165,
		// 495-511)
		__device__ __forceinline__ double phase_step(const ObsParams& p, int e, int c) {
			const double f = e == 0 ? p.ch[c].frequency0 : rec(p, e - 1, c).carrier_frequency;
			return f * 1e-3 + rec(p, e, c).phase_error * 0.25;
		}

		// One warp per channel, launched as 2-warp CTAs so the channels spread
		// over every SM: each lane loads 8 epochs of a 256-epoch group (32
		// apart) and the next group's 8 while the current group's 256 values are
		// added in epoch order (every lane replays the same serial adds), so 16
		// record loads per lane are in flight behind one dependent add chain.
		constexpr int kSigmaWarps = 2;
		__global__ void __launch_bounds__(kObsThreads) obs_sigma_kernel(ObsParams p) {
			const int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
			const int lane = threadIdx.x & 31;
			if (c >= p.n_channels)
				return;
			const int n = p.n_epochs;
			float q = 0.f, m = 0.f;
			float cur[8], nxt[8];
			auto load_group = [&](int g, float (&v)[8]) {
#pragma unroll
				for (int j = 0; j < 8; ++j) {
					const int e = g * 256 + j * 32 + lane;
					v[j] = e < n ? rec(p, e, c).taps[2][1] : 0.f;
				}
			};
			load_group(0, cur);
			for (int g = 0; g * 256 < n; ++g) {
				load_group(g + 1, nxt);
#pragma unroll
				for (int j = 0; j < 8; ++j) {
					const int e0 = g * 256 + j * 32;
					const int cnt = min(32, n - e0);
					if (cnt <= 0)
						break;
					if (cnt == 32) {
						// all 32 shuffles issue ahead of the two serial add chains
						float x[32];
#pragma unroll
						for (int k = 0; k < 32; ++k)
							x[k] = __shfl_sync(0xffffffffu, cur[j], k);
#pragma unroll
						for (int k = 0; k < 32; ++k) {
							q = __fadd_rn(q, __fmul_rn(x[k], x[k]));
							m = __fadd_rn(m, x[k]);
						}
					}
					else {
						for (int k = 0; k < cnt; ++k) {
							const float x = __shfl_sync(0xffffffffu, cur[j], k);
							q = __fadd_rn(q, __fmul_rn(x, x));
							m = __fadd_rn(m, x);
						}
					}
				}
#pragma unroll
				for (int j = 0; j < 8; ++j)
					cur[j] = nxt[j];
			}
			if (lane == 0) {
				float s = 0.f;
				if (n >= 2) {
					const float nf = static_cast<float>(n);
					const float var = __fdiv_rn(__fsub_rn(q, __fdiv_rn(__fmul_rn(m, m), nf)), static_cast<float>(n - 1));
					s = __fsqrt_rn(var);
				}
				p.sigma[c] = s;
			}
		}

		__global__ void __launch_bounds__(kObsThreads) obs_segsum_kernel(ObsParams p) {
			const long long wid = static_cast<long long>(blockIdx.x) * kObsWarps + (threadIdx.x >> 5);
			const int lane = threadIdx.x & 31;
			if (wid >= static_cast<long long>(p.n_channels) * p.n_segments)
				return;
			const int c = static_cast<int>(wid / p.n_segments), g = static_cast<int>(wid % p.n_segments);
			const int end = min(p.n_epochs, (g + 1) * kSegment);
			double s = 0.0;
			for (int e = g * kSegment + lane; e < end; e += 32)
				s += phase_step(p, e, c);
			for (int o = 16; o; o >>= 1)
				s += __shfl_xor_sync(0xffffffffu, s, o);
			if (lane == 0)
				p.segsum[wid] = s;
		}

		__global__ void __launch_bounds__(kObsThreads) obs_emit_kernel(ObsParams p) {
			const long long wid = static_cast<long long>(blockIdx.x) * kObsWarps + (threadIdx.x >> 5);
			const int lane = threadIdx.x & 31;
			if (wid >= static_cast<long long>(p.n_channels) * p.n_segments)
				return;
			const int c = static_cast<int>(wid / p.n_segments), g = static_cast<int>(wid % p.n_segments);
			const ObsChannel ch = p.ch[c];
			// phase before the segment: channel start + the earlier segments
			double base = 0.0;
			for (int h = lane; h < g; h += 32)
				base += p.segsum[static_cast<long long>(c) * p.n_segments + h];
			for (int o = 16; o; o >>= 1)
				base += __shfl_xor_sync(0xffffffffu, base, o);
			base += ch.phase0;
			// Observable: pseudorange_offset = int32(code_phases[position] * samples_to_ms_rate)
			const int range_offset = __double2int_rz(__dmul_rn(rec(p, static_cast<int>(ch.position), c).code_phase,
				ch.samples_to_ms));
			const float sigma = p.sigma[c];
			const int end = min(p.n_epochs, (g + 1) * kSegment);
			for (int e0 = g * kSegment; e0 < end; e0 += 32) {
				const int e = e0 + lane;
				const bool valid = e < end;
				double scan = valid ? phase_step(p, e, c) : 0.0;
				for (int o = 1; o < 32; o <<= 1) {
					const double up = __shfl_up_sync(0xffffffffu, scan, o);
					if (lane >= o)
						scan += up;
				}
				const double approx = base + scan;  // within far less than half a cycle
				base += __shfl_sync(0xffffffffu, scan, 31);
				if (!valid)
					continue;
				const ugsdr_track_output& r = rec(p, e, c);
				// the bank keeps the phase as a 64-bit fraction of a cycle:
				// its whole cycles come from the running sum
				// (times 1 / 2 pi: the FP64 division would be this pass's costliest
				// operation; the cycles differ from the quotient by an ulp)
				const double wrapped = r.carrier_phase * kInvTwoPi;
				const double cycles = rint(approx - wrapped) + wrapped;
				ugsdr_observable o;
				o.pseudorange = __dadd_rn(__dsub_rn(__dmul_rn(r.code_phase, ch.samples_to_ms),
					static_cast<double>(range_offset)), ch.correction);
				// phases[i] = -carrier_phase / 2 pi, plus (i + 1) * IF / 1e3
				o.pseudophase = __dadd_rn(-cycles, __dmul_rn(static_cast<double>(e + 1), ch.windup));
				o.doppler = __dsub_rn(r.carrier_frequency, ch.intermediate_frequency);
				// 27 + 20 * std::log10(|I| / sigma), all in float
				const float ratio = __fdiv_rn(fabsf(r.taps[2][0]), sigma);
				o.snr = static_cast<double>(__fadd_rn(27.f, __fmul_rn(20.f, log10f(ratio))));
				p.obs[static_cast<size_t>(e) * p.n_channels + c] = o;
			}
		}

		unsigned blocks_for_warps(long long warps) {
			return static_cast<unsigned>((warps + kObsWarps - 1) / kObsWarps);
		}

		// device copy of the bank outputs (or the caller's device pointer)
		const ugsdr_track_output* stage_outputs(ugsdr_ctx* ctx, const ugsdr_track_output* outputs, int on_device,
			size_t records) {
			if (on_device)
				return outputs;
			ctx->obs_in.reserve(sizeof(ugsdr_track_output) * records);
			UG_CUDA(cudaMemcpyAsync(ctx->obs_in.ptr, outputs, sizeof(ugsdr_track_output) * records,
				cudaMemcpyHostToDevice, ctx->stream));
			return ctx->obs_in.as<ugsdr_track_output>();
		}
	}
}

using namespace ugsdr_gpu;

#define UG_OBS_ENTRY(ctx) \
	if (!(ctx))           \
		return UGSDR_E_INVALID; \
	std::lock_guard<std::mutex> lock_((ctx)->mutex); \
	return guarded((ctx), [&]

extern "C" {

int ugsdr_preamble_search(ugsdr_ctx* ctx, const ugsdr_track_output* outputs, int outputs_on_device, int n_epochs,
	int n_channels, const int* messages, int* counts, int* indexes, int cap) {
	UG_OBS_ENTRY(ctx) {
		require(outputs && messages && counts, "null outputs, messages or counts");
		require(n_epochs >= 1 && n_epochs <= (1 << 30) && n_channels >= 1, "bad output array shape");
		require(cap >= 0 && (cap == 0 || indexes), "null indexes");
		for (int c = 0; c < n_channels; ++c)
			require(messages[c] == UGSDR_NAV_GPS_LNAV || messages[c] == UGSDR_NAV_GLONASS, "unknown navigation message");
		const size_t records = static_cast<size_t>(n_epochs) * n_channels;
		const ugsdr_track_output* d_out = stage_outputs(ctx, outputs, outputs_on_device, records);
		const size_t list_bytes = sizeof(int) * static_cast<size_t>(n_channels) * cap;
		ctx->obs_tmp.reserve(sizeof(int) * 2 * static_cast<size_t>(n_channels) + list_bytes + 16);
		int* d_msg = ctx->obs_tmp.as<int>();
		int* d_counts = d_msg + n_channels;
		int* d_idx = d_counts + n_channels;
		UG_CUDA(cudaMemcpyAsync(d_msg, messages, sizeof(int) * n_channels, cudaMemcpyHostToDevice, ctx->stream));
		PreambleParams p{d_out, n_epochs, n_channels, d_msg, d_counts, d_idx, cap};
		{
			KernelTimer timer(ctx, "obs_preamble");
			preamble_kernel<<<static_cast<unsigned>(n_channels), kObsThreads, 0, ctx->stream>>>(p);
			UG_CUDA(cudaGetLastError());
			note_launch(ctx);
		}
		UG_CUDA(cudaMemcpyAsync(counts, d_counts, sizeof(int) * n_channels, cudaMemcpyDeviceToHost, ctx->stream));
		if (list_bytes)
			UG_CUDA(cudaMemcpyAsync(indexes, d_idx, list_bytes, cudaMemcpyDeviceToHost, ctx->stream));
		UG_CUDA(cudaStreamSynchronize(ctx->stream));
	});
}

int ugsdr_observables(ugsdr_ctx* ctx, const ugsdr_track_output* outputs, int outputs_on_device, int n_epochs,
	int n_channels, const ugsdr_observable_channel* channels, ugsdr_observable* out) {
	UG_OBS_ENTRY(ctx) {
		require(outputs && channels && out, "null outputs, channels or observables");
		require(n_epochs >= 1 && n_epochs <= (1 << 30) && n_channels >= 1, "bad output array shape");
		std::vector<ObsChannel> ch(n_channels);
		for (int c = 0; c < n_channels; ++c) {
			const ugsdr_observable_channel& in = channels[c];
			require(in.sampling_rate > 0, "sampling rate must be positive");
			require(in.preamble_position >= 0 && in.preamble_position < n_epochs, "preamble position outside the epochs");
			ch[c].samples_to_ms = 1000 / in.sampling_rate;
			ch[c].windup = in.intermediate_frequency / 1e3;
			ch[c].intermediate_frequency = in.intermediate_frequency;
			ch[c].phase0 = in.carrier_phase / kTwoPi;
			ch[c].frequency0 = in.carrier_frequency;
			ch[c].correction = in.range_correction_ms;
			ch[c].position = in.preamble_position;
		}
		const size_t records = static_cast<size_t>(n_epochs) * n_channels;
		const ugsdr_track_output* d_out = stage_outputs(ctx, outputs, outputs_on_device, records);
		const int n_segments = (n_epochs + kSegment - 1) / kSegment;
		const size_t segs = static_cast<size_t>(n_channels) * n_segments;
		// scratch: channels | sigma | segment sums (256-byte aligned regions)
		auto align = [](size_t b) { return (b + 255) & ~static_cast<size_t>(255); };
		const size_t ch_bytes = align(sizeof(ObsChannel) * n_channels), sig_bytes = align(sizeof(float) * n_channels);
		ctx->obs_tmp.reserve(ch_bytes + sig_bytes + sizeof(double) * segs);
		char* base = ctx->obs_tmp.as<char>();
		ObsChannel* d_ch = reinterpret_cast<ObsChannel*>(base);
		float* d_sigma = reinterpret_cast<float*>(base + ch_bytes);
		double* d_seg = reinterpret_cast<double*>(base + ch_bytes + sig_bytes);
		UG_CUDA(cudaMemcpyAsync(d_ch, ch.data(), sizeof(ObsChannel) * n_channels, cudaMemcpyHostToDevice, ctx->stream));
		ugsdr_observable* d_obs = out;
		if (!outputs_on_device) {
			ctx->obs_out.reserve(sizeof(ugsdr_observable) * records);
			d_obs = ctx->obs_out.as<ugsdr_observable>();
		}
		ObsParams p{d_out, n_epochs, n_channels, n_segments, d_ch, d_sigma, d_seg, d_obs};
		{
			KernelTimer timer(ctx, "observables");
			obs_sigma_kernel<<<(n_channels + kSigmaWarps - 1) / kSigmaWarps, 32 * kSigmaWarps, 0, ctx->stream>>>(p);
			obs_segsum_kernel<<<blocks_for_warps(static_cast<long long>(segs)), kObsThreads, 0, ctx->stream>>>(p);
			obs_emit_kernel<<<blocks_for_warps(static_cast<long long>(segs)), kObsThreads, 0, ctx->stream>>>(p);
			UG_CUDA(cudaGetLastError());
			note_launch(ctx, 3);
		}
		if (!outputs_on_device)
			UG_CUDA(cudaMemcpyAsync(out, d_obs, sizeof(ugsdr_observable) * records, cudaMemcpyDeviceToHost, ctx->stream));
		UG_CUDA(cudaStreamSynchronize(ctx->stream));
	});
}

}

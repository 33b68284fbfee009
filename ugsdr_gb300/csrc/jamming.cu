// Interference mitigation on the device: the STFT, the jamming detector and
// the suppression engine the digital front end runs after resampling
// (src/dfe/dfe.hpp:199-202).
//
//   stft_kernel         one CTA per group of columns: Hann window, forward
//                       column DFTs (compile-time 128-point plan), spectra
//                       out, and — for the detector — per column the eight
//                       strongest bins with their peak / sigma
//                       (JammingDetector::IntermediateDetection,
//                       src/antijamming/jamming_detection.hpp:113-128)
//   host                AnalyzeStftData (130-189): the occupation vote over
//                       at most 8 candidates per column — branchy, a few KB
//   istft_cols_kernel   FilterWideband (src/antijamming/jse.hpp:70-87): bins
//                       with |.| >= 20 zeroed, inverse column DFTs scaled 2/W
//   overlap_add_kernel  OverlapAndAdd (src/math/stft.hpp:63-75) as a gather:
//                       each output sums its covering columns in column order
//   null_bins_kernel    FilterInFreqencyDomain (jse.hpp:61-68): +-128 bins
//                       around each narrowband jammer of the whole-signal DFT
#include "internal.hpp"
#include "acq_batched.cuh"
#include "fft_static.cuh"

#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

namespace ugsdr_gpu {
	namespace {
		constexpr int kJamThreads = 256;
		constexpr int kMaxCandidates = 8;      // max_inreference_cnt (jamming_detection.hpp:81)
		constexpr int kNullHalfWidth = 3;      // null_window_size (82)
		constexpr double kJnThreshold = 6.0;   // j_s_threshold (78)
		constexpr double kProbability = 0.9;   // probability_threshold (79)
		constexpr float kWidebandLevel = 20.0f;  // j_s_absolute_threshold (jse.hpp:43)
		constexpr int kNarrowNull = 128;       // null_window_size (jse.hpp:47)
		constexpr int kDetectWindow = 128;     // Transform's defaults (stft.hpp:19)
		constexpr int kDetectOverlap = 96;

		struct JamCandidate {
			double jn;  // peak / sigma
			int bin;
			int pad;
		};

		struct StftParams {
			const float2* x;
			int w, hop;
			int cols;
			int per_cta;           // columns per CTA
			const float* window;   // w floats
			FftPlanDev plan;
			float2* s;             // cols x w spectra
			int detect;
			JamCandidate* cand;    // cols x kMaxCandidates
			int* counts;           // cols
		};

		__device__ __forceinline__ float magnitude(float2 v) { return sqrtf(v.x * v.x + v.y * v.y); }

		// The warp's column: kMaxCandidates rounds of first-max (lowest index on
		// ties, as std::max_element) each followed by nulling +-3 bins
		// (NullRegion, jamming_detection.hpp:101-110), then one-pass float mean
		// and unbiased sigma over the nulled magnitudes (SequentialMeanStdDev,
		// src/math/mean_stddev.hpp:29-42) and J/N = peak / sigma in double;
		// candidates with J/N < 6 are erased, the rest kept in order.
		__device__ void detect_column(float* m, int w, JamCandidate* out, int* count) {
			const int lane = threadIdx.x & 31;
			int bins[kMaxCandidates];
			float peaks[kMaxCandidates];
#pragma unroll
			for (int r = 0; r < kMaxCandidates; ++r) {
				float bv = -1.0f;
				int bi = 0x7fffffff;
				for (int k = lane; k < w; k += 32) {
					const float v = m[k];
					if (v > bv) {
						bv = v;
						bi = k;
					}
				}
				for (int o = 16; o > 0; o >>= 1) {
					const float ov = __shfl_xor_sync(0xffffffffu, bv, o);
					const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
					if (ov > bv || (ov == bv && oi < bi)) {
						bv = ov;
						bi = oi;
					}
				}
				bins[r] = bi;
				peaks[r] = bv;
				__syncwarp();
				if (lane <= 2 * kNullHalfWidth)
					m[(bi - kNullHalfWidth + lane + w) % w] = 0.0f;
				__syncwarp();
			}
			if (lane != 0)
				return;
			float q = 0.0f, s = 0.0f;
			for (int k = 0; k < w; ++k) {
				const float el = m[k];
				q = __fadd_rn(q, __fmul_rn(el, el));
				s = __fadd_rn(s, el);
			}
			const float fw = static_cast<float>(w);
			const float var = __fdiv_rn(__fsub_rn(q, __fdiv_rn(__fmul_rn(s, s), fw)), static_cast<float>(w - 1));
			const double sigma = static_cast<double>(__fsqrt_rn(var));
			int c = 0;
#pragma unroll
			for (int r = 0; r < kMaxCandidates; ++r) {
				const double jn = static_cast<double>(peaks[r]) / sigma;
				if (!(jn < kJnThreshold)) {  // remove_if(jn < threshold): a NaN stays
					out[c].jn = jn;
					out[c].bin = bins[r];
					out[c].pad = 0;
					++c;
				}
			}
			*count = c;
		}

		template <class F>
		__global__ void __launch_bounds__(kJamThreads) stft_kernel(StftParams p) {
			extern __shared__ float2 sm[];
			const int w = fft_n<F>(p.plan.n);
			const int ld = w | 1;
			const int c0 = blockIdx.x * p.per_cta;
			const int nc = min(p.per_cta, p.cols - c0);
			float2* a = sm;
			float2* b = sm + p.per_cta * ld;
			float* win = reinterpret_cast<float*>(sm + 2 * p.per_cta * ld);
			const FftPlanDev plan = F::prepare(p.plan, win + w);
			for (int i = threadIdx.x; i < w; i += blockDim.x)
				win[i] = p.window[i];
			__syncthreads();
			// vec * complex(window, 0) (stft.hpp:55-56): both parts scaled
			for (int e = threadIdx.x; e < nc * w; e += blockDim.x) {
				const int f = e / w, i = e - f * w;
				const float2 v = p.x[static_cast<size_t>(c0 + f) * p.hop + i];
				a[f * ld + i] = c2(__fmul_rn(v.x, win[i]), __fmul_rn(v.y, win[i]));
			}
			__syncthreads();
			const float2* y = F::template run<false>(a, b, plan, nc, ld);
			for (int e = threadIdx.x; e < nc * w; e += blockDim.x) {
				const int f = e / w, i = e - f * w;
				p.s[static_cast<size_t>(c0 + f) * w + i] = y[f * ld + i];
			}
			if (!p.detect)
				return;
			// magnitudes into the free tile, one warp per column
			float* mags = reinterpret_cast<float*>(y == a ? b : a);
			const int warp = threadIdx.x >> 5, n_warps = blockDim.x >> 5;
			for (int f = warp; f < nc; f += n_warps) {
				float* m = mags + f * 2 * ld;
				for (int k = threadIdx.x & 31; k < w; k += 32)
					m[k] = magnitude(y[f * ld + k]);
				__syncwarp();
				const int col = c0 + f;
				detect_column(m, w, p.cand + static_cast<size_t>(col) * kMaxCandidates, p.counts + col);
				__syncwarp();
			}
		}

		struct IstftParams {
			const float2* s;       // cols x w
			int w;
			int cols;
			int per_cta;
			int zero_wideband;     // FilterWideband's |.| >= 20 -> 0
			FftPlanDev plan;
			float2* t;             // cols x w inverse columns
		};

		template <class F>
		__global__ void __launch_bounds__(kJamThreads) istft_cols_kernel(IstftParams p) {
			extern __shared__ float2 sm[];
			const int w = fft_n<F>(p.plan.n);
			const int ld = w | 1;
			const int c0 = blockIdx.x * p.per_cta;
			const int nc = min(p.per_cta, p.cols - c0);
			float2* a = sm;
			float2* b = sm + p.per_cta * ld;
			const FftPlanDev plan = F::prepare(p.plan, b + p.per_cta * ld);
			for (int e = threadIdx.x; e < nc * w; e += blockDim.x) {
				const int f = e / w, i = e - f * w;
				float2 v = p.s[static_cast<size_t>(c0 + f) * w + i];
				if (p.zero_wideband && magnitude(v) >= kWidebandLevel)
					v = c2(0.0f, 0.0f);
				a[f * ld + i] = v;
			}
			__syncthreads();
			const float2* y = F::template run<true>(a, b, plan, nc, ld);
			// SequentialDft inverse (src/math/dft.hpp:124-129): el /= size; el *= 2
			const float fw = static_cast<float>(w);
			for (int e = threadIdx.x; e < nc * w; e += blockDim.x) {
				const int f = e / w, i = e - f * w;
				const float2 v = y[f * ld + i];
				p.t[static_cast<size_t>(c0 + f) * w + i] =
					c2(__fmul_rn(__fdiv_rn(v.x, fw), 2.0f), __fmul_rn(__fdiv_rn(v.y, fw), 2.0f));
			}
		}

		// dst[i * hop + j] += column_i[j] for i = 0, 1, ... (stft.hpp:69-72)
		// gathered per output sample; samples past the synthesis length are the
		// zeros of the resize to n (jse.hpp:83-85).
		__global__ void overlap_add_kernel(const float2* __restrict__ t, int w, int hop, int cols, uint64_t n,
			float2* __restrict__ out) {
			const uint64_t len = static_cast<uint64_t>(w) + static_cast<uint64_t>(cols - 1) * hop;
			for (uint64_t k = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; k < n;
				 k += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
				float ax = 0.0f, ay = 0.0f;
				if (k < len) {
					const int lo = k >= static_cast<uint64_t>(w) ? static_cast<int>((k - w) / hop) + 1 : 0;
					const int hi = min(cols - 1, static_cast<int>(k / hop));
					for (int i = lo; i <= hi; ++i) {
						const float2 v = t[static_cast<size_t>(i) * w + (k - static_cast<uint64_t>(i) * hop)];
						ax = __fadd_rn(ax, v.x);
						ay = __fadd_rn(ay, v.y);
					}
				}
				out[k] = c2(ax, ay);
			}
		}

		struct NullRange {
			uint64_t start;  // first bin (mod n)
			uint64_t len;
		};
		struct NullParams {
			NullRange r[2 * kMaxCandidates];
			int n_ranges;
		};

		__global__ void null_bins_kernel(float2* x, uint64_t n, NullParams p) {
			for (int d = 0; d < p.n_ranges; ++d)
				for (uint64_t j = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; j < p.r[d].len;
					 j += static_cast<uint64_t>(gridDim.x) * blockDim.x)
					x[(p.r[d].start + j) % n] = c2(0.0f, 0.0f);
		}

		int blocks_for(uint64_t n) {
			return static_cast<int>(std::min<uint64_t>((n + kJamThreads - 1) / kJamThreads, 152 * 16));
		}

		template <class Fn>
		void with_column_fft(int w, Fn&& fn) {
			if (w == 128)
				fn(StaticFft<128, 16, 8>{});
			else
				fn(RuntimeFft{});
		}

		FftPlanDev column_plan(ugsdr_ctx* ctx, int w) {
			const FftPlanDesc& d = get_plan(ctx, w);
			FftPlanDev p{};
			p.n = d.n;
			p.n_pass = d.n_pass;
			for (int i = 0; i < d.n_pass; ++i)
				p.radix[i] = d.radix[i];
			p.tw = d.tw;
			return p;
		}

		// columns per CTA and the shared memory they take: two tiles of
		// per_cta x (w | 1) + the plan's table (w entries) + the window
		int columns_per_cta(ugsdr_ctx* ctx, int w, size_t& smem) {
			const size_t ld = static_cast<size_t>(w | 1);
			int per = 16;
			auto bytes = [&](int c) { return 2 * sizeof(float2) * c * ld + sizeof(float2) * w + 16 + sizeof(float) * w; };
			while (per > 1 && bytes(per) > ctx->smem_optin - 2048)
				per /= 2;
			require(bytes(per) <= ctx->smem_optin - 2048, "STFT window too long for one CTA", UGSDR_E_UNSUPPORTED);
			smem = bytes(per);
			return per;
		}

		// SequentialStft::GetWindow (stft.hpp:34-40): computed in double, stored as float
		const float* hann_window(ugsdr_ctx* ctx, int w) {
			if (ctx->jam_window_len != w) {
				std::vector<float> h(w);
				const double pi = 3.14159265358979323846;
				for (int i = 0; i < w; ++i)
					h[i] = static_cast<float>(0.5 * (1 - std::cos(2.0 * pi * static_cast<double>(i) / w)));
				ctx->jam_window.reserve(sizeof(float) * w);
				UG_CUDA(cudaMemcpyAsync(ctx->jam_window.ptr, h.data(), sizeof(float) * w, cudaMemcpyHostToDevice, ctx->stream));
				UG_CUDA(cudaStreamSynchronize(ctx->stream));
				ctx->jam_window_len = w;
			}
			return ctx->jam_window.as<float>();
		}

		size_t stft_columns(size_t n, int w, int overlap) {
			require(w >= 2 * kNullHalfWidth + 2 && overlap >= 0 && overlap < w, "STFT window must be >= 8 and above the overlap");
			require(n >= static_cast<size_t>(w), "fewer samples than one STFT window");
			const size_t cols = (n - static_cast<size_t>(overlap)) / static_cast<size_t>(w - overlap);
			require(cols <= (1u << 30), "too many STFT columns");
			return cols;
		}

		// STFT of device samples x into ctx->jam_s, with detection candidates
		// into ctx->jam_cand when `detect`
		void stft_device(ugsdr_ctx* ctx, const float2* x, size_t cols, int w, int overlap, bool detect) {
			size_t smem = 0;
			const int per = columns_per_cta(ctx, w, smem);
			ctx->jam_s.reserve(sizeof(float2) * cols * w);
			StftParams p{};
			p.x = x;
			p.w = w;
			p.hop = w - overlap;
			p.cols = static_cast<int>(cols);
			p.per_cta = per;
			p.window = hann_window(ctx, w);
			p.plan = column_plan(ctx, w);
			p.s = ctx->jam_s.as<float2>();
			p.detect = detect ? 1 : 0;
			if (detect) {
				ctx->jam_cand.reserve((sizeof(JamCandidate) * kMaxCandidates + sizeof(int)) * cols);
				p.cand = ctx->jam_cand.as<JamCandidate>();
				p.counts = reinterpret_cast<int*>(p.cand + cols * kMaxCandidates);
			}
			with_column_fft(w, [&](auto f) {
				using F = decltype(f);
				UG_CUDA(cudaFuncSetAttribute(stft_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
				stft_kernel<F><<<static_cast<unsigned>((cols + per - 1) / per), kJamThreads, smem, ctx->stream>>>(p);
				note_launch(ctx);
			});
		}

		// inverse columns of ctx->jam_s (zeroing |.| >= 20 when asked) into
		// ctx->jam_t, overlap-added into n samples at out
		void istft_device(ugsdr_ctx* ctx, size_t cols, int w, int overlap, bool zero_wideband, float2* out, size_t n) {
			size_t smem = 0;
			const int per = columns_per_cta(ctx, w, smem);
			ctx->jam_t.reserve(sizeof(float2) * cols * w);
			IstftParams p{};
			p.s = ctx->jam_s.as<float2>();
			p.w = w;
			p.cols = static_cast<int>(cols);
			p.per_cta = per;
			p.zero_wideband = zero_wideband ? 1 : 0;
			p.plan = column_plan(ctx, w);
			p.t = ctx->jam_t.as<float2>();
			with_column_fft(w, [&](auto f) {
				using F = decltype(f);
				UG_CUDA(cudaFuncSetAttribute(istft_cols_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
				istft_cols_kernel<F><<<static_cast<unsigned>((cols + per - 1) / per), kJamThreads, smem, ctx->stream>>>(p);
			});
			overlap_add_kernel<<<blocks_for(n), kJamThreads, 0, ctx->stream>>>(ctx->jam_t.as<float2>(), w, w - overlap,
				static_cast<int>(cols), n, out);
			note_launch(ctx, 2);
		}

		struct Detection {
			int type;
			int bin;
			double frequency;
			double jn;
		};

		// AnalyzeStftData (jamming_detection.hpp:130-189) over the columns'
		// candidates, restated with its float/double and integer conversions;
		// frequency = bin * fs / 128 as the candidates are built (120).
		std::vector<Detection> analyze(const std::vector<int>& counts, const std::vector<JamCandidate>& cand, double fs, int w) {
			std::vector<Detection> dst;
			const size_t cols = counts.size();
			size_t mean_jammers = 0;
			for (int c : counts)
				mean_jammers += static_cast<size_t>(c);
			mean_jammers /= cols;
			struct Occupation {
				double count = 0;
				int bin = 0;
				double frequency = 0;
				double jn = 0;
			};
			for (size_t i = 0; i < mean_jammers; ++i) {
				std::map<double, Occupation> occ;
				double quantity = 0;
				for (size_t c = 0; c < cols; ++c) {
					if (static_cast<size_t>(counts[c]) <= i)
						continue;
					const JamCandidate& k = cand[c * kMaxCandidates + i];
					const double f = static_cast<double>(k.bin) * fs / static_cast<double>(w);
					Occupation& o = occ[f];
					o.count += 1;
					o.frequency = f;
					o.bin = k.bin;
					o.jn += k.jn;
					++quantity;
				}
				for (auto& kv : occ) {
					kv.second.count /= quantity;
					kv.second.jn /= quantity;
				}
				size_t cnt_wideband = 0;
				const Occupation* wide = &occ.begin()->second;
				for (auto& kv : occ) {
					const double probability = kv.second.count;
					if (probability >= kProbability) {
						dst.push_back({UGSDR_INTERFERENCE_NARROWBAND, kv.second.bin, kv.second.frequency, kv.second.jn});
						break;
					}
					if (probability >= kProbability / static_cast<double>(occ.size())) {
						++cnt_wideband;
						wide = &kv.second;
					}
				}
				// a single occupied frequency makes the bound 0: the reference
				// then reports it as wideband as well
				if (cnt_wideband >= static_cast<size_t>(occ.size() * kProbability))
					dst.push_back({UGSDR_INTERFERENCE_WIDEBAND, wide->bin, wide->frequency, wide->jn});
			}
			return dst;
		}

		// detector over device samples x (n): STFT + candidates on the device,
		// analysis on the host
		std::vector<Detection> detect_device(ugsdr_ctx* ctx, const float2* x, size_t n, double fs) {
			require(fs > 0, "sampling rate must be positive");
			const size_t cols = stft_columns(n, kDetectWindow, kDetectOverlap);
			stft_device(ctx, x, cols, kDetectWindow, kDetectOverlap, true);
			std::vector<JamCandidate> cand(cols * kMaxCandidates);
			std::vector<int> counts(cols);
			const JamCandidate* dc = ctx->jam_cand.as<JamCandidate>();
			UG_CUDA(cudaMemcpyAsync(cand.data(), dc, sizeof(JamCandidate) * cand.size(), cudaMemcpyDeviceToHost, ctx->stream));
			UG_CUDA(cudaMemcpyAsync(counts.data(), dc + cols * kMaxCandidates, sizeof(int) * cols, cudaMemcpyDeviceToHost, ctx->stream));
			UG_CUDA(cudaStreamSynchronize(ctx->stream));
			return analyze(counts, cand, fs, kDetectWindow);
		}

		void report(const std::vector<Detection>& det, ugsdr_jamming_detection* out, int cap, int* n_detections) {
			if (n_detections)
				*n_detections = static_cast<int>(det.size());
			for (int i = 0; out && i < cap && i < static_cast<int>(det.size()); ++i) {
				out[i].type = det[i].type;
				out[i].frequency_bin = det[i].bin;
				out[i].frequency = det[i].frequency;
				out[i].jammer_to_noise = det[i].jn;
			}
		}

		// the samples on the device: the caller's pointer or a staged copy
		float2* stage(ugsdr_ctx* ctx, const float* iq, size_t n, int on_device) {
			require(iq != nullptr && n > 0, "null or empty signal");
			if (on_device)
				return reinterpret_cast<float2*>(const_cast<float*>(iq));
			ctx->jam_x.reserve(sizeof(float2) * n);
			UG_CUDA(cudaMemcpyAsync(ctx->jam_x.ptr, iq, sizeof(float2) * n, cudaMemcpyHostToDevice, ctx->stream));
			return ctx->jam_x.as<float2>();
		}
	}
}

using namespace ugsdr_gpu;

#define UG_JAM_ENTRY(ctx) \
	if (!(ctx))           \
		return UGSDR_E_INVALID; \
	std::lock_guard<std::mutex> lock_((ctx)->mutex); \
	return guarded((ctx), [&]

extern "C" {

int ugsdr_stft(ugsdr_ctx* ctx, const float* in_iq, size_t n, int window_length, int overlap_length, float* out_iq,
	size_t* n_columns) {
	UG_JAM_ENTRY(ctx) {
		require(in_iq != nullptr, "null signal");
		const size_t cols = stft_columns(n, window_length, overlap_length);
		if (n_columns)
			*n_columns = cols;
		if (!out_iq)
			return;
		const float2* x = stage(ctx, in_iq, n, 0);
		stft_device(ctx, x, cols, window_length, overlap_length, false);
		UG_CUDA(cudaMemcpyAsync(out_iq, ctx->jam_s.ptr, sizeof(float2) * cols * window_length, cudaMemcpyDeviceToHost, ctx->stream));
		UG_CUDA(cudaStreamSynchronize(ctx->stream));
	});
}

int ugsdr_istft(ugsdr_ctx* ctx, const float* in_iq, size_t n_columns, int window_length, int overlap_length,
	float* out_iq) {
	UG_JAM_ENTRY(ctx) {
		require(in_iq && out_iq && n_columns > 0, "null or empty columns");
		require(window_length >= 2 * kNullHalfWidth + 2 && overlap_length >= 0 && overlap_length < window_length,
			"STFT window must be >= 8 and above the overlap");
		const size_t w = static_cast<size_t>(window_length);
		const size_t len = w + (n_columns - 1) * (w - overlap_length);
		ctx->jam_s.reserve(sizeof(float2) * n_columns * w);
		UG_CUDA(cudaMemcpyAsync(ctx->jam_s.ptr, in_iq, sizeof(float2) * n_columns * w, cudaMemcpyHostToDevice, ctx->stream));
		ctx->jam_x.reserve(sizeof(float2) * len);
		istft_device(ctx, n_columns, window_length, overlap_length, false, ctx->jam_x.as<float2>(), len);
		UG_CUDA(cudaMemcpyAsync(out_iq, ctx->jam_x.ptr, sizeof(float2) * len, cudaMemcpyDeviceToHost, ctx->stream));
		UG_CUDA(cudaStreamSynchronize(ctx->stream));
	});
}

int ugsdr_jamming_detect(ugsdr_ctx* ctx, const float* iq, size_t n, double fs, int samples_on_device,
	ugsdr_jamming_detection* out, int cap, int* n_detections) {
	UG_JAM_ENTRY(ctx) {
		const float2* x = stage(ctx, iq, n, samples_on_device);
		report(detect_device(ctx, x, n, fs), out, cap, n_detections);
	});
}

int ugsdr_jamming_suppress(ugsdr_ctx* ctx, float* iq, size_t n, double fs, int samples_on_device,
	ugsdr_jamming_detection* out, int cap, int* n_detections) {
	UG_JAM_ENTRY(ctx) {
		float2* x = stage(ctx, iq, n, samples_on_device);
		const std::vector<Detection> det = detect_device(ctx, x, n, fs);
		report(det, out, cap, n_detections);
		if (det.empty())
			return;
		const bool wideband = std::any_of(det.begin(), det.end(), [](const Detection& d) { return d.type == UGSDR_INTERFERENCE_WIDEBAND; });
		if (wideband) {
			const size_t cols = stft_columns(n, kDetectWindow, kDetectOverlap);
			istft_device(ctx, cols, kDetectWindow, kDetectOverlap, true, x, n);
		}
		else {
			// idx = size_t(frequency / fs * n); zero [idx - 128 + n, idx + 128]
			// (+ n when that wraps) modulo n (jse.hpp:50-59, 64-66)
			require(det.size() <= 2 * kMaxCandidates, "too many narrowband detections");
			NullParams np{};
			np.n_ranges = static_cast<int>(det.size());
			const long long nn = static_cast<long long>(n);
			for (size_t i = 0; i < det.size(); ++i) {
				const long long idx = static_cast<long long>(static_cast<size_t>(det[i].frequency / fs * static_cast<double>(n)));
				const long long start = idx - kNarrowNull + nn;
				long long finish = idx + kNarrowNull;
				if (finish < start)
					finish += nn;
				np.r[i].start = static_cast<uint64_t>(start);
				np.r[i].len = finish >= start ? static_cast<uint64_t>(finish - start + 1) : 0;
			}
			ctx->jam_t.reserve(sizeof(float2) * n);
			float2* spec = ctx->jam_t.as<float2>();
			dft_scaled(ctx, x, spec, n, false, ctx->jam_tmp);
			null_bins_kernel<<<blocks_for(2 * kNarrowNull + 1), kJamThreads, 0, ctx->stream>>>(spec, n, np);
			note_launch(ctx);
			dft_scaled(ctx, spec, x, n, true, ctx->jam_tmp);
		}
		if (!samples_on_device)
			UG_CUDA(cudaMemcpyAsync(iq, x, sizeof(float2) * n, cudaMemcpyDeviceToHost, ctx->stream));
		UG_CUDA(cudaStreamSynchronize(ctx->stream));
	});
}
}

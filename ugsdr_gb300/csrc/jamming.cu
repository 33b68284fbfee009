// Interference mitigation on the device: the STFT, the jamming detector and
// the suppression engine the digital front end runs after resampling
// (src/dfe/dfe.hpp:199-202).
//
//   detect_kernel       the detector's STFT, one warp per column with the
//                       128-point transform in registers and shuffles
//                       (Warp128), then the eight strongest bins with their
//                       peak / sigma (JammingDetector::IntermediateDetection,
//                       src/antijamming/jamming_detection.hpp:113-128) and
//                       each CTA's occupation histograms
//   stft_kernel         the per-op STFT (spectra out): columns per CTA in
//                       shared memory (compile-time 128-point plan)
//   decide_kernel,      AnalyzeStftData (130-189): the occupation vote per
//   jn_sum_kernel       round, then the reported J/N sums; only the detection
//                       list goes back to the host
//   wideband_kernel     FilterWideband (src/antijamming/jse.hpp:70-87) fused,
//                       one warp per run of output slots: the covering columns
//                       re-transformed from the samples (Warp128), bins with
//                       |.| >= 20 zeroed, inverse transforms scaled 2/W,
//                       overlap-added in column order in registers
//   istft_cols_kernel,  the per-op OverlapAndAdd (src/math/stft.hpp:63-75):
//   overlap_add_kernel  inverse columns, then a gather in column order
//   null_bins_kernel    FilterInFreqencyDomain (jse.hpp:61-68): +-128 bins
//                       around each narrowband jammer of the whole-signal DFT
#include "internal.hpp"
#include "acq_batched.cuh"
#include "fft_static.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace ugsdr_gpu {
	namespace {
		constexpr int kJamThreads = 256;
		constexpr int kMaxCandidates = 8;      // max_inreference_cnt (jamming_detection.hpp:81)
		constexpr int kNullHalfWidth = 3;      // null_window_size (82)
		constexpr float kJnThreshold = 6.0f;   // j_s_threshold (78)
		constexpr double kProbability = 0.9;   // probability_threshold (79)
		constexpr float kWidebandLevel = 20.0f;  // j_s_absolute_threshold (jse.hpp:43)
		constexpr int kNarrowNull = 128;       // null_window_size (jse.hpp:47)
		constexpr int kDetectWindow = 128;     // Transform's defaults (stft.hpp:19)
		constexpr int kDetectOverlap = 96;

		constexpr int kDetectBins = 128;        // the detector's window
		constexpr int kMaxDetections = 2 * kMaxCandidates;  // two per round at most
		constexpr int kSumCtas = 256;           // CTAs of the J/N sums
		constexpr uint8_t kNoBin = 0xFF;

		struct Detection {
			int type;
			int bin;
			double frequency;
			double jn;
		};

		struct DetectionList {
			int n;
			int pad;
			Detection d[kMaxDetections];
		};

		// Device scratch of the detector (one allocation, 256-byte regions):
		// per round r the occupation histogram over bins, the candidate count,
		// the decisions, the J/N partial sums and the detection list; then the
		// per-column candidates as rounds x columns arrays (bin, J/N).
		struct DetectScratch {
			int* hist;                  // [kMaxCandidates][kDetectBins]
			unsigned long long* total;  // candidates over all columns
			unsigned int* done;         // CTAs of jn_sum_kernel finished
			int* picks;                 // [kMaxCandidates][2]: narrowband, wideband bin or -1
			double* quantity;           // [kMaxCandidates]
			int* rounds;                // mean candidates per column
			DetectionList* list;
			double* partials;           // [kSumCtas][kMaxDetections]
			uint8_t* bins;              // [kMaxCandidates][cols], kNoBin past the column's count
			float* jn;                  // [kMaxCandidates][cols]
		};

		struct DetectLayout {
			size_t hist, total, done, picks, quantity, rounds, list, partials, bins, jn, bytes, zero_bytes;
			explicit DetectLayout(size_t cols) {
				size_t at = 0;
				auto take = [&](size_t b) {
					const size_t r = at;
					at = (at + b + 255) / 256 * 256;
					return r;
				};
				hist = take(sizeof(int) * kMaxCandidates * kDetectBins);
				total = take(sizeof(unsigned long long));
				done = take(sizeof(unsigned int));
				zero_bytes = at;  // hist, total and done start at zero
				picks = take(sizeof(int) * kMaxCandidates * 2);
				quantity = take(sizeof(double) * kMaxCandidates);
				rounds = take(sizeof(int));
				list = take(sizeof(DetectionList));
				partials = take(sizeof(double) * kSumCtas * kMaxDetections);
				bins = take(kMaxCandidates * cols);
				jn = take(sizeof(float) * kMaxCandidates * cols);
				bytes = at;
			}
			DetectScratch carve(void* base) const {
				char* b = static_cast<char*>(base);
				return DetectScratch{reinterpret_cast<int*>(b + hist), reinterpret_cast<unsigned long long*>(b + total),
					reinterpret_cast<unsigned int*>(b + done), reinterpret_cast<int*>(b + picks),
					reinterpret_cast<double*>(b + quantity), reinterpret_cast<int*>(b + rounds),
					reinterpret_cast<DetectionList*>(b + list), reinterpret_cast<double*>(b + partials),
					reinterpret_cast<uint8_t*>(b + bins), reinterpret_cast<float*>(b + jn)};
			}
		};

		struct StftParams {
			const float2* x;
			int w, hop;
			int cols;
			int per_cta;           // columns per CTA
			const float* window;   // w floats
			FftPlanDev plan;
			float2* s;             // cols x w spectra
		};

		__device__ __forceinline__ float magnitude(float2 v) { return sqrtf(v.x * v.x + v.y * v.y); }

		// The warp's column, magnitudes in registers (mv[j] of lane l is bin idx[j]):
		// kMaxCandidates rounds of first-max — the largest magnitude (redux max
		// over the bit patterns, which order as non-negative floats do), then
		// the lowest bin holding it (redux min), as std::max_element — each
		// followed by nulling +-3 bins (NullRegion, jamming_detection.hpp:
		// 101-110); then the float mean and unbiased sigma of the nulled
		// magnitudes with SequentialMeanStdDev's formula (src/math/
		// mean_stddev.hpp:29-42; the sums in warp-tree order) and J/N =
		// peak / sigma.  Candidates with J/N < 6 are erased, the rest
		// kept in order: kept candidate r of column `col` goes to [r][col] and
		// into the CTA's round-r occupation histogram.
		__device__ void detect_column(float (&mv)[kDetectBins / 32], const int (&idx)[kDetectBins / 32], const DetectScratch& d,
			size_t col, size_t cols, int* s_hist, unsigned int* s_total) {
			constexpr int J = kDetectBins / 32;
			const int lane = threadIdx.x & 31;
			int bins[kMaxCandidates];
			float peaks[kMaxCandidates];
#pragma unroll
			for (int r = 0; r < kMaxCandidates; ++r) {
				unsigned int top = 0;
#pragma unroll
				for (int j = 0; j < J; ++j)
					top = max(top, __float_as_uint(mv[j]));
				top = __reduce_max_sync(0xffffffffu, top);
				unsigned int first = 0xffffffffu;
#pragma unroll
				for (int j = 0; j < J; ++j)
					if (__float_as_uint(mv[j]) == top)
						first = min(first, static_cast<unsigned int>(idx[j]));
				const int bi = static_cast<int>(__reduce_min_sync(0xffffffffu, first));
				bins[r] = bi;
				peaks[r] = __uint_as_float(top);
#pragma unroll
				for (int j = 0; j < J; ++j) {
					const int dist = (idx[j] - bi + kDetectBins) % kDetectBins;
					if (dist <= kNullHalfWidth || dist >= kDetectBins - kNullHalfWidth)
						mv[j] = 0.0f;
				}
			}
			float q = 0.0f, s = 0.0f;
#pragma unroll
			for (int j = 0; j < J; ++j) {
				q = __fadd_rn(q, __fmul_rn(mv[j], mv[j]));
				s = __fadd_rn(s, mv[j]);
			}
			for (int o = 16; o > 0; o >>= 1) {
				q = __fadd_rn(q, __shfl_xor_sync(0xffffffffu, q, o));
				s = __fadd_rn(s, __shfl_xor_sync(0xffffffffu, s, o));
			}
			if (lane != 0)
				return;
			const float fw = static_cast<float>(kDetectBins);
			const float var = __fdiv_rn(__fsub_rn(q, __fdiv_rn(__fmul_rn(s, s), fw)), static_cast<float>(kDetectBins - 1));
			const float sigma = __fsqrt_rn(var);
			int c = 0;
#pragma unroll
			for (int r = 0; r < kMaxCandidates; ++r) {
				// double(peak) / double(sigma) < 6 exactly when peak - 6 sigma < 0
				// (two floats' double quotient cannot round onto 6 unless it is 6),
				// and fmaf rounds that difference once, keeping its sign: the
				// reference's double test without FP64 (a NaN stays, as in
				// remove_if(jn < threshold)).  The kept J/N is the float quotient.
				if (!(fmaf(-kJnThreshold, sigma, peaks[r]) < 0.0f)) {
					d.bins[static_cast<size_t>(c) * cols + col] = static_cast<uint8_t>(bins[r]);
					d.jn[static_cast<size_t>(c) * cols + col] = __fdiv_rn(peaks[r], sigma);
					atomicAdd(&s_hist[c * kDetectBins + bins[r]], 1);
					++c;
				}
			}
			for (int r = c; r < kMaxCandidates; ++r)
				d.bins[static_cast<size_t>(r) * cols + col] = kNoBin;
			atomicAdd(s_total, static_cast<unsigned int>(c));
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
		}

		// 128-point DFT of one warp in registers: lane l holds v[j] =
		// x[l + 32 j]; a radix-4 step over j, the twiddle W_128^{l k1}, then per
		// k1 a 32-point DFT across the lanes in five radix-2
		// decimation-in-frequency shuffle stages (h = 16 .. 1).  Lane l then
		// holds X[k1 + 4 rev5(l)] in v[k1] (X[k1 + 4 k2] = sum_l W_128^{l k1}
		// W_32^{l k2} sum_j x[l + 32 j] W_4^{j k1}).  The inverse runs the
		// network backwards with conjugate twiddles, from that layout back to
		// x[l + 32 j], unnormalised (x 128).  No shared memory, no barrier.
		struct Warp128 {
			float2 tw[3];  // W_128^{l k1}, k1 = 1..3
			float2 ts[5];  // W_{2h}^{l mod h}, h = 16, 8, 4, 2, 1
			__device__ __forceinline__ void init(const float2* tab, int lane) {
#pragma unroll
				for (int k1 = 1; k1 < 4; ++k1)
					tw[k1 - 1] = tab[(lane * k1) & 127];
#pragma unroll
				for (int st = 0; st < 5; ++st) {
					const int h = 16 >> st;
					ts[st] = tab[(lane & (h - 1)) * (64 / h)];
				}
			}
			__device__ __forceinline__ static int natural(int j, int lane) { return j + 4 * static_cast<int>(__brev(lane) >> 27); }
			__device__ __forceinline__ void forward(float2 (&v)[4], int lane) const {
				const float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
				const float2 b0 = cadd(v[1], v[3]), dd = csub(v[1], v[3]);
				const float2 b1 = c2(dd.y, -dd.x);  // (v1 - v3)(-i)
				v[0] = cadd(a0, b0);
				v[2] = csub(a0, b0);
				v[1] = cadd(a1, b1);
				v[3] = csub(a1, b1);
#pragma unroll
				for (int k1 = 1; k1 < 4; ++k1)
					v[k1] = cmul(v[k1], tw[k1 - 1]);
#pragma unroll
				for (int st = 0; st < 5; ++st) {
					const int h = 16 >> st;
					const bool hi = (lane & h) != 0;
#pragma unroll
					for (int j = 0; j < 4; ++j) {
						const float2 o = c2(__shfl_xor_sync(0xffffffffu, v[j].x, h), __shfl_xor_sync(0xffffffffu, v[j].y, h));
						v[j] = hi ? cmul(csub(o, v[j]), ts[st]) : cadd(v[j], o);
					}
				}
			}
			__device__ __forceinline__ void inverse(float2 (&v)[4], int lane) const {
#pragma unroll
				for (int st = 4; st >= 0; --st) {
					const int h = 16 >> st;
					const bool hi = (lane & h) != 0;
#pragma unroll
					for (int j = 0; j < 4; ++j) {
						const float2 q = hi ? cmulc(v[j], ts[st]) : v[j];
						const float2 o = c2(__shfl_xor_sync(0xffffffffu, q.x, h), __shfl_xor_sync(0xffffffffu, q.y, h));
						v[j] = hi ? csub(o, q) : cadd(q, o);
					}
				}
#pragma unroll
				for (int k1 = 1; k1 < 4; ++k1)
					v[k1] = cmulc(v[k1], tw[k1 - 1]);
				const float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
				const float2 b0 = cadd(v[1], v[3]), dd = csub(v[1], v[3]);
				const float2 b1 = c2(-dd.y, dd.x);  // (v1 - v3)(+i)
				v[0] = cadd(a0, b0);
				v[2] = csub(a0, b0);
				v[1] = cadd(a1, b1);
				v[3] = csub(a1, b1);
			}
		};

		struct DetectParams {
			const float2* x;       // samples; column c starts at 32 c
			int cols;
			const float* window;   // 128 Hann coefficients
			const float2* tw;      // W_128^m, m < 128
			DetectScratch det;
		};

		// JammingDetector's STFT and per-column candidates, one warp per column
		// (grid-stride), the column's transform in registers (Warp128)
		__global__ void __launch_bounds__(kJamThreads) detect_kernel(DetectParams p) {
			__shared__ float2 tab[kDetectBins];
			__shared__ int s_hist[kMaxCandidates * kDetectBins];
			__shared__ unsigned int s_total;
			for (int e = threadIdx.x; e < kDetectBins; e += blockDim.x)
				tab[e] = p.tw[e];
			for (int e = threadIdx.x; e < kMaxCandidates * kDetectBins; e += blockDim.x)
				s_hist[e] = 0;
			if (threadIdx.x == 0)
				s_total = 0;
			__syncthreads();
			const int lane = threadIdx.x & 31;
			Warp128 fft;
			fft.init(tab, lane);
			float win[4];
			int idx[4];
#pragma unroll
			for (int j = 0; j < 4; ++j) {
				win[j] = p.window[lane + 32 * j];
				idx[j] = Warp128::natural(j, lane);
			}
			const int warps = gridDim.x * (blockDim.x >> 5);
			for (int c = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); c < p.cols; c += warps) {
				const float2* xc = p.x + static_cast<size_t>(c) * 32;
				float2 v[4];
#pragma unroll
				for (int j = 0; j < 4; ++j) {
					const float2 smp = xc[lane + 32 * j];
					// vec * complex(window, 0) (stft.hpp:55-56): both parts scaled
					v[j] = c2(__fmul_rn(smp.x, win[j]), __fmul_rn(smp.y, win[j]));
				}
				fft.forward(v, lane);
				float mv[4];
#pragma unroll
				for (int j = 0; j < 4; ++j)
					mv[j] = magnitude(v[j]);
				detect_column(mv, idx, p.det, static_cast<size_t>(c), static_cast<size_t>(p.cols), s_hist, &s_total);
			}
			__syncthreads();
			for (int e = threadIdx.x; e < kMaxCandidates * kDetectBins; e += blockDim.x)
				if (s_hist[e])
					atomicAdd(p.det.hist + e, s_hist[e]);
			if (threadIdx.x == 0 && s_total)
				atomicAdd(p.det.total, static_cast<unsigned long long>(s_total));
		}

		struct IstftParams {
			const float2* s;       // cols x w
			int w;
			int cols;
			int per_cta;
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
				a[f * ld + i] = p.s[static_cast<size_t>(c0 + f) * w + i];
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

		struct WidebandParams {
			const float2* x;       // n input samples
			uint64_t n;
			int cols;
			int slots_per_warp;    // 32-sample output slots per warp
			const float* window;
			const float2* tw;      // W_128^m, m < 128
			float2* out;           // n output samples (not x)
		};

		// FilterWideband (jse.hpp:70-87) + OverlapAndAdd + resize to n, one warp
		// per run of 32-sample output slots: it walks the covering columns in
		// order (its first slot's three predecessors first), re-transforming each
		// from the samples as the detector did (Warp128), zeroing |.| >= 20,
		// inverse-transforming and scaling (v / 128) * 2; column i's value j
		// belongs to slot i + j, so four slot accumulators per lane take the
		// columns in column order, and slot i is complete after column i.
		__global__ void __launch_bounds__(kJamThreads) wideband_kernel(WidebandParams p) {
			__shared__ float2 tab[kDetectBins];
			for (int e = threadIdx.x; e < kDetectBins; e += blockDim.x)
				tab[e] = p.tw[e];
			__syncthreads();
			const int lane = threadIdx.x & 31;
			const long long total_slots = static_cast<long long>((p.n + 31) / 32);
			const long long s0 = (static_cast<long long>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5)) * p.slots_per_warp;
			if (s0 >= total_slots)
				return;
			const long long s1 = min(s0 + p.slots_per_warp, total_slots);
			Warp128 fft;
			fft.init(tab, lane);
			float win[4];
#pragma unroll
			for (int j = 0; j < 4; ++j)
				win[j] = p.window[lane + 32 * j];
			const float fw = static_cast<float>(kDetectBins);
			float2 acc[4];
#pragma unroll
			for (int j = 0; j < 4; ++j)
				acc[j] = c2(0.0f, 0.0f);
			auto put = [&](long long s, float2 v) {
				const uint64_t k = static_cast<uint64_t>(s) * 32 + lane;
				if (k < p.n)
					p.out[k] = v;
			};
			const long long i_lo = max(0LL, s0 - 3);
			const long long i_hi = min(static_cast<long long>(p.cols) - 1, s1 - 1);
			for (long long i = i_lo; i <= i_hi; ++i) {
				const float2* xc = p.x + static_cast<size_t>(i) * 32;
				float2 v[4];
#pragma unroll
				for (int j = 0; j < 4; ++j) {
					const float2 smp = xc[lane + 32 * j];
					v[j] = c2(__fmul_rn(smp.x, win[j]), __fmul_rn(smp.y, win[j]));
				}
				fft.forward(v, lane);
#pragma unroll
				for (int j = 0; j < 4; ++j)
					if (magnitude(v[j]) >= kWidebandLevel)
						v[j] = c2(0.0f, 0.0f);
				fft.inverse(v, lane);
#pragma unroll
				for (int j = 0; j < 4; ++j) {
					const long long s = i + j;
					if (s >= s0 && s < s1) {
						float2& a = acc[s & 3];
						a = c2(__fadd_rn(a.x, __fmul_rn(__fdiv_rn(v[j].x, fw), 2.0f)),
							__fadd_rn(a.y, __fmul_rn(__fdiv_rn(v[j].y, fw), 2.0f)));
					}
				}
				if (i >= s0) {
					put(i, acc[i & 3]);
					acc[i & 3] = c2(0.0f, 0.0f);
				}
			}
			// past the last column: the synthesis tail (slots cols .. cols + 2),
			// then the zeros of the resize to n
			const long long len_slots = static_cast<long long>(p.cols) + 3;
			for (long long s = max(s0, static_cast<long long>(p.cols)); s < s1; ++s)
				put(s, s < len_slots ? acc[s & 3] : c2(0.0f, 0.0f));
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

		// STFT of device samples x into ctx->jam_s (the per-op Transform)
		void stft_device(ugsdr_ctx* ctx, const float2* x, size_t cols, int w, int overlap) {
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
			KernelTimer timer(ctx, "jam_stft");
			with_column_fft(w, [&](auto f) {
				using F = decltype(f);
				UG_CUDA(cudaFuncSetAttribute(stft_kernel<F>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
				stft_kernel<F><<<static_cast<unsigned>((cols + per - 1) / per), kJamThreads, smem, ctx->stream>>>(p);
				note_launch(ctx);
			});
		}

		// inverse columns of ctx->jam_s into ctx->jam_t, overlap-added into n
		// samples at out
		void istft_device(ugsdr_ctx* ctx, size_t cols, int w, int overlap, float2* out, size_t n) {
			size_t smem = 0;
			const int per = columns_per_cta(ctx, w, smem);
			ctx->jam_t.reserve(sizeof(float2) * cols * w);
			IstftParams p{};
			p.s = ctx->jam_s.as<float2>();
			p.w = w;
			p.cols = static_cast<int>(cols);
			p.per_cta = per;
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

		int grid_for_warps(ugsdr_ctx* ctx, long long warps) {
			const long long per_cta = kJamThreads / 32;
			return static_cast<int>(std::max<long long>(1, std::min<long long>((warps + per_cta - 1) / per_cta,
				static_cast<long long>(ctx->sm_count) * 64)));
		}

		// FilterWideband + OverlapAndAdd + resize to n, fused: x -> out
		void wideband_device(ugsdr_ctx* ctx, const float2* x, size_t n, float2* out) {
			constexpr int kSlotsPerWarp = 64;
			WidebandParams p{};
			p.x = x;
			p.n = n;
			p.cols = static_cast<int>(stft_columns(n, kDetectWindow, kDetectOverlap));
			p.slots_per_warp = kSlotsPerWarp;
			p.window = hann_window(ctx, kDetectWindow);
			p.tw = get_plan(ctx, kDetectWindow).tw;
			p.out = out;
			const long long warps = (static_cast<long long>((n + 31) / 32) + kSlotsPerWarp - 1) / kSlotsPerWarp;
			const long long ctas = (warps + kJamThreads / 32 - 1) / (kJamThreads / 32);
			require(ctas < (1LL << 31), "signal too long");
			KernelTimer timer(ctx, "jam_wideband");
			wideband_kernel<<<static_cast<unsigned>(ctas), kJamThreads, 0, ctx->stream>>>(p);
			note_launch(ctx);
		}

		// deterministic block sum of per-thread doubles (fixed tree order)
		__device__ double block_sum(double v, double* scratch) {
			for (int o = 16; o > 0; o >>= 1)
				v += __shfl_down_sync(0xffffffffu, v, o);
			const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
			__syncthreads();
			if (lane == 0)
				scratch[warp] = v;
			__syncthreads();
			if (warp == 0) {
				v = lane < (blockDim.x >> 5) ? scratch[lane] : 0.0;
				for (int o = 16; o > 0; o >>= 1)
					v += __shfl_down_sync(0xffffffffu, v, o);
				if (lane == 0)
					scratch[0] = v;
			}
			__syncthreads();
			return scratch[0];
		}

		// AnalyzeStftData (jamming_detection.hpp:130-189), decisions.  Round i
		// looks at every column's i-th candidate: its occupation map is keyed
		// by frequency = bin * fs / w, which orders as the bins do, so the
		// reference's walk over the map is a walk over occupied bins in
		// increasing order of the round's histogram.
		__global__ void decide_kernel(DetectScratch d, unsigned long long cols) {
			if (threadIdx.x != 0)
				return;
			const int rounds = static_cast<int>(*d.total / cols);
			for (int i = 0; i < rounds; ++i) {
				const int* occ = d.hist + i * kDetectBins;
				double quantity = 0;
				int occupied = 0;
				for (int b = 0; b < kDetectBins; ++b)
					if (occ[b]) {
						quantity += occ[b];
						++occupied;
					}
				int narrow = -1, wide = -1, first = -1;
				unsigned long long cnt_wideband = 0;
				for (int b = 0; b < kDetectBins; ++b) {
					if (!occ[b])
						continue;
					if (first < 0)
						first = b;
					const double probability = occ[b] / quantity;
					if (probability >= kProbability) {
						narrow = b;
						break;
					}
					if (probability >= kProbability / static_cast<double>(occupied)) {
						++cnt_wideband;
						wide = b;
					}
				}
				if (wide < 0)
					wide = first;  // the reference's pointer starts at the map's first entry
				d.picks[2 * i] = narrow;
				// one occupied bin makes the bound 0: reported as wideband too
				d.picks[2 * i + 1] = cnt_wideband >= static_cast<unsigned long long>(occupied * kProbability) ? wide : -1;
				d.quantity[i] = quantity;
			}
			*d.rounds = rounds;
		}

		// The reported J/N of each pick: the mean of the round's candidate J/N
		// at that bin.  Per-CTA partial sums over a fixed column split, combined
		// in CTA order by the last CTA, which also writes the detection list —
		// deterministic, within rounding of the reference's column-order sum.
		__global__ void __launch_bounds__(kJamThreads) jn_sum_kernel(DetectScratch d, unsigned long long cols, double fs) {
			__shared__ double scratch[32];
			__shared__ bool s_last;
			const int rounds = *d.rounds;
			for (int i = 0; i < rounds; ++i)
				for (int k = 0; k < 2; ++k) {
					const int b = d.picks[2 * i + k];
					if (b < 0)
						continue;
					double part = 0;
					const uint8_t* bins = d.bins + static_cast<size_t>(i) * cols;
					const float* jn = d.jn + static_cast<size_t>(i) * cols;
					for (unsigned long long c = blockIdx.x * static_cast<unsigned long long>(blockDim.x) + threadIdx.x; c < cols;
						 c += static_cast<unsigned long long>(gridDim.x) * blockDim.x)
						if (bins[c] == b)
							part += jn[c];
					const double sum = block_sum(part, scratch);
					if (threadIdx.x == 0)
						d.partials[blockIdx.x * kMaxDetections + 2 * i + k] = sum;
				}
			__syncthreads();
			if (threadIdx.x == 0) {
				__threadfence();
				s_last = atomicAdd(d.done, 1u) == gridDim.x - 1;
			}
			__syncthreads();
			if (!s_last || threadIdx.x != 0)
				return;
			__threadfence();
			int n = 0;
			for (int i = 0; i < rounds; ++i)
				for (int k = 0; k < 2; ++k) {
					const int b = d.picks[2 * i + k];
					if (b < 0 || n >= kMaxDetections)
						continue;
					double sum = 0;
					for (unsigned int g = 0; g < gridDim.x; ++g)
						sum += __ldcg(d.partials + g * kMaxDetections + 2 * i + k);
					Detection& out = d.list->d[n++];
					out.type = k == 0 ? UGSDR_INTERFERENCE_NARROWBAND : UGSDR_INTERFERENCE_WIDEBAND;
					out.bin = b;
					out.frequency = static_cast<double>(b) * fs / static_cast<double>(kDetectBins);
					out.jn = sum / d.quantity[i];
				}
			d.list->n = n;
		}

		// detector over device samples x (n): STFT + candidates, decisions and
		// J/N sums on the device; only the detection list comes back
		std::vector<Detection> detect_device(ugsdr_ctx* ctx, const float2* x, size_t n, double fs) {
			require(fs > 0, "sampling rate must be positive");
			const size_t cols = stft_columns(n, kDetectWindow, kDetectOverlap);
			const DetectLayout lay(cols);
			ctx->jam_cand.reserve(lay.bytes);
			const DetectScratch d = lay.carve(ctx->jam_cand.ptr);
			UG_CUDA(cudaMemsetAsync(ctx->jam_cand.ptr, 0, lay.zero_bytes, ctx->stream));
			DetectParams dp{};
			dp.x = x;
			dp.cols = static_cast<int>(cols);
			dp.window = hann_window(ctx, kDetectWindow);
			dp.tw = get_plan(ctx, kDetectWindow).tw;
			dp.det = d;
			{
				KernelTimer timer(ctx, "jam_stft_detect");
				detect_kernel<<<grid_for_warps(ctx, static_cast<long long>(cols)), kJamThreads, 0, ctx->stream>>>(dp);
			}
			note_launch(ctx);
			decide_kernel<<<1, 32, 0, ctx->stream>>>(d, cols);
			jn_sum_kernel<<<kSumCtas, kJamThreads, 0, ctx->stream>>>(d, cols, fs);
			note_launch(ctx, 2);
			DetectionList host{};
			UG_CUDA(cudaMemcpyAsync(&host, d.list, sizeof(DetectionList), cudaMemcpyDeviceToHost, ctx->stream));
			UG_CUDA(cudaStreamSynchronize(ctx->stream));
			return std::vector<Detection>(host.d, host.d + std::min(host.n, kMaxDetections));
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
		stft_device(ctx, x, cols, window_length, overlap_length);
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
		istft_device(ctx, n_columns, window_length, overlap_length, ctx->jam_x.as<float2>(), len);
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
			// out of place (a tile reads its neighbours' inputs), then back
			ctx->jam_t.reserve(sizeof(float2) * n);
			wideband_device(ctx, x, n, ctx->jam_t.as<float2>());
			if (samples_on_device)
				UG_CUDA(cudaMemcpyAsync(x, ctx->jam_t.ptr, sizeof(float2) * n, cudaMemcpyDeviceToDevice, ctx->stream));
			else
				x = ctx->jam_t.as<float2>();
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

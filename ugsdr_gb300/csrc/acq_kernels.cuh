// Device kernels of the batched acquisition engine (single-CTA FFT sizes).
//
// Replaces, for one search, the reference's per-(PRN, Doppler) chain
//   TableMixer::Translate -> SequentialMatchedFilter::FilterOptimized ->
//   GetOneMsPeak (Abs, ReshapeAndSum) -> MaxIndex, MeanStdDev
// (src/acquisition/fse.hpp:250-269) by three fused kernels:
//   code_spectrum_kernel   conj(FFT(upsampled code)), once per code, cached
//   acq_forward_kernel     int8/int16/float samples -> LUT-NCO Doppler mix ->
//                          forward FFT, once per (Doppler, block): the mixed
//                          spectrum does not depend on the PRN, so it is not
//                          recomputed per PRN as the reference does (fse.hpp:253)
//   acq_inverse_kernel     per (code, Doppler) row: X * C -> inverse FFT ->
//                          scale -> |.| or |.|^2 -> fold -> accumulate over the
//                          K blocks in shared memory -> first-max / mean / std
//                          -> one 16-byte cell record to HBM
// plus acq_select_kernel (per code: first strictly greater level over Doppler,
// fse.hpp:265).
#pragma once

#include "fft_core.cuh"
#include "../../include/ugsdr_cuda.h"

#include <cstdint>

namespace ugsdr_gpu {

	struct FftPlanDev {
		int n;
		int n_pass;
		int radix[12];
		const float2* tw;
	};

	struct AcqCellDev {
		float level;
		uint32_t index;
		float mean;
		float std;
	};

	// ------------------------------------------------------------ samples
	template <int ST>
	__device__ __forceinline__ float2 load_sample(const void* base, size_t i) {
		if constexpr (ST == UGSDR_SAMPLES_CF32) {
			return static_cast<const float2*>(base)[i];
		}
		else if constexpr (ST == UGSDR_SAMPLES_CI8) {
			const char2 v = static_cast<const char2*>(base)[i];
			return c2(static_cast<float>(v.x), static_cast<float>(v.y));
		}
		else if constexpr (ST == UGSDR_SAMPLES_CI16) {
			const short2 v = static_cast<const short2*>(base)[i];
			return c2(static_cast<float>(v.x), static_cast<float>(v.y));
		}
		else {
			const signed char v = static_cast<const signed char*>(base)[i];
			return c2(static_cast<float>(v), 0.f);
		}
	}

	// TableMixer sample i: exp index = top 6 bits of the 32-bit NCO holder
	// (phase0 + i * adder mod 2^32, i.e. i additions of the adder), then the
	// complex<float> product evaluated without contraction, as the reference's
	// std::complex<float> multiply (table_mixer.hpp:86-97).
	// The same product from the holder itself (callers that step it: sample
	// i + d has holder + d * adder mod 2^32)
	__device__ __forceinline__ float2 table_mix_holder(float2 x, uint32_t holder, const float* lut) {
		const uint32_t idx = holder >> 26;
		const float c = lut[idx + 16], s = lut[idx];
		return c2(__fsub_rn(__fmul_rn(x.x, c), __fmul_rn(x.y, s)), __fadd_rn(__fmul_rn(x.x, s), __fmul_rn(x.y, c)));
	}
	__device__ __forceinline__ float2 table_mix(float2 x, uint64_t i, uint32_t adder, uint32_t phase0, const float* lut) {
		return table_mix_holder(x, phase0 + static_cast<uint32_t>(i * static_cast<uint64_t>(adder)), lut);
	}

	// ------------------------------------------------------------- passes
	// Runs every Stockham pass of `plan` with the whole CTA; returns the
	// buffer holding the result (a or b).
	template <bool INV>
	__device__ float2* fft_passes(float2* a, float2* b, const FftPlanDev& plan) {
		int ns = 1;
		for (int s = 0; s < plan.n_pass; ++s) {
			const int r = plan.radix[s];
			const int nb = plan.n / r;
			const float inv_ns = 1.0f / static_cast<float>(ns);
			for (int j = threadIdx.x; j < nb; j += blockDim.x)
				butterfly_dispatch<INV>(r, a, b, plan.n, ns, plan.tw, j, j - fdiv(j, inv_ns) * ns);
			__syncthreads();
			float2* t = a;
			a = b;
			b = t;
			ns *= r;
		}
		return a;
	}

	// -------------------------------------------------------------- codes
	struct CodeSpecParams {
		const float* chips;
		int n_chips;
		int repeats;
		uint32_t sign_mask;
		int sign_segment;
		int one_sided;
		float2* out;
		FftPlanDev plan;
	};

	// RepeatCodeNTimes + SequentialUpsampler (common.hpp:78-85, upsampler.hpp:30-37):
	// sample i takes chip ((i * L / S) % L) % len, L = len * repeats.
	__device__ __forceinline__ float code_sample(const float* chips, int n_chips, int repeats, int n, int i,
		uint32_t sign_mask, int sign_segment) {
		const uint64_t total = static_cast<uint64_t>(n_chips) * repeats;
		const uint64_t pos = (static_cast<uint64_t>(i) * total / static_cast<uint64_t>(n)) % total;
		float v = chips[pos % n_chips];
		if (sign_segment > 0) {
			const int seg = i / sign_segment;
			if (seg < 32 && ((sign_mask >> seg) & 1u))
				v = -v;
		}
		return v;
	}

	static __global__ void code_spectrum_kernel(CodeSpecParams p) {
		extern __shared__ float2 smem[];
		float2* a = smem;
		float2* b = smem + p.plan.n;
		const int n = p.plan.n;
		for (int i = threadIdx.x; i < n; i += blockDim.x)
			a[i] = c2(code_sample(p.chips, p.n_chips, p.repeats, n, i, p.sign_mask, p.sign_segment), 0.f);
		__syncthreads();
		float2* y = fft_passes<false>(a, b, p.plan);
		for (int i = threadIdx.x; i < n; i += blockDim.x) {
			const float2 v = y[i];
			// SequentialConj; one-sided: r2c leaves bins above N/2 zero
			p.out[i] = (p.one_sided && i > n / 2) ? c2(0.f, 0.f) : c2(v.x, -v.y);
		}
	}

	// --------------------------------------------------------- acquisition
	struct AcqParams {
		const void* samples;
		int n;              // block samples N
		int k_blocks;       // K
		int n_doppler;
		int n_codes;
		int m;              // output length after folding (N when not folded)
		int fold_mode;      // 0 none, 1 |.| then fold, 2 fold complex then |.|
		int stat;           // 0 |.|, 1 |.|^2
		int one_sided;
		const uint32_t* adders;       // per Doppler bin
		uint32_t phase0;
		uint32_t fe_adder;            // front-end Translate adder (used when fe_on)
		int fe_on;
		int d_base;                   // first Doppler bin of this launch (grid processed in chunks)
		const float* lut;             // 80-entry sine table
		float2* spectra;              // [d][b][N]
		const float2* const* codes;   // per code spectrum
		AcqCellDev* cells;            // [code][doppler]
		FftPlanDev plan;
	};

	template <int ST>
	__global__ void acq_forward_kernel(AcqParams p) {
		extern __shared__ float2 smem[];
		__shared__ float lut[80];
		float2* a = smem;
		float2* b = smem + p.n;
		const int d = blockIdx.x / p.k_blocks;
		const int blk = blockIdx.x % p.k_blocks;
		for (int i = threadIdx.x; i < 80; i += blockDim.x)
			lut[i] = p.lut[i];
		__syncthreads();
		const uint32_t adder = p.adders[p.d_base + d];
		const uint64_t base = static_cast<uint64_t>(blk) * p.n;
		for (int i = threadIdx.x; i < p.n; i += blockDim.x) {
			const uint64_t g = base + i;
			float2 v = load_sample<ST>(p.samples, g);
			if (p.fe_on)
				v = table_mix(v, g, p.fe_adder, 0u, lut);
			a[i] = table_mix(v, g, adder, p.phase0, lut);
		}
		__syncthreads();
		float2* y = fft_passes<false>(a, b, p.plan);
		float2* dst = p.spectra + (static_cast<size_t>(d) * p.k_blocks + blk) * p.n;
		const int limit = p.one_sided ? p.n / 2 + 1 : p.n;
		for (int i = threadIdx.x; i < limit; i += blockDim.x)
			dst[i] = y[i];
	}

	// |v| of a correlation sample: the hardware square-root approximation
	// (PTX sqrt.approx.f32, one instruction; exact at 0), whose relative error
	// is a few float ulps, far inside the search's 1e-4 tolerance
	__device__ __forceinline__ float sqrt_approx(float x) {
		float r;
		asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
		return r;
	}
	__device__ __forceinline__ float stat_of(float2 v, int stat) {
		const float q = v.x * v.x + v.y * v.y;
		return stat ? q : sqrt_approx(q);
	}

	// block-wide first-max / sum reduction helpers
	struct MaxIdx {
		float v;
		uint32_t i;
	};
	__device__ __forceinline__ MaxIdx better(MaxIdx a, MaxIdx b) {
		if (b.v > a.v || (b.v == a.v && b.i < a.i))
			return b;
		return a;
	}

	// reduces acc[0..m) into one cell (first maximum, mean, unbiased std)
	static __device__ void reduce_cell(const float* acc, int m, AcqCellDev* out) {
		__shared__ MaxIdx s_max[32];
		__shared__ double s_sum[32];
		__shared__ double s_mean;
		const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = (blockDim.x + 31) >> 5;
		MaxIdx best{-1.0f, 0xFFFFFFFFu};
		float sum = 0.f;
		for (int i = threadIdx.x; i < m; i += blockDim.x) {
			const float v = acc[i];
			if (v > best.v) {
				best.v = v;
				best.i = static_cast<uint32_t>(i);
			}
			sum += v;
		}
		double dsum = sum;
		for (int o = 16; o > 0; o >>= 1) {
			MaxIdx other{__shfl_down_sync(0xffffffffu, best.v, o), __shfl_down_sync(0xffffffffu, best.i, o)};
			best = better(best, other);
			dsum += __shfl_down_sync(0xffffffffu, dsum, o);
		}
		if (lane == 0) {
			s_max[warp] = best;
			s_sum[warp] = dsum;
		}
		__syncthreads();
		if (threadIdx.x == 0) {
			MaxIdx b0 = s_max[0];
			double t = s_sum[0];
			for (int w = 1; w < nwarp; ++w) {
				b0 = better(b0, s_max[w]);
				t += s_sum[w];
			}
			s_max[0] = b0;
			s_mean = t / m;
		}
		__syncthreads();
		const float mean = static_cast<float>(s_mean);
		float sq = 0.f;
		for (int i = threadIdx.x; i < m; i += blockDim.x) {
			const float dlt = acc[i] - mean;
			sq += dlt * dlt;
		}
		double dsq = sq;
		for (int o = 16; o > 0; o >>= 1)
			dsq += __shfl_down_sync(0xffffffffu, dsq, o);
		__syncthreads();
		if (lane == 0)
			s_sum[warp] = dsq;
		__syncthreads();
		if (threadIdx.x == 0) {
			double t = 0;
			for (int w = 0; w < nwarp; ++w)
				t += s_sum[w];
			AcqCellDev c;
			c.level = s_max[0].v;
			c.index = s_max[0].i;
			c.mean = static_cast<float>(s_mean);
			c.std = m > 1 ? static_cast<float>(sqrt(t / (m - 1))) : 0.f;
			*out = c;
		}
	}

	static __global__ void acq_inverse_kernel(AcqParams p) {
		extern __shared__ float2 smem[];
		float2* a = smem;
		float2* b = smem + p.n;
		float* acc = reinterpret_cast<float*>(smem + 2 * p.n);
		const int row = blockIdx.x;
		const int c = row % p.n_codes;
		const int d = row / p.n_codes;
		const int n = p.n;
		const float2* code = p.codes[c];
		const int half = n / 2;
		const float inv_n = 1.0f / static_cast<float>(n);
		const float post = p.one_sided ? 2.0f : 1.0f;
		for (int i = threadIdx.x; i < p.m; i += blockDim.x)
			acc[i] = 0.f;
		for (int blk = 0; blk < p.k_blocks; ++blk) {
			const float2* x = p.spectra + (static_cast<size_t>(d) * p.k_blocks + blk) * n;
			for (int i = threadIdx.x; i < n; i += blockDim.x)
				a[i] = (p.one_sided && i > half) ? c2(0.f, 0.f) : cmul(__ldg(x + i), __ldg(code + i));
			__syncthreads();
			const float2* y = fft_passes<true>(a, b, p.plan);
			// y / N * 2 (dft.hpp:194-198) or y / N, then GetOneMsPeak
			if (p.fold_mode == 0) {
				for (int i = threadIdx.x; i < n; i += blockDim.x) {
					const float2 v = cscale(cscale(y[i], inv_n), post);
					acc[i] += stat_of(v, p.stat);
				}
			}
			else if (p.fold_mode == 1) {
				const int folds = n / p.m;
				for (int i = threadIdx.x; i < p.m; i += blockDim.x) {
					float s = 0.f;
					for (int f = 0; f < folds; ++f)
						s += stat_of(cscale(cscale(y[i + f * p.m], inv_n), post), p.stat);
					acc[i] += s;
				}
			}
			else {
				const int folds = n / p.m;
				for (int i = threadIdx.x; i < p.m; i += blockDim.x) {
					float2 s = c2(0.f, 0.f);
					for (int f = 0; f < folds; ++f)
						s = cadd(s, cscale(cscale(y[i + f * p.m], inv_n), post));
					acc[i] += stat_of(s, p.stat);
				}
			}
			__syncthreads();
		}
		reduce_cell(acc, p.m, p.cells + static_cast<size_t>(c) * p.n_doppler + p.d_base + d);
	}

	// per code: keep the first Doppler with a strictly greater level (fse.hpp:265)
	static __global__ void acq_select_kernel(const AcqCellDev* cells, int n_codes, int n_doppler, int* best_bin) {
		const int c = blockIdx.x * blockDim.x + threadIdx.x;
		if (c >= n_codes)
			return;
		const AcqCellDev* row = cells + static_cast<size_t>(c) * n_doppler;
		int best = 0;
		float lvl = row[0].level;
		for (int d = 1; d < n_doppler; ++d)
			if (lvl < row[d].level) {
				lvl = row[d].level;
				best = d;
			}
		best_bin[c] = best;
	}
}

// Compile-time FFT plans for the sub-transform sizes of the four-step path.
//
// The runtime Stockham passes (acq_batched.cuh passes_batch) switch on the
// radix per butterfly and derive every index from runtime sizes.  For the
// block sizes the configurations use (1 ms at 50 MHz: 200 x 250; 4 ms at
// 50 MHz: 400 x 500; 10 ms at 20.46 MHz: 440 x 465) the plan is a type:
// radices, strides and twiddle steps are constants, index division is by
// constants, and each pass's butterfly loop is the only runtime loop.
// Arithmetic per butterfly is the same Dft<R> as the runtime path.
#pragma once

#include "acq_kernels.cuh"

namespace ugsdr_gpu {

	// One radix-R Stockham pass of an N-point transform whose previous passes
	// span NS points, over `batch` transforms at a[f * ld + i] (whole CTA).
	template <int N, int R, int NS, bool INV>
	__device__ __forceinline__ void static_pass(const float2* __restrict__ in, float2* __restrict__ out, const float2* __restrict__ tw,
		int batch, int ld) {
		constexpr int NB = N / R;           // butterflies per transform
		constexpr int TW_STEP = N / (NS * R);
		const int total = NB * batch;
		for (int u = threadIdx.x; u < total; u += blockDim.x) {
			const int f = u / NB;
			const int j = u - f * NB;
			const int k = NS == 1 ? 0 : j % NS;
			const float2* src = in + f * ld + j;
			float2 v[R];
#pragma unroll
			for (int r = 0; r < R; ++r)
				v[r] = src[r * NB];
			if constexpr (NS > 1) {
				const int step = TW_STEP * k;
#pragma unroll
				for (int r = 1; r < R; ++r) {
					const float2 w = tw[r * step];  // generic load: the table may sit in shared memory
					v[r] = INV ? cmulc(v[r], w) : cmul(v[r], w);
				}
			}
			Dft<R, INV>::run(v);
			float2* dst = out + f * ld + (j - k) * R + k;
#pragma unroll
			for (int r = 0; r < R; ++r)
				dst[r * NS] = v[r];
		}
	}

	// A plan: N = R0 * R1 * ... ; run() leaves the result in `a` or `b` and
	// returns it (Stockham ping-pong, one __syncthreads per pass).
	template <int N, int NS, bool INV, int... Rs>
	struct StaticPasses;

	template <int N, int NS, bool INV>
	struct StaticPasses<N, NS, INV> {
		__device__ static float2* run(float2* a, float2*, const float2*, int, int) { return a; }
	};

	template <int N, int NS, bool INV, int R, int... Rest>
	struct StaticPasses<N, NS, INV, R, Rest...> {
		__device__ static float2* run(float2* a, float2* b, const float2* tw, int batch, int ld) {
			static_pass<N, R, NS, INV>(a, b, tw, batch, ld);
			__syncthreads();
			return StaticPasses<N, NS * R, INV, Rest...>::run(b, a, tw, batch, ld);
		}
	};

	template <int... Rs>
	constexpr int radix_product() {
		return (1 * ... * Rs);
	}

	template <int... Rs>
	constexpr int radix_min() {
		int m = 1 << 30;
		((m = Rs < m ? Rs : m), ...);
		return m;
	}

	// An N-point FFT policy for the batched kernels; the twiddle table is the
	// runtime plan's table of the same size, exp(-2 pi i m / N).
	template <int N_, int... Rs>
	struct StaticFft {
		static_assert(radix_product<Rs...>() == N_, "radices must multiply to N");
		static constexpr int N = N_;
		// most butterflies of one pass over `batch` transforms
		static constexpr int most_butterflies(int batch) { return batch * (N_ / radix_min<Rs...>()); }
		template <bool INV>
		__device__ static float2* run(float2* a, float2* b, const FftPlanDev& plan, int batch, int ld) {
			return StaticPasses<N_, 1, INV, Rs...>::run(a, b, plan.tw, batch, ld);
		}
	};
}

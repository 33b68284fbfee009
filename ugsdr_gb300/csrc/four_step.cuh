// Single-CTA four-step transform for the per-op DFT entry (ugsdr_dft and the
// matched filter on sizes above one CTA's shared memory): one CTA runs
//   x[N2 n1 + n2] --(N1-point FFTs over n1, twiddle W_N^{n2 k1})-->
//   A[k1][n2] --(N2-point FFTs over n2)--> X_T[k1][k2] = X[k1 + N1 k2]
// using its output buffer as the transpose scratch.  The acquisition engine
// uses the batched kernels of acq_batched.cuh instead.
#pragma once

#include "acq_kernels.cuh"

namespace ugsdr_gpu {

	// Stockham passes over `batch` independent FFTs laid out at a[f * n + i].
	template <bool INV>
	__device__ float2* fft_passes_batch(float2* a, float2* b, const FftPlanDev& plan, int batch) {
		int ns = 1;
		const int n = plan.n;
		for (int s = 0; s < plan.n_pass; ++s) {
			const int r = plan.radix[s];
			const int nb = n / r;
			const int total = nb * batch;
			for (int u = threadIdx.x; u < total; u += blockDim.x) {
				const int f = u / nb;
				const int j = u - f * nb;
				butterfly_dispatch<INV>(r, a + f * n, b + f * n, n, ns, plan.tw, j, j % ns);
			}
			__syncthreads();
			float2* t = a;
			a = b;
			b = t;
			ns *= r;
		}
		return a;
	}

	struct LargeParams {
		AcqParams base;
		FftPlanDev p1, p2;       // N1- and N2-point plans
		int n1, n2;
		int cw, rw;              // columns / rows per tile
		const float2* tw;        // N-point table, W_N^m = exp(-2 pi i m/N)
		float2* slab;            // per CTA: N complex (B) + M floats (acc) + M complex (fold)
		size_t slab_elems;       // float2 units per CTA
		// code spectrum job
		const float* chips;
		int n_chips, repeats, sign_segment;
		uint32_t sign_mask;
		float2* code_out;
	};

	__device__ __forceinline__ float2 twiddle_n(const float2* tw, int n, uint64_t e, bool inv) {
		const float2 w = __ldg(tw + (e % static_cast<uint64_t>(n)));
		return inv ? c2(w.x, -w.y) : w;
	}

	// Forward four-step of one block whose samples come from `load(i)`;
	// output (and transpose scratch) is `out` in the k1-major layout.
	template <typename Load>
	__device__ void four_step_forward(const LargeParams& p, float2* tile_a, float2* tile_b, float2* out, Load load) {
		const int n1 = p.n1, n2 = p.n2, n = p.base.n;
		// columns: N1-point FFTs over n1 for each n2
		for (int c0 = 0; c0 < n2; c0 += p.cw) {
			const int cw = min(p.cw, n2 - c0);
			for (int e = threadIdx.x; e < cw * n1; e += blockDim.x) {
				const int f = e % cw, i1 = e / cw;
				tile_a[f * n1 + i1] = load(static_cast<int64_t>(n2) * i1 + c0 + f);
			}
			__syncthreads();
			const float2* y = fft_passes_batch<false>(tile_a, tile_b, p.p1, cw);
			for (int e = threadIdx.x; e < cw * n1; e += blockDim.x) {
				const int f = e % cw, k1 = e / cw;
				const float2 w = twiddle_n(p.tw, n, static_cast<uint64_t>(c0 + f) * k1, false);
				out[static_cast<size_t>(k1) * n2 + c0 + f] = cmul(y[f * n1 + k1], w);
			}
			__syncthreads();
		}
		// rows: N2-point FFTs over n2 for each k1, in place
		for (int r0 = 0; r0 < n1; r0 += p.rw) {
			const int rw = min(p.rw, n1 - r0);
			for (int e = threadIdx.x; e < rw * n2; e += blockDim.x)
				tile_a[e] = out[static_cast<size_t>(r0) * n2 + e];
			__syncthreads();
			const float2* y = fft_passes_batch<false>(tile_a, tile_b, p.p2, rw);
			for (int e = threadIdx.x; e < rw * n2; e += blockDim.x)
				out[static_cast<size_t>(r0) * n2 + e] = y[e];
			__syncthreads();
		}
	}
}

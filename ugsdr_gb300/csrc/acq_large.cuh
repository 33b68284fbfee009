// Large-N acquisition path: coherent blocks whose FFT does not fit one CTA's
// shared memory (N = 50,000 at 50 MHz / 1 ms, 200,000 for 4 ms, 204,600 for
// L5 at 20.46 MHz / 10 ms, up to 1,000,000).
//
// Four-step transform N = N1 * N2 run entirely by one CTA per work item,
// with a CTA-private slab in global memory (L2-resident) for the transpose:
//   forward  x[N2 n1 + n2] --(N1-point FFTs over n1, twiddle W_N^{n2 k1})-->
//            A[k1][n2] --(N2-point FFTs over n2)--> X_T[k1][k2] = X[k1 + N1 k2]
//   inverse  Z_T[k1][k2] --(N2-point IFFTs over k2, twiddle W_N^{-n2 k1})-->
//            B[k1][n2] --(N1-point IFFTs over k1)--> y[N2 n1 + n2]
// Spectra (signal and code) stay in the k1-major layout X_T, so the pointwise
// product needs no transpose.  Kernels are persistent (grid = resident CTAs),
// each CTA owning one slab, looping over work items.
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
				butterfly_dispatch<INV>(r, a + f * n, b + f * n, n, ns, plan.tw, j);
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

	template <int ST>
	__global__ void acq_forward_large_kernel(LargeParams p) {
		extern __shared__ float2 smem[];
		__shared__ float lut[80];
		const int tile = max(p.cw * p.n1, p.rw * p.n2);
		float2* tile_a = smem;
		float2* tile_b = smem + tile;
		if (threadIdx.x < 80)
			lut[threadIdx.x] = p.base.lut[threadIdx.x];
		__syncthreads();
		const int items = p.base.n_doppler * p.base.k_blocks;
		for (int item = blockIdx.x; item < items; item += gridDim.x) {
			const int d = item / p.base.k_blocks;
			const int blk = item % p.base.k_blocks;
			const uint32_t adder = p.base.adders[d];
			const uint64_t base = static_cast<uint64_t>(blk) * p.base.n;
			float2* out = p.base.spectra + static_cast<size_t>(item) * p.base.n;
			four_step_forward(p, tile_a, tile_b, out, [&](int64_t i) {
				const uint64_t g = base + static_cast<uint64_t>(i);
				float2 v = load_sample<ST>(p.base.samples, g);
				if (p.base.fe_on)
					v = table_mix(v, g, p.base.fe_adder, 0u, lut);
				return table_mix(v, g, adder, p.base.phase0, lut);
			});
		}
	}

	// code spectrum in the k1-major layout; one CTA
	static __global__ void code_spectrum_large_kernel(LargeParams p) {
		extern __shared__ float2 smem[];
		const int tile = max(p.cw * p.n1, p.rw * p.n2);
		float2* tile_a = smem;
		float2* tile_b = smem + tile;
		const int n = p.base.n;
		four_step_forward(p, tile_a, tile_b, p.code_out, [&](int64_t i) {
			return c2(code_sample(p.chips, p.n_chips, p.repeats, n, static_cast<int>(i), p.sign_mask, p.sign_segment), 0.f);
		});
		__syncthreads();
		const int half = n / 2;
		for (int e = threadIdx.x; e < n; e += blockDim.x) {
			const int k1 = e / p.n2, k2 = e % p.n2;
			const int64_t k = k1 + static_cast<int64_t>(p.n1) * k2;
			const float2 v = p.code_out[e];
			p.code_out[e] = (p.base.one_sided && k > half) ? c2(0.f, 0.f) : c2(v.x, -v.y);
		}
	}

	static __global__ void acq_inverse_large_kernel(LargeParams p) {
		extern __shared__ float2 smem[];
		const int tile = max(p.cw * p.n1, p.rw * p.n2);
		float2* tile_a = smem;
		float2* tile_b = smem + tile;
		const AcqParams& q = p.base;
		const int n1 = p.n1, n2 = p.n2, n = q.n, m = q.m;
		float2* bslab = p.slab + static_cast<size_t>(blockIdx.x) * p.slab_elems;
		float* acc = reinterpret_cast<float*>(bslab + n);
		float2* zc = bslab + n + (m + 1) / 2;  // complex fold accumulator (fold_mode 2)
		const int half = n / 2;
		const float inv_n = 1.0f / static_cast<float>(n);
		const float post = q.one_sided ? 2.0f : 1.0f;
		const int rows = q.n_codes * q.n_doppler;
		for (int row = blockIdx.x; row < rows; row += gridDim.x) {
			const int c = row % q.n_codes;
			const int d = row / q.n_codes;
			const float2* code = q.codes[c];
			for (int i = threadIdx.x; i < m; i += blockDim.x) {
				acc[i] = 0.f;
				if (q.fold_mode == 2)
					zc[i] = c2(0.f, 0.f);
			}
			__syncthreads();
			for (int blk = 0; blk < q.k_blocks; ++blk) {
				const float2* x = q.spectra + (static_cast<size_t>(d) * q.k_blocks + blk) * n;
				// rows: IFFT over k2 for each k1
				for (int r0 = 0; r0 < n1; r0 += p.rw) {
					const int rw = min(p.rw, n1 - r0);
					for (int e = threadIdx.x; e < rw * n2; e += blockDim.x) {
						const int ri = e / n2, k2 = e - ri * n2;
						const int64_t k = (r0 + ri) + static_cast<int64_t>(n1) * k2;
						const size_t at = static_cast<size_t>(r0) * n2 + e;
						tile_a[e] = (q.one_sided && k > half) ? c2(0.f, 0.f) : cmul(__ldg(x + at), __ldg(code + at));
					}
					__syncthreads();
					const float2* y = fft_passes_batch<true>(tile_a, tile_b, p.p2, rw);
					for (int e = threadIdx.x; e < rw * n2; e += blockDim.x) {
						const int ri = e / n2, i2 = e - ri * n2;
						const float2 w = twiddle_n(p.tw, n, static_cast<uint64_t>(i2) * (r0 + ri), true);
						bslab[static_cast<size_t>(r0) * n2 + e] = cmul(y[e], w);
					}
					__syncthreads();
				}
				// columns: IFFT over k1 for each n2
				for (int c0 = 0; c0 < n2; c0 += p.cw) {
					const int cw = min(p.cw, n2 - c0);
					for (int e = threadIdx.x; e < cw * n1; e += blockDim.x) {
						const int f = e % cw, k1 = e / cw;
						tile_a[f * n1 + k1] = bslab[static_cast<size_t>(k1) * n2 + c0 + f];
					}
					__syncthreads();
					const float2* y = fft_passes_batch<true>(tile_a, tile_b, p.p1, cw);
					for (int e = threadIdx.x; e < cw * n1; e += blockDim.x) {
						const int f = e % cw, i1 = e / cw;
						const int64_t tau = static_cast<int64_t>(n2) * i1 + c0 + f;
						const float2 v = cscale(cscale(y[f * n1 + i1], inv_n), post);
						if (q.fold_mode == 0)
							acc[tau] += stat_of(v, q.stat);
						else if (q.fold_mode == 1)
							atomicAdd(acc + (tau % m), stat_of(v, q.stat));
						else {
							float2* z = zc + (tau % m);
							atomicAdd(&z->x, v.x);
							atomicAdd(&z->y, v.y);
						}
					}
					__syncthreads();
				}
				if (q.fold_mode == 2) {
					for (int i = threadIdx.x; i < m; i += blockDim.x) {
						acc[i] += stat_of(zc[i], q.stat);
						zc[i] = c2(0.f, 0.f);
					}
					__syncthreads();
				}
			}
			reduce_cell(acc, m, q.cells + static_cast<size_t>(c) * q.n_doppler + d);
			__syncthreads();
		}
	}
}

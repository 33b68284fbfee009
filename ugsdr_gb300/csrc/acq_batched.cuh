// Large-N acquisition as batched two-stage transforms.
//
// For block sizes above one CTA's shared memory (N = 50,000 at 50 MHz / 1 ms,
// 200,000 at 4 ms, 204,600 for L5 at 20.46 MHz / 10 ms, up to 1,000,000) the
// N-point transform is split N = N1 * N2 (four-step) and each step is one
// kernel over every sub-transform of a batch, so every launch has thousands
// of independent CTAs:
//   forward   fwd_cols  x[N2 n1 + n2] -> N1-point FFTs over n1, times W_N^{n2 k1}
//             fwd_rows  N2-point FFTs over n2 -> X_T[k1][k2] = X[k1 + N1 k2]
//   inverse   inv_rows  Z_T = X_T * C_T -> N2-point IFFTs over k2, times W_N^{-n2 k1}
//                       -> B[row][block][k1][n2]
//             inv_cols  per (row, column chunk): for each block (the next
//                       block's tile prefetched with cp.async while the current
//                       one is transformed), N1-point IFFTs over k1 ->
//                       y[N2 n1 + n2] -> |.| or |.|^2 accumulated over the K
//                       blocks in shared memory -> chunk partial (first max,
//                       sum, sum of squares); the last CTA of a row combines
//                       the partials into the row's cell.
// Folded outputs (reshape, fse.hpp:209-218) accumulate through atomics into a
// per-row buffer reduced by a finishing kernel.
// Spectra (signal and code) stay in the k1-major layout X_T, so the pointwise
// product needs no transpose; only bins k <= N/2 are written/read one-sided.
#pragma once

#include "acq_kernels.cuh"
#include "fft_static.cuh"

namespace ugsdr_gpu {

	// Stockham passes over `batch` FFTs laid out at a[f * ld + i] (whole CTA).
	template <bool INV>
	__device__ float2* passes_batch(float2* a, float2* b, const FftPlanDev& plan, int batch, int ld) {
		int ns = 1;
		const int n = plan.n;
		for (int s = 0; s < plan.n_pass; ++s) {
			const int r = plan.radix[s];
			const int nb = n / r;
			const int total = nb * batch;
			const float inv_nb = 1.0f / static_cast<float>(nb), inv_ns = 1.0f / static_cast<float>(ns);
			for (int u = threadIdx.x; u < total; u += blockDim.x) {
				const int f = fdiv(u, inv_nb);
				const int j = u - f * nb;
				butterfly_dispatch<INV>(r, a + f * ld, b + f * ld, n, ns, plan.tw, j, j - fdiv(j, inv_ns) * ns);
			}
			__syncthreads();
			float2* t = a;
			a = b;
			b = t;
			ns *= r;
		}
		return a;
	}

	// The plan's twiddle table copied into shared memory at `dst` (16-byte
	// aligned, n entries); returns the plan pointing at the copy.  Call before
	// the CTA's first __syncthreads.
	__device__ __forceinline__ FftPlanDev plan_in_smem(const FftPlanDev& plan, void* dst, int n) {
		float2* t = reinterpret_cast<float2*>((reinterpret_cast<uintptr_t>(dst) + 15) & ~static_cast<uintptr_t>(15));
		for (int i = threadIdx.x; i < n; i += blockDim.x)
			t[i] = __ldg(plan.tw + i);
		FftPlanDev out = plan;
		out.tw = t;
		return out;
	}

	// FFT policy of the runtime plan (any plannable size); StaticFft is the
	// compile-time alternative for the configured sizes.
	struct RuntimeFft {
		static constexpr int N = 0;
		static constexpr bool kHooked = false;
		static constexpr int kPasses = 0;
		static constexpr int kLastNS = 0;
		static constexpr bool kRowsCompact = false;
		static constexpr int kRowsMaxThreads = 256;
		static constexpr int kRowsMinBlocks = 3;
		static constexpr bool kColsCompact = false;
		static constexpr int kColsMaxThreads = 256;
		static constexpr int kColsMinBlocks = 2;
		static constexpr int kFwdColsMinBlocks = 3;
		__device__ static FftPlanDev prepare(const FftPlanDev& plan, void* dst) { return plan_in_smem(plan, dst, plan.n); }
		template <bool INV>
		__device__ static float2* run(float2* a, float2* b, const FftPlanDev& plan, int batch, int ld) {
			return passes_batch<INV>(a, b, plan, batch, ld);
		}
	};

	// sub-transform length and division by it: constants for a static plan
	template <class F>
	__device__ __forceinline__ int fft_n(int runtime_n) {
		if constexpr (F::N > 0)
			return F::N;
		else
			return runtime_n;
	}
	template <class F>
	__device__ __forceinline__ int div_fft_n(int e, float inv_runtime_n) {
		if constexpr (F::N > 0)
			return e / F::N;
		else
			return fdiv(e, inv_runtime_n);
	}

	// W_N^e (conjugated when inv) for 0 <= e < N: sincospi of 2 e' / N with
	// e' = e or e - N reduced to (-N/2, N/2] (float argument error < 2^-24 of
	// the angle; the inter-step twiddle's contribution stays near 1e-7).
	__device__ __forceinline__ float2 tw_n(uint32_t e, uint32_t n, float inv_n2, bool inv) {
		const int32_t er = e > n / 2 ? static_cast<int32_t>(e) - static_cast<int32_t>(n) : static_cast<int32_t>(e);
		float s, c;
		sincospif(static_cast<float>(er) * inv_n2, &s, &c);
		return c2(c, inv ? s : -s);
	}

	__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
		const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
		asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem));
	}
	__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
		const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
		asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem));
	}
	__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
	__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

	struct BatchedParams {
		AcqParams base;         // n, k_blocks, n_doppler, n_codes, m, fold_mode, stat, one_sided, adders, lut, spectra, codes, cells
		FftPlanDev p1, p2;      // N1-point, N2-point plans
		int n1, n2;
		int n2p;                // blocked B layout (inv_cols_warp_kernel): N2 padded to a multiple of its CW
		int cw, rw;             // columns per column-kernel CTA (power of two), rows per row-kernel CTA
		int cw_shift;           // log2(cw)
		int ld1;                // column-tile stride: N1 rounded up to odd (conflict-free smem)
		// forward / code items
		int code_mode;          // 1: items are codes (chips -> spectra), 0: signal (Doppler, block)
		int row_keep;           // signal spectra: elements k2 < row_keep of each row stored (0: all)
		const float* chips;     // code mode: chips of code `item` at chips + item * chip_stride
		int n_chips, chip_stride, repeats, sign_segment;
		const uint32_t* sign_masks;
		float2* out;            // forward output base (item * N)
		// inverse batch
		int row0, rows;         // rows [row0, row0 + rows) of (code fastest, Doppler) in this batch
		float2* bbuf;           // B[row - row0][block][N]
		float4* partials;       // [row - row0][chunk]: (max, index bits, -, -)
		double2* sums;          // [row - row0][chunk]: (sum, sum of squares)
		unsigned int* counters; // [row - row0], zeroed per batch
		float* accg;            // fold modes: [row - row0][M]
		float2* zcg;            // fold mode 2: [row - row0][block][M]
	};

	// ----------------------------------------- single CTA, compile-time plan
	// acq_forward_kernel / acq_inverse_kernel for a block size whose plan is a
	// type (F::N): the mix-and-load is pass 0's gather and the spectrum store
	// (forward) or the |.| accumulation (inverse, unfolded) its last pass.
	template <int ST>
	struct SmallFwdLoad {
		const void* samples;
		const float* lut;
		uint64_t base;
		uint32_t adder, fe_adder, phase0;
		int fe_on;
		__device__ __forceinline__ float2 operator()(int, int i) const {
			const uint64_t g = base + static_cast<uint64_t>(i);
			float2 v = load_sample<ST>(samples, g);
			if (fe_on)
				v = table_mix(v, g, fe_adder, 0u, lut);
			return table_mix(v, g, adder, phase0, lut);
		}
	};
	struct SmallFwdEmit {
		float2* dst;
		int limit;  // one-sided: bins 0..N/2
		template <int R, int NS>
		__device__ __forceinline__ void put(int, int base, const float2 (&v)[R]) const {
#pragma unroll
			for (int r = 0; r < R; ++r)
				if (base + r * NS < limit)
					dst[base + r * NS] = v[r];
		}
	};
	// grid: Doppler bins x K blocks, one transform each
	template <int ST, class F>
	__global__ void __launch_bounds__(256) acq_forward_static_kernel(AcqParams p) {
		extern __shared__ float2 smem[];
		__shared__ float lut[80];
		float2* a = smem;
		float2* b = smem + F::N;
		const FftPlanDev plan = F::prepare(p.plan, smem + 2 * F::N);
		for (int i = threadIdx.x; i < 80; i += blockDim.x)
			lut[i] = p.lut[i];
		__syncthreads();
		const int d = blockIdx.x / p.k_blocks;
		const int blk = blockIdx.x - d * p.k_blocks;
		const SmallFwdLoad<ST> load{p.samples, lut, static_cast<uint64_t>(blk) * F::N, p.adders[p.d_base + d], p.fe_adder,
			p.phase0, p.fe_on};
		const SmallFwdEmit emit{p.spectra + (static_cast<size_t>(d) * p.k_blocks + blk) * F::N, p.one_sided ? F::N / 2 + 1 : F::N};
		F::template run_hooked<false, true>(a, b, plan, 1, F::N, load, emit);
	}

	struct SmallInvLoad {
		const float2* x;
		const float2* code;
		int half, one_sided;
		__device__ __forceinline__ float2 operator()(int, int i) const {
			return (one_sided && i > half) ? c2(0.f, 0.f) : cmul(__ldg(x + i), __ldg(code + i));
		}
	};
	struct SmallInvEmit {
		float* acc;
		float inv_n, post;
		int stat;
		template <int R, int NS>
		__device__ __forceinline__ void put(int, int base, const float2 (&v)[R]) const {
#pragma unroll
			for (int r = 0; r < R; ++r)
				acc[base + r * NS] += stat_of(cscale(cscale(v[r], inv_n), post), stat);
		}
	};
	// one-sided: Z is zero above N/2, so pass 0 reads only its live inputs
	template <int ZF>
	struct SmallInvLoadZ : SmallInvLoad {
		static constexpr int kZeroFrom = ZF;
	};
	// grid: codes x Doppler bins; unfolded rows (m == N) only.  Each thread
	// owns the same last-pass outputs in every block, so its accumulator
	// entries need no barrier between blocks.  HALF: one-sided spectra (the
	// pruned pass 0 of SmallInvLoadZ)
	template <class F, bool HALF = false>
	__global__ void __launch_bounds__(256) acq_inverse_static_kernel(AcqParams p) {
		extern __shared__ float2 smem[];
		float2* a = smem;
		float2* b = smem + F::N;
		float* acc = reinterpret_cast<float*>(smem + 2 * F::N);
		const FftPlanDev plan = F::prepare(p.plan, acc + F::N);
		const int row = blockIdx.x;
		const int c = row % p.n_codes;
		const int d = row / p.n_codes;
		for (int i = threadIdx.x; i < F::N; i += blockDim.x)
			acc[i] = 0.f;
		__syncthreads();
		const SmallInvEmit emit{acc, 1.0f / static_cast<float>(F::N), p.one_sided ? 2.0f : 1.0f, p.stat};
		for (int blk = 0; blk < p.k_blocks; ++blk) {
			const SmallInvLoadZ<HALF ? F::N / 2 + 1 : F::N> load{SmallInvLoad{p.spectra + (static_cast<size_t>(d) * p.k_blocks + blk) * F::N,
				p.codes[c], F::N / 2, p.one_sided}};
			F::template run_hooked<true, true>(a, b, plan, 1, F::N, load, emit);
			__syncthreads();  // pass 0 of the next block rewrites the tiles
		}
		reduce_cell(acc, F::N, p.cells + static_cast<size_t>(c) * p.n_doppler + p.d_base + d);
	}

	// ------------------------------------------------------------- forward
	template <int ST>
	__device__ __forceinline__ float2 fwd_load(const BatchedParams& p, int item, int64_t i, const float* lut) {
		if (p.code_mode) {
			const float* chips = p.chips + static_cast<size_t>(item) * p.chip_stride;
			const uint32_t mask = p.sign_masks ? p.sign_masks[item] : 0u;
			return c2(code_sample(chips, p.n_chips, p.repeats, p.base.n, static_cast<int>(i), mask, p.sign_segment), 0.f);
		}
		const int d = item / p.base.k_blocks;
		const int blk = item - d * p.base.k_blocks;
		const uint64_t g = static_cast<uint64_t>(blk) * p.base.n + static_cast<uint64_t>(i);
		float2 v = load_sample<ST>(p.base.samples, g);
		if (p.base.fe_on)
			v = table_mix(v, g, p.base.fe_adder, 0u, lut);
		return table_mix(v, g, p.base.adders[p.base.d_base + d], p.base.phase0, lut);
	}

	// grid: items * ceil(N2 / cw)
	template <int ST, class F1>
	__global__ void __launch_bounds__(F1::kColsMaxThreads, F1::kFwdColsMinBlocks) fwd_cols_kernel(BatchedParams p) {
		extern __shared__ float2 smem[];
		__shared__ float lut[80];
		// the 80-entry table whatever the block size (64-thread CTAs for 2-column tiles)
		for (int i = threadIdx.x; i < 80 && p.base.lut; i += blockDim.x)
			lut[i] = p.base.lut[i];
		__syncthreads();
		const int n1 = fft_n<F1>(p.n1), n2 = p.n2;
		const int chunks = (n2 + p.cw - 1) >> p.cw_shift;
		const int item = blockIdx.x / chunks;
		const int c0 = (blockIdx.x - item * chunks) << p.cw_shift;
		const int cw = min(p.cw, n2 - c0);
		const int ld = p.ld1;
		const int mask = p.cw - 1;
		float2* a = smem;
		float2* b = smem + p.cw * ld;
		const FftPlanDev p1 = F1::prepare(p.p1, smem + 2 * p.cw * ld);
		// consecutive threads take consecutive columns of one n1 row: coalesced reads
		if (p.code_mode) {
			for (int e = threadIdx.x; e < p.cw * n1; e += blockDim.x) {
				const int f = e & mask, i1 = e >> p.cw_shift;
				if (f < cw)
					a[f * ld + i1] = fwd_load<ST>(p, item, static_cast<int64_t>(n2) * i1 + c0 + f, lut);
			}
		}
		else {
			// signal items: (Doppler, block) and the NCO adders once per CTA
			const int d = item / p.base.k_blocks;
			const int blk = item - d * p.base.k_blocks;
			const uint32_t adder = p.base.adders[p.base.d_base + d];
			const int fe_on = p.base.fe_on;
			const uint32_t fe_adder = p.base.fe_adder, phase0 = p.base.phase0;
			// a thread keeps its column f (the block is a multiple of cw) and
			// steps its row by di: the sample index and both NCO holders
			// advance by constants
			const int f = threadIdx.x & mask, di = blockDim.x >> p.cw_shift;
			if (f < cw) {
				const int i10 = threadIdx.x >> p.cw_shift;
				uint64_t g = static_cast<uint64_t>(blk) * p.base.n + c0 + f + static_cast<uint64_t>(n2) * i10;
				const uint64_t dg = static_cast<uint64_t>(n2) * di;
				uint32_t hf = static_cast<uint32_t>(g) * fe_adder, hd = phase0 + static_cast<uint32_t>(g) * adder;
				const uint32_t dhf = static_cast<uint32_t>(dg) * fe_adder, dhd = static_cast<uint32_t>(dg) * adder;
				float2* col = a + f * ld;
				// eight rows' samples in flight per thread, then their mixes
				constexpr int U = 8;
				for (int i1 = i10; i1 < n1; i1 += U * di) {
					float2 v[U];
#pragma unroll
					for (int u = 0; u < U; ++u)
						if (i1 + u * di < n1)
							v[u] = load_sample<ST>(p.base.samples, g + static_cast<uint64_t>(u) * dg);
#pragma unroll
					for (int u = 0; u < U; ++u) {
						if (i1 + u * di < n1) {
							float2 w = v[u];
							if (fe_on)
								w = table_mix_holder(w, hf, lut);
							col[i1 + u * di] = table_mix_holder(w, hd, lut);
							hf += dhf;
							hd += dhd;
						}
					}
					g += U * dg;
				}
			}
		}
		__syncthreads();
		const float2* y = F1::template run<false>(a, b, p1, cw, ld);
		float2* out = p.out + static_cast<size_t>(item) * p.base.n;
		const float inv_n2 = 2.0f / static_cast<float>(p.base.n);
		// inter-step twiddle W_N^{(c0 + f) k1}: a thread keeps its column f
		// (the block is a multiple of cw) and steps k1 by blockDim / cw, so its
		// twiddle advances by a fixed W_N^{(c0 + f) blockDim / cw} (two
		// sincospif per thread, at most N1 cw / blockDim products in the chain)
		const uint32_t nn = static_cast<uint32_t>(p.base.n);
		const int e0 = threadIdx.x, f0 = e0 & mask;
		const uint32_t col = static_cast<uint32_t>(c0 + f0);
		float2 w = tw_n((col * static_cast<uint32_t>(e0 >> p.cw_shift)) % nn, p.base.n, inv_n2, false);
		const float2 step = tw_n((col * static_cast<uint32_t>(blockDim.x >> p.cw_shift)) % nn, p.base.n, inv_n2, false);
		for (int e = e0; e < p.cw * n1; e += blockDim.x) {
			const int k1 = e >> p.cw_shift;
			if (f0 < cw)
				out[static_cast<size_t>(k1) * n2 + c0 + f0] = cmul(y[f0 * ld + k1], w);
			w = cmul(w, step);
		}
	}

	// Row stage of the forward transform, hooked plans: pass 0 reads the
	// CTA's staged rows, the last pass stores the spectrum (one-sided: bins
	// above N/2 are never read, so they are not written; code mode conjugates
	// and zeroes them: conj(FFT(code)))
	struct FwdRowsLoad {
		const float2* xs;
		int n2;
		__device__ __forceinline__ float2 operator()(int f, int k2) const { return xs[f * n2 + k2]; }
	};
	struct FwdRowsEmit {
		float2* out;
		int n1, n2, r0, half, one_sided, code_mode, keep;
		template <int R, int NS>
		__device__ __forceinline__ void put(int f, int base, const float2 (&v)[R]) const {
			float2* o = out + static_cast<size_t>(f) * n2 + base;
#pragma unroll
			for (int r = 0; r < R; ++r) {
				const int k2 = base + r * NS;
				const bool zero = one_sided && (r0 + f) + static_cast<int64_t>(n1) * k2 > half;
				// signal spectra: the elements the inverse gather reads, k2 < keep
				// (the whole row, or the lower part the pruned gather reads); it
				// multiplies by the one-sided code spectrum, zero above N/2, with
				// no test
				if (code_mode)
					o[r * NS] = zero ? c2(0.f, 0.f) : c2(v[r].x, -v[r].y);
				else if (k2 < keep)
					o[r * NS] = v[r];
			}
		}
	};
	// items per CTA of the hooked forward rows
	constexpr int kFwdRowItems = 4;

	// grid: items * ceil(N1 / rw), or for compact plans ceil(items / 4) *
	// ceil(N1 / rw) with each CTA over up to four items (the next item's rows
	// copied in while the current item's last pass runs); code mode also
	// conjugates and masks (conj(FFT(code)))
	template <class F2>
	__global__ void __launch_bounds__(256, 3) fwd_rows_kernel(BatchedParams p, int items) {
		extern __shared__ float2 smem[];
		const int n1 = p.n1, n2 = fft_n<F2>(p.n2);
		const int chunks = (n1 + p.rw - 1) / p.rw;
		if constexpr (F2::kRowsCompact) {  // hooked, two passes: one work tile (pass 1 emits)
			const int group = blockIdx.x / chunks;
			const int r0 = (blockIdx.x - group * chunks) * p.rw;
			const int rw = min(p.rw, n1 - r0);
			const int tile = p.rw * n2;
			float2* b = smem;
			float2* xs = smem + tile;
			const FftPlanDev p2 = F2::prepare(p.p2, smem + 2 * tile);
			const int it0 = group * kFwdRowItems;
			const int it1 = min(items, it0 + kFwdRowItems);
			const int elems = rw * n2;
			const bool wide = (n2 % 2 == 0) && (p.base.n % 2 == 0);
			auto copy_rows = [&](int item) {
				const float2* src = p.out + static_cast<size_t>(item) * p.base.n + static_cast<size_t>(r0) * n2;
				if (wide) {
					for (int e = 2 * threadIdx.x; e < elems; e += 2 * blockDim.x)
						cp_async16(xs + e, src + e);
				}
				else {
					for (int e = threadIdx.x; e < elems; e += blockDim.x)
						cp_async8(xs + e, src + e);
				}
				cp_async_commit();
			};
			copy_rows(it0);
			const FwdRowsLoad load{xs, n2};
			for (int item = it0; item < it1; ++item) {
				cp_async_wait_all();
				__syncthreads();
				const FwdRowsEmit emit{p.out + static_cast<size_t>(item) * p.base.n + static_cast<size_t>(r0) * n2, n1, n2, r0,
					p.base.n / 2, p.base.one_sided, p.code_mode, p.row_keep > 0 ? p.row_keep : n2};
				auto next = [&] {
					if (item + 1 < it1)
						copy_rows(item + 1);
				};
				F2::template run_hooked<false, true>(b, b, p2, rw, n2, load, emit, next);
			}
			return;
		}
		const int item = blockIdx.x / chunks;
		const int r0 = (blockIdx.x - item * chunks) * p.rw;
		const int rw = min(p.rw, n1 - r0);
		float2* a = smem;
		float2* b = smem + p.rw * n2;
		const FftPlanDev p2 = F2::prepare(p.p2, smem + 2 * p.rw * n2);
		float2* out = p.out + static_cast<size_t>(item) * p.base.n + static_cast<size_t>(r0) * n2;
		for (int e = threadIdx.x; e < rw * n2; e += blockDim.x)
			a[e] = out[e];
		__syncthreads();
		const float2* y = F2::template run<false>(a, b, p2, rw, n2);
		const int half = p.base.n / 2;
		const float inv_n2f = 1.0f / static_cast<float>(n2);
		for (int e = threadIdx.x; e < rw * n2; e += blockDim.x) {
			const int ri = div_fft_n<F2>(e, inv_n2f), k2 = e - ri * n2;
			const int64_t k = (r0 + ri) + static_cast<int64_t>(n1) * k2;
			const bool zero = p.base.one_sided && k > half;
			if (p.code_mode) {
				const float2 v = y[e];
				out[e] = zero ? c2(0.f, 0.f) : c2(v.x, -v.y);
			}
			else {
				out[e] = y[e];  // whole spectrum (see FwdRowsEmit)
			}
		}
	}

	// Warp-owned forward rows (signal items of the two-pass row plans): each
	// warp of the CTA takes RPW of its RPW x WARPS rows through both passes
	// for up to kFwdRowItems items, the next item's rows copied into its
	// private tile by cp.async once pass 0 has read the current ones, with
	// only __syncwarp between its passes; the pass tables are built once per
	// CTA, its only barrier.  grid: ceil(items / kFwdRowItems) x
	// ceil(N1 / (RPW WARPS)).
	template <class F2, int RPW, int WARPS>
	constexpr size_t fwd_rows_warp_smem() {
		return sizeof(float2) * (static_cast<size_t>(WARPS) * RPW * 2 * F2::N + F2::N) + 16;
	}
	template <class F2, int RPW, int WARPS>
	__global__ void __launch_bounds__(32 * WARPS) fwd_rows_warp_kernel(BatchedParams p, int items) {
		static_assert(F2::kHooked && F2::kPasses == 2, "warp-owned rows run two-pass hooked plans (one work tile)");
		static_assert((F2::N * sizeof(float2)) % 16 == 0, "16-byte aligned rows");
		extern __shared__ float2 smem[];
		constexpr int N2 = F2::N, RW = RPW * WARPS, WT = RPW * N2;
		const int n1 = p.n1, n = p.base.n;
		const int chunks = (n1 + RW - 1) / RW;
		const int group = blockIdx.x / chunks;
		const int rc = (blockIdx.x - group * chunks) * RW;  // the CTA's first row
		const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
		const int r0 = rc + warp * RPW;                   // the warp's first row
		const int rw = max(0, min(RPW, n1 - r0));         // its rows (0: idle)
		float2* b = smem + warp * 2 * WT;
		float2* xs = b + WT;
		const FftPlanDev p2 = F2::prepare(p.p2, smem + WARPS * 2 * WT);
		__syncthreads();  // pass tables: the CTA's only barrier
		if (rw == 0)
			return;
		const int it0 = group * kFwdRowItems;
		const int it1 = min(items, it0 + kFwdRowItems);
		const int elems = rw * N2;
		const bool wide = (n % 2 == 0);  // every row start 16-byte aligned
		auto copy_rows = [&](int item) {
			const float2* src = p.out + static_cast<size_t>(item) * n + static_cast<size_t>(r0) * N2;
			if (wide) {
				for (int e = 2 * lane; e < elems; e += 64)
					cp_async16(xs + e, src + e);
			}
			else {
				for (int e = lane; e < elems; e += 32)
					cp_async8(xs + e, src + e);
			}
			cp_async_commit();
		};
		copy_rows(it0);
		const FwdRowsLoad load{xs, N2};
		const int keep = p.row_keep > 0 ? p.row_keep : N2;
		for (int item = it0; item < it1; ++item) {
			cp_async_wait_all();
			__syncwarp();  // this item's rows; the previous item's last pass is done with `b`
			const FwdRowsEmit emit{p.out + static_cast<size_t>(item) * n + static_cast<size_t>(r0) * N2, n1, N2, r0, n / 2,
				p.base.one_sided, 0, keep};
			auto next = [&] {  // pass 0 has read xs: the next item's rows go there
				if (item + 1 < it1)
					copy_rows(item + 1);
			};
			F2::template run_hooked_warp<false, true>(b, b, p2, rw, N2, load, emit, next);
		}
	}

	// ------------------------------------------------------------- inverse
	// Hooks of the static inverse plans.  Row stage: pass 0 gathers Z = X * C
	// straight from the spectra (bins above N/2 are zero one-sided), the last
	// pass applies W_N^{-i2 k1} (per-butterfly recurrence over its outputs,
	// i2 = base + r NS) and stores B.
	struct InvRowsLoad {
		const float2* x;
		const float2* code;
		int n1, n2, r0, half, one_sided;
		__device__ __forceinline__ float2 operator()(int f, int k2) const {
			if (one_sided && (r0 + f) + n1 * k2 > half)
				return c2(0.f, 0.f);
			const size_t off = static_cast<size_t>(f) * n2 + k2;
			return cmul(__ldg(x + off), __ldg(code + off));
		}
	};
	// the same gather from shared-memory copies of the CTA's rows: X of the
	// current block, and the code rows (or, when those are not staged, the
	// code rows straight from global memory)
	struct InvRowsLoadStaged {
		const float2* xs;
		const float2* cs;
		const float2* code_g;
		// one-sided: Z = 0 above N/2 because the code spectrum is zero there and
		// the forward kernels write the whole signal spectrum (finite values)
		__device__ __forceinline__ float2 operator()(int f, int k2, int n2) const {
			const int off = f * n2 + k2;
			return cmul(xs[off], cs ? cs[off] : __ldg(code_g + off));
		}
	};
	struct InvRowsLoadStagedN {
		InvRowsLoadStaged g;
		int n2;
		__device__ __forceinline__ float2 operator()(int f, int k2) const { return g(f, k2, n2); }
	};
	// the same gather with Z known to be zero at k2 >= ZF in every row
	template <int ZF>
	struct InvRowsLoadStagedZ : InvRowsLoadStagedN {
		static constexpr int kZeroFrom = ZF;
	};
	// One-sided code spectra are zero above N/2, so Z = X C is zero at
	// k = k1 + N1 k2 > N/2, which holds in every row for k2 >= ZF =
	// floor(N/2 / N1) + 1.  The pruned row gather reads the elements k2 < ZF
	// rounded up to its pass-0 stride: the row elements the forward stage
	// must store for it.
	template <class F2>
	constexpr int half_zero_from(int n1) {
		return (n1 * F2::N / 2) / n1 + 1;
	}
	template <class F2>
	constexpr int half_row_elems(int n1) {
		const int zf = half_zero_from<F2>(n1), nb = F2::kFirstNB;
		const int zl = (zf + nb - 1) / nb * nb;
		return zl < F2::N ? zl : F2::N;
	}
	// Inter-step twiddle seeds of the row stage, per CTA: for each of its rows
	// k1 = r0 + f, W_N^{-j k1} for j < NS and W_N^{-NS k1} at j = NS, where NS
	// is the stride of the plan's last pass (whose butterflies start at base
	// = j < NS); built once per CTA and reused over the K blocks.
	__device__ __forceinline__ void build_row_seeds(float2* seeds, int rows, int ns, int r0, uint32_t n) {
		const float inv_n2 = 2.0f / static_cast<float>(n);
		for (int e = threadIdx.x; e < rows * (ns + 1); e += blockDim.x) {
			const int f = e / (ns + 1), j = e - f * (ns + 1);
			seeds[e] = tw_n((static_cast<uint32_t>(j) * static_cast<uint32_t>(r0 + f)) % n, n, inv_n2, true);
		}
	}

	struct InvRowsEmit {
		float2* out;
		int n2, r0;
		const float2* seeds;  // build_row_seeds
		template <int R, int NS>
		__device__ __forceinline__ void put(int f, int base, const float2 (&v)[R]) const {
			float2 w = seeds[f * (NS + 1) + base];
			const float2 step = seeds[f * (NS + 1) + NS];
			float2* o = out + static_cast<size_t>(f) * n2 + base;
#pragma unroll
			for (int r = 0; r < R; ++r) {
				o[r * NS] = cmul(v[r], w);
				w = cmul(w, step);
			}
		}
	};
	// The same store into the blocked layout B[n2 / CW][k1][n2 % CW] of the
	// warp-owned column kernel (out: the (row, block) base, N1 x n2p entries).
	template <int CW, int N1>
	struct InvRowsEmitBlocked {
		float2* out;
		int r0;
		const float2* seeds;  // build_row_seeds
		// In the last pass base < NS (NB = NS), so when CW divides NS every
		// output of the butterfly sits a compile-time distance from the first:
		// n2 = base + r NS lies in chunk base / CW + r NS / CW at column base % CW.
		template <int R, int NS>
		__device__ __forceinline__ void put(int f, int base, const float2 (&v)[R]) const {
			const int k1 = r0 + f;
			float2 w = seeds[f * (NS + 1) + base];
			const float2 step = seeds[f * (NS + 1) + NS];
			constexpr int S = N1 * CW;  // one chunk of the blocked layout
			if constexpr (NS % CW == 0) {
				float2* o = out + (k1 * CW + (base / CW) * S + base % CW);
#pragma unroll
				for (int r = 0; r < R; ++r) {
					o[r * (NS / CW) * S] = cmul(v[r], w);
					w = cmul(w, step);
				}
			}
			else {
				float2* o = out + k1 * CW;
#pragma unroll
				for (int r = 0; r < R; ++r) {
					const int n2 = base + r * NS;
					o[(n2 / CW) * S + (n2 % CW)] = cmul(v[r], w);
					w = cmul(w, step);
				}
			}
		}
	};

	// Column stage: the last pass scales each output (1/N, x2 one-sided),
	// takes |.| or |.|^2 and accumulates it (or, folded, adds it to the row's
	// fold buffer) instead of storing the transform.
	struct InvColsEmit {
		float* acc;
		int ld, stat, fold_mode, n2, c0, m;
		float scale;
		float* ag;
		float2* zg;
		template <int R, int NS>
		__device__ __forceinline__ void put(int f, int base, const float2 (&v)[R]) const {
			if (fold_mode == 0) {
				float* a = acc + f * ld + base;
#pragma unroll
				for (int r = 0; r < R; ++r)
					a[r * NS] += stat_of(cscale(v[r], scale), stat);
				return;
			}
#pragma unroll
			for (int r = 0; r < R; ++r) {
				const uint32_t tau = static_cast<uint32_t>(n2) * static_cast<uint32_t>(base + r * NS) + c0 + f;
				const float2 y = cscale(v[r], scale);
				if (fold_mode == 1) {
					atomicAdd(ag + tau % static_cast<uint32_t>(m), stat_of(y, stat));
				}
				else {
					float2* z = zg + tau % static_cast<uint32_t>(m);
					atomicAdd(&z->x, y.x);
					atomicAdd(&z->y, y.y);
				}
			}
		}
	};

	// a compact plan (hooked, two passes) gathers pass 0 from its staged
	// rows: one work tile
	template <class F>
	constexpr bool rows_one_tile() { return F::kRowsCompact; }
	// hooked plans run one CTA per (row, chunk of rw sub-rows) over all K
	// blocks: X of block k + 1 is copied in while block k's last pass runs,
	// and the code rows (the same for every block) are staged once (N2 <= 512:
	// for 500-point rows three 32 KB tiles leave two CTAs per SM, still
	// faster than re-reading the code rows from L2 for every block)
	template <class F>
	constexpr bool rows_stage_code() { return F::kHooked && F::N <= 512; }
	template <class F>
	constexpr int rows_tiles() {
		return (rows_one_tile<F>() ? 1 : 2) + (F::kHooked ? 1 : 0) + (rows_stage_code<F>() ? 1 : 0);
	}

	// hooked plans: grid rows * ceil(N1 / rw), each CTA over the K blocks;
	// others: grid rows * K * ceil(N1 / rw)
	// BCW > 0: B goes out in the blocked layout of inv_cols_warp_kernel with
	// CW = BCW (hooked plans only)
	template <class F2, int BCW = 0, int BN1 = 0>
	__global__ void __launch_bounds__(F2::kRowsMaxThreads, F2::kRowsMinBlocks) inv_rows_kernel(BatchedParams p) {
		extern __shared__ float2 smem[];
		const AcqParams& q = p.base;
		const int n1 = p.n1, n2 = fft_n<F2>(p.n2), n = q.n;
		const int chunks = (n1 + p.rw - 1) / p.rw;
		const int half = n / 2;
		const int tile = p.rw * n2;
		float2* a = smem;
		float2* b = rows_one_tile<F2>() ? smem : smem + tile;
		if constexpr (F2::kHooked) {
			const int lrow = blockIdx.x / chunks;
			const int r0 = (blockIdx.x - lrow * chunks) * p.rw;
			const int rw = min(p.rw, n1 - r0);
			const int row = p.row0 + lrow;
			const int c = row % q.n_codes;
			const int d = row / q.n_codes;
			float2* xs = b + tile;
			float2* cs = rows_stage_code<F2>() ? xs + tile : nullptr;
			const FftPlanDev p2 = F2::prepare(p.p2, smem + rows_tiles<F2>() * tile);
			const float2* code = q.codes[c] + static_cast<size_t>(r0) * n2;
			const float2* xg = q.spectra + static_cast<size_t>(d) * q.k_blocks * n + static_cast<size_t>(r0) * n2;
			const int elems = rw * n2;
			// 16-byte copies when every row start is 16-byte aligned
			const bool wide = (n2 % 2 == 0) && (n % 2 == 0);
			auto copy_rows = [&](float2* dst, const float2* src) {
				if (wide) {
					for (int e = 2 * threadIdx.x; e < elems; e += 2 * blockDim.x)
						cp_async16(dst + e, src + e);
				}
				else {
					for (int e = threadIdx.x; e < elems; e += blockDim.x)
						cp_async8(dst + e, src + e);
				}
			};
			if (cs)
				copy_rows(cs, code);
			copy_rows(xs, xg);
			cp_async_commit();
			const InvRowsLoadStagedN load{InvRowsLoadStaged{xs, cs, code}, n2};
			// twiddle seeds after the pass tables (N2 entries)
			float2* seeds = const_cast<float2*>(p2.tw) + F2::N;
			build_row_seeds(seeds, rw, F2::kLastNS, r0, static_cast<uint32_t>(n));
			for (int blk = 0; blk < q.k_blocks; ++blk) {
				cp_async_wait_all();
				__syncthreads();  // this block's X (and the twiddle table) in shared memory
				const size_t item = static_cast<size_t>(lrow) * q.k_blocks + blk;
				auto next = [&] {  // pass 0 has read xs: the next block's X goes there
					if (blk + 1 < q.k_blocks) {
						copy_rows(xs, xg + static_cast<size_t>(blk + 1) * n);
						cp_async_commit();
					}
				};
				if constexpr (BCW > 0) {
					const InvRowsEmitBlocked<BCW, BN1> emit{p.bbuf + item * (static_cast<size_t>(n1) * p.n2p), r0, seeds};
					F2::template run_hooked<true, true>(a, b, p2, rw, n2, load, emit, next);
				}
				else {
					const InvRowsEmit emit{p.bbuf + item * n + static_cast<size_t>(r0) * n2, n2, r0, seeds};
					F2::template run_hooked<true, true>(a, b, p2, rw, n2, load, emit, next);
				}
				// the next iteration's first barrier orders this block's last-pass
				// reads of `b` before its first pass writes it again
			}
			return;
		}
		static_assert(BCW == 0 || F2::kHooked, "the blocked B layout needs a hooked row plan");
		const int item = blockIdx.x / chunks;       // (local row, block)
		const int r0 = (blockIdx.x - item * chunks) * p.rw;
		const int rw = min(p.rw, n1 - r0);
		const int lrow = item / q.k_blocks;
		const int blk = item - lrow * q.k_blocks;
		const int row = p.row0 + lrow;
		const int c = row % q.n_codes;
		const int d = row / q.n_codes;
		const float2* x = q.spectra + (static_cast<size_t>(d) * q.k_blocks + blk) * n + static_cast<size_t>(r0) * n2;
		const float2* code = q.codes[c] + static_cast<size_t>(r0) * n2;
		const FftPlanDev p2 = F2::prepare(p.p2, smem + (rows_one_tile<F2>() ? 1 : 2) * tile);
		const float inv_n2f = 1.0f / static_cast<float>(n2);
		// Z = X * C, four element pairs in flight per thread
		const int total = rw * n2;
		for (int e0 = threadIdx.x; e0 < total; e0 += 4 * blockDim.x) {
			float2 xv[4], cv[4];
#pragma unroll
			for (int u = 0; u < 4; ++u) {
				const int e = e0 + u * blockDim.x;
				if (e < total) {
					xv[u] = __ldg(x + e);
					cv[u] = __ldg(code + e);
				}
			}
#pragma unroll
			for (int u = 0; u < 4; ++u) {
				const int e = e0 + u * blockDim.x;
				if (e < total) {
					const int ri = div_fft_n<F2>(e, inv_n2f), k2 = e - ri * n2;
					const int64_t k = (r0 + ri) + static_cast<int64_t>(n1) * k2;
					a[e] = (q.one_sided && k > half) ? c2(0.f, 0.f) : cmul(xv[u], cv[u]);
				}
			}
		}
		__syncthreads();
		const float2* y = F2::template run<true>(a, b, p2, rw, n2);
		float2* out = p.bbuf + static_cast<size_t>(item) * n + static_cast<size_t>(r0) * n2;
		const float inv_n2 = 2.0f / static_cast<float>(n);
		// inter-step twiddle W_N^{-i2 k1}: one warp per row k1, lane l takes
		// i2 = l, l + 32, ... and advances its twiddle by W_N^{-32 k1} (two
		// sincospif per lane and row, at most n2 / 32 products in the chain)
		const int lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
		for (int ri = threadIdx.x >> 5; ri < rw; ri += nwarps) {
			const uint32_t k1 = static_cast<uint32_t>(r0 + ri);
			float2 w = tw_n((static_cast<uint32_t>(lane) * k1) % static_cast<uint32_t>(n), n, inv_n2, true);
			const float2 step = tw_n((32u * k1) % static_cast<uint32_t>(n), n, inv_n2, true);
			const float2* yr = y + ri * n2;
			float2* orow = out + ri * n2;
			for (int i2 = lane; i2 < n2; i2 += 32) {
				orow[i2] = cmul(yr[i2], w);
				w = cmul(w, step);
			}
		}
	}

	// Warp-owned row stage (two-pass hooked row plans): each warp of the CTA
	// takes RPW of the CTA's RPW x WARPS rows through both passes for all K
	// blocks with only __syncwarp between its passes — its X rows (the next
	// block's copied in once pass 0 has read the current one), its code rows
	// (staged once) and its work tile are private to it; the pass tables and
	// the twiddle seeds are built once per CTA.  B goes out in the blocked
	// layout of inv_cols_warp_kernel.  grid: rows * ceil(N1 / (RPW WARPS)).
	// CODE: the code rows staged in shared memory (else read through L1 / L2,
	// which leaves room for more rows per warp).
	// HALF (one-sided code spectra): the code spectrum is zero above N/2, so
	// Z = X C is zero at k = k1 + N1 k2 > N/2, which holds in every row for
	// k2 >= ZF = floor(N/2 / N1) + 1; pass 0 reads only the elements k2 < ZL
	// (its live inputs: ZF rounded up to its butterfly stride), and only
	// those of the X and code rows are staged.
	// staged elements per row: the pruned gather's part, or the whole row
	template <class F2, int BN1, bool HALF>
	constexpr int rows_warp_staged() {
		return HALF ? half_row_elems<F2>(BN1) : F2::N;
	}
	// per warp: the work tile (RPW rows of N2), the staged X rows and (CODE)
	// code rows (RPW rows of SL each); per CTA: pass tables (N2) and seeds
	template <class F2, int BN1, int RPW, int WARPS, bool CODE, bool HALF>
	constexpr size_t rows_warp_smem() {
		constexpr size_t SL = rows_warp_staged<F2, BN1, HALF>();
		return sizeof(float2) * (static_cast<size_t>(WARPS) * RPW * (F2::N + (CODE ? 2 : 1) * SL) + F2::N +
			static_cast<size_t>(WARPS) * RPW * (F2::kLastNS + 1)) + 16;
	}
	// the gather of the warp kernel: staged X (and code) rows at stride SL,
	// or code rows from global memory at stride N2; Z zero at k2 >= ZF
	template <int ZF, int SL, int N2, bool CODE>
	struct InvRowsLoadWarp {
		const float2* xs;
		const float2* cs;
		const float2* code_g;
		static constexpr int kZeroFrom = ZF;
		__device__ __forceinline__ float2 operator()(int f, int k2) const {
			const int off = f * SL + k2;
			if constexpr (CODE)
				return cmul(xs[off], cs[off]);
			else
				return cmul(xs[off], __ldg(code_g + f * N2 + k2));
		}
	};
	template <class F2, int BCW, int BN1, int RPW, int WARPS, bool CODE = true, bool HALF = false>
	__global__ void __launch_bounds__(32 * WARPS) inv_rows_warp_kernel(BatchedParams p) {
		static_assert(F2::kHooked && F2::kPasses == 2, "warp-owned rows run two-pass hooked plans (one work tile)");
		extern __shared__ float2 smem[];
		constexpr int N2 = F2::N, NS = F2::kLastNS, RW = RPW * WARPS;
		constexpr int ZF = HALF ? half_zero_from<F2>(BN1) : N2;
		constexpr int SL = rows_warp_staged<F2, BN1, HALF>();  // staged elements per row
		using Load = InvRowsLoadWarp<ZF, SL, N2, CODE>;
		static_assert(SL == live_inputs<Load, N2, N2 / F2::kFirstNB>() * F2::kFirstNB && SL >= ZF,
			"pass 0 reads the staged elements only");
		static_assert((N2 * sizeof(float2)) % 16 == 0 && (SL * sizeof(float2)) % 16 == 0, "16-byte aligned tiles");
		constexpr int WT = RPW * (N2 + (CODE ? 2 : 1) * SL);  // a warp's region
		const AcqParams& q = p.base;
		const int n1 = p.n1, n = q.n;
		const int chunks = (n1 + RW - 1) / RW;
		const int lrow = blockIdx.x / chunks;
		const int rc = (blockIdx.x - lrow * chunks) * RW;  // the CTA's first row
		const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
		const int r0 = rc + warp * RPW;                   // the warp's first row
		const int rw = max(0, min(RPW, n1 - r0));         // its rows (0: idle)
		const int row = p.row0 + lrow;
		const int c = row % q.n_codes;
		const int d = row / q.n_codes;
		float2* b = smem + warp * WT;
		float2* xs = b + RPW * N2;
		float2* cs = CODE ? xs + RPW * SL : nullptr;
		const FftPlanDev p2 = F2::prepare(p.p2, smem + WARPS * WT);
		float2* seeds = const_cast<float2*>(p2.tw) + N2;  // after the pass tables (N2 entries)
		build_row_seeds(seeds, min(RW, n1 - rc), NS, rc, static_cast<uint32_t>(n));
		__syncthreads();  // pass tables and seeds: the CTA's only barrier
		if (rw == 0)
			return;
		const float2* code = q.codes[c] + static_cast<size_t>(r0) * N2;
		const float2* xg = q.spectra + static_cast<size_t>(d) * q.k_blocks * n + static_cast<size_t>(r0) * N2;
		const bool wide = (n % 2 == 0);  // every row start 16-byte aligned (N2 even)
		// the first SL elements of each of the warp's rows: src stride N2, dst stride SL
		auto copy_rows = [&](float2* dst, const float2* src) {
			if (wide) {
				constexpr int HP = SL / 2;
				for (int e = lane; e < rw * HP; e += 32) {
					const int ri = e / HP, h = 2 * (e - ri * HP);
					cp_async16(dst + ri * SL + h, src + ri * N2 + h);
				}
			}
			else {
				for (int e = lane; e < rw * SL; e += 32) {
					const int ri = e / SL, h = e - ri * SL;
					cp_async8(dst + ri * SL + h, src + ri * N2 + h);
				}
			}
		};
		if constexpr (CODE)
			copy_rows(cs, code);
		copy_rows(xs, xg);
		cp_async_commit();
		const Load load{xs, cs, code};
		const float2* wseeds = seeds + warp * RPW * (NS + 1);
		for (int blk = 0; blk < q.k_blocks; ++blk) {
			cp_async_wait_all();
			__syncwarp();  // this block's X rows; the previous block's last pass is done with `b`
			const size_t item = static_cast<size_t>(lrow) * q.k_blocks + blk;
			auto next = [&] {  // pass 0 has read xs: the next block's X goes there
				if (blk + 1 < q.k_blocks) {
					copy_rows(xs, xg + static_cast<size_t>(blk + 1) * n);
					cp_async_commit();
				}
			};
			const InvRowsEmitBlocked<BCW, BN1> emit{p.bbuf + item * (static_cast<size_t>(n1) * p.n2p), r0, wseeds};
			F2::template run_hooked_warp<true, true>(b, b, p2, rw, N2, load, emit, next);
		}
	}

	// grid: rows * ceil(N2 / cw); shared: 3 * cw * ld1 float2 (input, work, prefetch) + cw * ld1 float
	template <class F1>
	__global__ void __launch_bounds__(F1::kColsMaxThreads, F1::kColsMinBlocks) inv_cols_kernel(BatchedParams p) {
		extern __shared__ float2 smem[];
		__shared__ MaxIdx s_max[8];
		__shared__ double s_sum[8], s_sq[8];
		__shared__ bool s_last;
		const AcqParams& q = p.base;
		const int n1 = fft_n<F1>(p.n1), n2 = p.n2, n = q.n, m = q.m;
		const int chunks = (n2 + p.cw - 1) >> p.cw_shift;
		const int lrow = blockIdx.x / chunks;
		const int chunk = blockIdx.x - lrow * chunks;
		const int c0 = chunk << p.cw_shift;
		const int cw = min(p.cw, n2 - c0);
		const int ld = p.ld1;
		const int mask = p.cw - 1;
		const int tile = p.cw * ld;
		constexpr bool kCompact = F1::kColsCompact;  // no prefetch tile: the next block lands in `in` after pass 0
		float2* in = smem;
		float2* work = smem + tile;
		float2* pre = smem + 2 * tile;
		float* acc = reinterpret_cast<float*>(smem + (kCompact ? 2 : 3) * tile);
		const FftPlanDev p1 = F1::prepare(p.p1, acc + tile);
		const float inv_n = 1.0f / static_cast<float>(n);
		const float post = q.one_sided ? 2.0f : 1.0f;
		const float inv_n1 = 1.0f / static_cast<float>(n1);
		for (int e = threadIdx.x; e < tile; e += blockDim.x)
			acc[e] = 0.f;
		auto prefetch = [&](float2* dst, int blk) {
			const float2* bsrc = p.bbuf + (static_cast<size_t>(lrow) * q.k_blocks + blk) * n + c0;
			for (int e = threadIdx.x; e < p.cw * n1; e += blockDim.x) {
				const int f = e & mask, k1 = e >> p.cw_shift;
				if (f < cw)
					cp_async8(dst + f * ld + k1, bsrc + static_cast<size_t>(k1) * n2 + f);
			}
			cp_async_commit();
		};
		prefetch(in, 0);
		for (int blk = 0; blk < q.k_blocks; ++blk) {
			cp_async_wait_all();
			__syncthreads();
			if (!kCompact && blk + 1 < q.k_blocks)
				prefetch(pre, blk + 1);
			if constexpr (F1::kHooked) {
				float2* zg = q.fold_mode == 2 ? p.zcg + (static_cast<size_t>(lrow) * q.k_blocks + blk) * m : nullptr;
				const InvColsEmit emit{acc, ld, q.stat, q.fold_mode, n2, c0, m, inv_n * post,
					q.fold_mode == 1 ? p.accg + static_cast<size_t>(lrow) * m : nullptr, zg};
				const NoLoad none{};
				if constexpr (kCompact) {
					// the next iteration's first barrier orders this block's last-pass
					// reads of `work` and writes of `acc` before they are reused
					auto mid = [&] {
						if (blk + 1 < q.k_blocks)
							prefetch(in, blk + 1);
					};
					F1::template run_hooked<true, false>(in, work, p1, cw, ld, none, emit, mid);
					continue;
				}
				F1::template run_hooked<true, false>(in, work, p1, cw, ld, none, emit);
				__syncthreads();
				float2* t = in;
				in = pre;
				pre = t;
				continue;
			}
			const float2* y = F1::template run<true>(in, work, p1, cw, ld);
			if (q.fold_mode == 0) {
				for (int e = threadIdx.x; e < cw * n1; e += blockDim.x) {
					const int f = div_fft_n<F1>(e, inv_n1), i1 = e - f * n1;
					acc[f * ld + i1] += stat_of(cscale(cscale(y[f * ld + i1], inv_n), post), q.stat);
				}
			}
			else if (q.fold_mode == 1) {
				float* ag = p.accg + static_cast<size_t>(lrow) * m;
				for (int e = threadIdx.x; e < cw * n1; e += blockDim.x) {
					const int f = div_fft_n<F1>(e, inv_n1), i1 = e - f * n1;
					const uint32_t tau = static_cast<uint32_t>(n2) * i1 + c0 + f;
					atomicAdd(ag + tau % static_cast<uint32_t>(m), stat_of(cscale(cscale(y[f * ld + i1], inv_n), post), q.stat));
				}
			}
			else {
				float2* zg = p.zcg + (static_cast<size_t>(lrow) * q.k_blocks + blk) * m;
				for (int e = threadIdx.x; e < cw * n1; e += blockDim.x) {
					const int f = div_fft_n<F1>(e, inv_n1), i1 = e - f * n1;
					const uint32_t tau = static_cast<uint32_t>(n2) * i1 + c0 + f;
					const float2 v = cscale(cscale(y[f * ld + i1], inv_n), post);
					float2* z = zg + tau % static_cast<uint32_t>(m);
					atomicAdd(&z->x, v.x);
					atomicAdd(&z->y, v.y);
				}
			}
			__syncthreads();
			float2* t = in;  // the consumed input buffer receives the block after next
			in = pre;
			pre = t;
		}
		if constexpr (kCompact)
			__syncthreads();  // the last block's accumulation is complete
		if (q.fold_mode != 0)
			return;
		// chunk partial: first max (lowest natural index on ties), sum, sum of squares
		MaxIdx best{-1.0f, 0xFFFFFFFFu};
		float sum = 0.f, sq = 0.f;
		for (int e = threadIdx.x; e < cw * n1; e += blockDim.x) {
			const int f = div_fft_n<F1>(e, inv_n1), i1 = e - f * n1;
			const float v = acc[f * ld + i1];
			const MaxIdx cand{v, static_cast<uint32_t>(n2) * i1 + c0 + f};
			best = better(best, cand);
			sum += v;
			sq += v * v;
		}
		double dsum = sum, dsq = sq;
		for (int o = 16; o > 0; o >>= 1) {
			const MaxIdx other{__shfl_down_sync(0xffffffffu, best.v, o), __shfl_down_sync(0xffffffffu, best.i, o)};
			best = better(best, other);
			dsum += __shfl_down_sync(0xffffffffu, dsum, o);
			dsq += __shfl_down_sync(0xffffffffu, dsq, o);
		}
		const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
		if (lane == 0) {
			s_max[warp] = best;
			s_sum[warp] = dsum;
			s_sq[warp] = dsq;
		}
		__syncthreads();
		if (threadIdx.x == 0) {
			for (int w = 1; w < (blockDim.x + 31) / 32; ++w) {
				s_max[0] = better(s_max[0], s_max[w]);
				s_sum[0] += s_sum[w];
				s_sq[0] += s_sq[w];
			}
			const size_t slot = static_cast<size_t>(lrow) * chunks + chunk;
			p.partials[slot] = make_float4(s_max[0].v, __uint_as_float(s_max[0].i), 0.f, 0.f);
			p.sums[slot] = make_double2(s_sum[0], s_sq[0]);
			__threadfence();
			s_last = atomicAdd(p.counters + lrow, 1u) == static_cast<unsigned>(chunks - 1);
		}
		__syncthreads();
		if (!s_last || threadIdx.x != 0)
			return;
		// last chunk of this row: combine every chunk's partial into the cell
		__threadfence();
		MaxIdx rb{-1.0f, 0xFFFFFFFFu};
		double ts = 0, tq = 0;
		for (int k = 0; k < chunks; ++k) {
			const size_t slot = static_cast<size_t>(lrow) * chunks + k;
			const float4 pt = __ldcg(p.partials + slot);
			const double2 sm = __ldcg(p.sums + slot);
			rb = better(rb, MaxIdx{pt.x, __float_as_uint(pt.y)});
			ts += sm.x;
			tq += sm.y;
		}
		const int row = p.row0 + lrow;
		const int c = row % q.n_codes;
		const int d = q.d_base + row / q.n_codes;  // rows are local to the Doppler chunk
		const double mean = ts / m;
		const double var = m > 1 ? (tq - ts * mean) / (m - 1) : 0.0;
		AcqCellDev cell;
		cell.level = rb.v;
		cell.index = rb.i;
		cell.mean = static_cast<float>(mean);
		cell.std = static_cast<float>(sqrt(var > 0 ? var : 0.0));
		q.cells[static_cast<size_t>(c) * q.n_doppler + d] = cell;
	}

	// folded rows: acc (fold 1) or |complex fold| summed over blocks (fold 2) -> cell; grid: rows
	static __global__ void __launch_bounds__(256) fold_finish_kernel(BatchedParams p) {
		const AcqParams& q = p.base;
		const int lrow = blockIdx.x;
		const int m = q.m;
		float* ag = p.accg + static_cast<size_t>(lrow) * m;
		if (q.fold_mode == 2) {
			const float2* zg = p.zcg + static_cast<size_t>(lrow) * q.k_blocks * m;
			for (int i = threadIdx.x; i < m; i += blockDim.x) {
				float s = 0.f;
				for (int blk = 0; blk < q.k_blocks; ++blk)
					s += stat_of(zg[static_cast<size_t>(blk) * m + i], q.stat);
				ag[i] = s;
			}
			__syncthreads();
		}
		const int row = p.row0 + lrow;
		const int c = row % q.n_codes;
		const int d = q.d_base + row / q.n_codes;
		reduce_cell(ag, m, q.cells + static_cast<size_t>(c) * q.n_doppler + d);
	}
}

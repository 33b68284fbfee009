// Column stage of the four-step inverse with warp-owned columns.
//
// The row stage (inv_rows_kernel) leaves B[k1][n2] = W_N^{-n2 k1} x
// IFFT_{N2}(Z_T[k1][.])[n2] for every (row, block); this stage takes, for
// each column n2, the N1-point IFFT over k1 and accumulates |y| (or |y|^2)
// of y[N2 n1 + n2] over the K blocks, then reduces the row to its cell
// (first maximum, mean, unbiased sigma: max_index.hpp:31-42,
// mean_stddev.hpp:29-42).
//
// Layout of B for this kernel ("blocked"): B[chunk][k1][c] with
// n2 = chunk * CW + c, N2 padded up to a multiple of CW (the padded columns
// are computed and ignored), so one CTA's columns of one block are a single
// contiguous N1 x CW region.
//
// Work split: the CTA has WARPS warps and every warp owns CPW adjacent
// columns for all K blocks, so the only synchronisation inside the block
// loop is __syncwarp.  N1 = R0 x R1 with R1 = 25 last: the last pass has
// N1 / R1 = R0 butterflies per column, CPW = 32 / R0 columns make it exactly
// one butterfly per lane, and each lane keeps the R1 outputs it produces
// (n1 = j + r R0, the same in every block) in registers as its accumulators.
// Pass 0 (radix R0, no twiddles) runs NB0 = R1 butterflies per column over
// the lanes.  Tiles are [k1][CPW] with one pad row every R0 rows: pass 0's
// stride-R0 stores and both passes' loads then fall in distinct banks.
#pragma once

#include "acq_batched.cuh"

namespace ugsdr_gpu {

	template <int N1_, int R0_, int R1_, int WARPS_, int MINB_>
	struct ColsWarpPlan {
		static constexpr int N1 = N1_, R0 = R0_, R1 = R1_, WARPS = WARPS_, MINB = MINB_;
		static constexpr int NB0 = N1 / R0;             // pass-0 butterflies per column
		static constexpr int CPW = 32 / R0;             // columns per warp (pass 1: one butterfly per lane)
		static constexpr int CW = CPW * WARPS;          // columns per CTA
		static constexpr int ROWS = N1 + N1 / R0;       // padded tile rows
		static constexpr int TILE = ROWS * CPW;         // float2 per warp tile
		static constexpr int TW = (R1 - 1) * R0;        // pass-1 twiddles
		static_assert(R0 * R1 == N1 && R0 * CPW == 32 && CPW % 2 == 0, "plan shape");
		static constexpr size_t smem_bytes() { return sizeof(float2) * (static_cast<size_t>(WARPS) * 2 * TILE + TW); }
		__device__ static __forceinline__ int prow(int k1) { return k1 + k1 / R0; }
	};

	// grid: rows x (N2 padded / CW); one CTA per (row, column chunk) over the K
	// blocks.  STAT: the job's statistic (UGSDR_STAT_ABS2 non-zero: |y|^2)
	template <class P, int STAT>
	__global__ void __launch_bounds__(32 * P::WARPS, P::MINB) inv_cols_warp_kernel(BatchedParams p) {
		extern __shared__ float2 smem[];
		__shared__ MaxIdx s_max[P::WARPS];
		__shared__ double s_sum[P::WARPS], s_sq[P::WARPS];
		__shared__ bool s_last;
		const AcqParams& q = p.base;
		const int n2 = p.n2;
		const int chunks = p.n2p / P::CW;
		const int lrow = blockIdx.x / chunks;
		const int chunk = blockIdx.x - lrow * chunks;
		const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
		float2* in = smem + warp * 2 * P::TILE;
		float2* work = in + P::TILE;
		float2* tw1 = smem + P::WARPS * 2 * P::TILE;
		// pass-1 twiddles W_N1^{r k} (exponent r k N1 / (R0 R1) = r k), laid
		// out [r - 1][k]: the lanes of a load differ in k only
		for (int e = threadIdx.x; e < P::TW; e += blockDim.x) {
			const int r = e / P::R0 + 1, k = e - (r - 1) * P::R0;
			tw1[e] = __ldg(p.p1.tw + r * k);
		}
		const size_t block_elems = static_cast<size_t>(P::N1) * p.n2p;
		const float2* bsrc = p.bbuf + static_cast<size_t>(lrow) * q.k_blocks * block_elems +
			static_cast<size_t>(chunk) * (P::N1 * P::CW) + warp * P::CPW;
		constexpr int H = P::CPW / 2;  // 16-byte pieces per k1 row of the warp's columns
		auto prefetch = [&](int blk) {
			const float2* src = bsrc + static_cast<size_t>(blk) * block_elems;
			for (int e = lane; e < P::N1 * H; e += 32) {
				const int k1 = e / H, h = e - k1 * H;
				cp_async16(in + P::prow(k1) * P::CPW + 2 * h, src + k1 * P::CW + 2 * h);
			}
			cp_async_commit();
		};
		prefetch(0);
		__syncthreads();  // twiddle table
		float acc[P::R1];
#pragma unroll
		for (int r = 0; r < P::R1; ++r)
			acc[r] = 0.f;
		const int j1 = lane / P::CPW, c1 = lane - j1 * P::CPW;  // pass-1 butterfly of this lane (k = j1)
		for (int blk = 0; blk < q.k_blocks; ++blk) {
			cp_async_wait_all();
			__syncwarp();  // the block's tile is in `in`; last block's pass-1 reads of `work` are done
			// pass 0: radix R0, v_r = in[j + r NB0], out[j R0 + r]
			for (int u = lane; u < P::NB0 * P::CPW; u += 32) {
				const int j = u / P::CPW, c = u - j * P::CPW;
				float2 v[P::R0];
#pragma unroll
				for (int r = 0; r < P::R0; ++r)
					v[r] = in[P::prow(j + r * P::NB0) * P::CPW + c];
				Dft<P::R0, true>::run(v);
				float2* o = work + (j * P::R0 + j) * P::CPW + c;  // prow(j R0 + r) = j R0 + r + j
#pragma unroll
				for (int r = 0; r < P::R0; ++r)
					o[r * P::CPW] = v[r];
			}
			__syncwarp();  // `work` complete, `in` consumed
			if (blk + 1 < q.k_blocks)
				prefetch(blk + 1);
			// pass 1: radix R1 with twiddles, v_r = work[j + r R0] W^{-r j}; outputs n1 = j + r R0
			{
				float2 v[P::R1];
#pragma unroll
				for (int r = 0; r < P::R1; ++r)
					v[r] = work[(j1 + r * P::R0 + r) * P::CPW + c1];  // prow(j + r R0) = j + r R0 + r
#pragma unroll
				for (int r = 1; r < P::R1; ++r)
					v[r] = cmulc(v[r], tw1[(r - 1) * P::R0 + j1]);
				Dft<P::R1, true>::run(v);
#pragma unroll
				for (int r = 0; r < P::R1; ++r) {
					const float m2 = v[r].x * v[r].x + v[r].y * v[r].y;
					acc[r] += STAT ? m2 : sqrt_approx(m2);
				}
			}
		}
		// scale once: |s y| = s |y| with s = 2 / N one-sided (1 / N two-sided)
		const float s = (q.one_sided ? 2.0f : 1.0f) / static_cast<float>(q.n);
		const float sc = STAT ? s * s : s;
		const int n2g = chunk * P::CW + warp * P::CPW + c1;
		MaxIdx best{-1.0f, 0xFFFFFFFFu};
		float sum = 0.f, sq = 0.f;
		if (n2g < n2) {
#pragma unroll
			for (int r = 0; r < P::R1; ++r) {  // n1 increases with r: strict > keeps the first maximum
				const float v = acc[r] * sc;
				if (v > best.v) {
					best.v = v;
					best.i = static_cast<uint32_t>(n2) * static_cast<uint32_t>(j1 + r * P::R0) + static_cast<uint32_t>(n2g);
				}
				sum += v;
				sq += v * v;
			}
		}
		double dsum = sum, dsq = sq;
		for (int o = 16; o > 0; o >>= 1) {
			const MaxIdx other{__shfl_down_sync(0xffffffffu, best.v, o), __shfl_down_sync(0xffffffffu, best.i, o)};
			best = better(best, other);
			dsum += __shfl_down_sync(0xffffffffu, dsum, o);
			dsq += __shfl_down_sync(0xffffffffu, dsq, o);
		}
		if (lane == 0) {
			s_max[warp] = best;
			s_sum[warp] = dsum;
			s_sq[warp] = dsq;
		}
		__syncthreads();
		if (threadIdx.x == 0) {
			for (int w = 1; w < P::WARPS; ++w) {
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
		const int d = q.d_base + row / q.n_codes;
		const int m = q.m;
		const double mean = ts / m;
		const double var = m > 1 ? (tq - ts * mean) / (m - 1) : 0.0;
		AcqCellDev cell;
		cell.level = rb.v;
		cell.index = rb.i;
		cell.mean = static_cast<float>(mean);
		cell.std = static_cast<float>(sqrt(var > 0 ? var : 0.0));
		q.cells[static_cast<size_t>(c) * q.n_doppler + d] = cell;
	}
}

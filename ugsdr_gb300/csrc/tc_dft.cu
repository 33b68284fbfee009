// Batched 25-point complex DFTs two ways, the measurement behind the
// transforms' place on the CUDA cores: the radix-25 stage of the four-step
// inverse (acq_batched.cuh) done
//   * on the 5th-generation tensor cores: per CTA a tile of 128 transforms is
//     one product D (128 x 64) = A (128 x 56) B^T with A the inputs as real
//     rows [re 0..24, im 0..24, 0...] and B the 25-point DFT as its real 50 x 50
//     block form, in TF32 with the 3xTF32 split (A_hi B_hi + A_hi B_lo +
//     A_lo B_hi, ~FP32 accuracy): 21 tcgen05.mma (M 128, N 64, K 8) from
//     shared-memory descriptors into a TMEM accumulator, completion through
//     an mbarrier (bounded wait), results read back with tcgen05.ld;
//   * on the CUDA cores: Dft<25> (fft_core.cuh) in registers, one transform
//     per thread — the butterfly the Stockham passes run.
// Entry: ugsdr_dft25_batch (device buffers, kernel time by CUDA events).
#include "internal.hpp"
#include "fft_core.cuh"

#include <cmath>

namespace ugsdr_gpu {
	namespace {
		constexpr int kTcM = 128;                      // transforms per tile (MMA M)
		constexpr int kTcK = 56;                       // 50 real inputs, 7 K steps of 8
		constexpr int kTcN = 64;                       // 50 real outputs, padded
		constexpr int kTcThreads = 128;                // 4 warps: warp w reads TMEM lanes 32w..32w+31
		constexpr int kCore = 128;                     // core matrix: 8 rows x 16 bytes
		constexpr int kLbo = kCore;                    // K-adjacent core matrices
		constexpr int kSbo = (kTcK / 4) * kCore;       // 8-row groups: 1792 bytes
		constexpr int kABytes = (kTcM / 8) * kSbo;     // 28,672
		constexpr int kBBytes = (kTcN / 8) * kSbo;     // 14,336
		constexpr int kStageBytes = kTcM * 25 * 8;        // a tile's outputs, staged for a coalesced store
		constexpr int kTcSmem = 2 * kABytes + 2 * kBBytes + kStageBytes + 128;
		constexpr int kTmemCols = 64;
		constexpr long long kSpinLimit = 1ll << 20;    // mbarrier polls before the tile is given up

		// byte offset of element (row, k) in a K-major, unswizzled tile of core matrices
		__device__ __forceinline__ int kmaj(int row, int k) {
			return (row >> 3) * kSbo + (k >> 2) * kCore + (row & 7) * 16 + (k & 3) * 4;
		}
		__device__ __forceinline__ uint32_t smem_u32(const void* p) {
			return static_cast<uint32_t>(__cvta_generic_to_shared(p));
		}
		__device__ __forceinline__ float tf32_round(float x) {
			uint32_t r;
			asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
			return __uint_as_float(r);
		}
		// hi / lo TF32 parts of x, stored at byte offset off of the two tiles
		__device__ __forceinline__ void put_split(unsigned char* hi, unsigned char* lo, int off, float x) {
			const float h = tf32_round(x);
			*reinterpret_cast<float*>(hi + off) = h;
			*reinterpret_cast<float*>(lo + off) = tf32_round(x - h);
		}
		// shared-memory matrix descriptor: start >> 4, LBO >> 4, SBO >> 4,
		// descriptor version 1, base offset 0, no swizzle
		__device__ __forceinline__ uint64_t smem_desc(uint32_t addr) {
			return static_cast<uint64_t>((addr & 0x3FFFFu) >> 4) | (static_cast<uint64_t>(kLbo >> 4) << 16) |
				(static_cast<uint64_t>(kSbo >> 4) << 32) | (1ull << 46);
		}
		// instruction descriptor, kind::tf32: D f32, A and B tf32, both K-major, N, M
		constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | (static_cast<uint32_t>(kTcN >> 3) << 17) |
			(static_cast<uint32_t>(kTcM >> 4) << 24);

		__device__ __forceinline__ void tc_mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
			asm volatile(
				"{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
				"tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
				"l"(a), "l"(b), "r"(kIdesc), "r"(accumulate));
		}
		__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
			uint32_t ok;
			asm volatile(
				"{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
				: "=r"(ok)
				: "r"(mbar), "r"(parity)
				: "memory");
			return ok != 0;
		}
#define UG_R8(i) "=r"(v[i]), "=r"(v[i + 1]), "=r"(v[i + 2]), "=r"(v[i + 3]), "=r"(v[i + 4]), "=r"(v[i + 5]), "=r"(v[i + 6]), "=r"(v[i + 7])
		// 32 consecutive TMEM columns of this warp's 32 lanes: v[j] = column col + j of lane (warp lane)
		__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
			asm volatile(
				"tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
				"%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
				: UG_R8(0), UG_R8(8), UG_R8(16), UG_R8(24)
				: "r"(taddr));
		}
#undef UG_R8

		// grid-stride over tiles of 128 transforms; `err` set when a tile's MMAs
		// did not complete within the poll limit
		__global__ void __launch_bounds__(kTcThreads) dft25_tc_kernel(const float2* __restrict__ in, float2* __restrict__ out,
			size_t count, int* err) {
			extern __shared__ __align__(128) unsigned char tc_smem[];
			unsigned char* a_hi = tc_smem;
			unsigned char* a_lo = a_hi + kABytes;
			unsigned char* b_hi = a_lo + kABytes;
			unsigned char* b_lo = b_hi + kBBytes;
			float2* stage = reinterpret_cast<float2*>(b_lo + kBBytes);
			__shared__ __align__(8) unsigned long long s_mbar;
			__shared__ uint32_t s_tmem;
			const int tid = threadIdx.x, warp = tid >> 5;
			// B: the 25-point DFT as a real 50 x 50 block (rows n: outputs re 0..24,
			// im 0..24; columns k: inputs re 0..24, im 0..24), zero padded
			for (int e = tid; e < kTcN * kTcK; e += blockDim.x) {
				const int n = e / kTcK, k = e - n * kTcK;
				double v = 0.0;
				if (n < 50 && k < 50) {
					const int on = n % 25, ik = k % 25;
					double s, c;
					sincospi(2.0 * static_cast<double>((on * ik) % 25) / 25.0, &s, &c);
					// y_re = sum xr c + xi s; y_im = sum -xr s + xi c
					v = n < 25 ? (k < 25 ? c : s) : (k < 25 ? -s : c);
				}
				put_split(b_hi, b_lo, kmaj(n, k), static_cast<float>(v));
			}
			// A's padding columns (k 50..55) stay zero
			for (int e = tid; e < kTcM * (kTcK - 50); e += blockDim.x) {
				const int m = e / (kTcK - 50), k = 50 + e % (kTcK - 50);
				put_split(a_hi, a_lo, kmaj(m, k), 0.f);
			}
			if (tid == 0) {
				asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&s_mbar)));
				asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
			}
			if (warp == 0) {
				asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_u32(&s_tmem)),
					"r"(kTmemCols));
				asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
			}
			asm volatile("tcgen05.fence::before_thread_sync;\n");
			__syncthreads();
			asm volatile("tcgen05.fence::after_thread_sync;\n");
			const uint32_t tmem = s_tmem;
			const uint32_t mbar = smem_u32(&s_mbar);
			const uint32_t a_hi_s = smem_u32(a_hi), a_lo_s = smem_u32(a_lo), b_hi_s = smem_u32(b_hi), b_lo_s = smem_u32(b_lo);
			const size_t tiles = (count + kTcM - 1) / kTcM;
			uint32_t parity = 0;
			for (size_t t = blockIdx.x; t < tiles; t += gridDim.x) {
				const size_t m0 = t * kTcM;
				const int rows = static_cast<int>(min(static_cast<size_t>(kTcM), count - m0));
				// the tile's inputs, coalesced, into A (rows past `count` keep stale values; never stored)
				const float2* src = in + m0 * 25;
				for (int e = tid; e < rows * 25; e += blockDim.x) {
					const int m = e / 25, j = e - m * 25;
					const float2 x = src[e];
					put_split(a_hi, a_lo, kmaj(m, j), x.x);
					put_split(a_hi, a_lo, kmaj(m, 25 + j), x.y);
				}
				asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // generic writes -> tensor core reads
				__syncthreads();
				if (tid == 0) {
					asm volatile("tcgen05.fence::after_thread_sync;\n");
					const uint32_t as[3] = {a_lo_s, a_hi_s, a_hi_s}, bs[3] = {b_hi_s, b_lo_s, b_hi_s};  // small terms first
					uint32_t acc = 0;
					for (int pr = 0; pr < 3; ++pr)
						for (int s = 0; s < kTcK / 8; ++s) {
							tc_mma(tmem, smem_desc(as[pr] + s * 2 * kCore), smem_desc(bs[pr] + s * 2 * kCore), acc);
							acc = 1;
						}
					asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mbar)
						: "memory");
				}
				bool done = false;
				for (long long it = 0; it < kSpinLimit && !done; ++it)
					done = mbar_try(mbar, parity);
				if (__syncthreads_or(!done)) {
					if (tid == 0)
						atomicExch(err, 1);
					break;  // every thread leaves the loop together
				}
				parity ^= 1u;
				asm volatile("tcgen05.fence::after_thread_sync;\n");
				// thread tid holds transform m0 + tid: columns 0..24 re, 25..49 im;
				// staged for a coalesced store
				uint32_t lo[32], hi[32];
				const uint32_t lane_base = tmem + (static_cast<uint32_t>(warp * 32) << 16);
				tmem_ld32(lane_base, lo);
				tmem_ld32(lane_base + 32, hi);
				asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
				for (int k = 0; k < 25; ++k) {
					const uint32_t im = 25 + k < 32 ? lo[25 + k] : hi[25 + k - 32];
					stage[tid * 25 + k] = c2(__uint_as_float(lo[k]), __uint_as_float(im));
				}
				asm volatile("tcgen05.fence::before_thread_sync;\n");
				__syncthreads();  // TMEM read, outputs staged
				float2* dst = out + m0 * 25;
				for (int e = tid; e < rows * 25; e += blockDim.x)
					dst[e] = stage[e];
				__syncthreads();  // the stage read before the next tile rewrites it
			}
			__syncthreads();
			if (warp == 0) {
				asm volatile("tcgen05.fence::after_thread_sync;\n");
				asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols));
			}
		}

		// CUDA-core butterfly: one 25-point transform per thread, tiles of 128
		// transforms staged through shared memory as the tensor-core kernel does
		__global__ void __launch_bounds__(kTcThreads) dft25_cuda_kernel(const float2* __restrict__ in, float2* __restrict__ out,
			size_t count) {
			__shared__ float2 stage[kTcM * 25];
			const int tid = threadIdx.x;
			const size_t tiles = (count + kTcM - 1) / kTcM;
			for (size_t t = blockIdx.x; t < tiles; t += gridDim.x) {
				const size_t m0 = t * kTcM;
				const int rows = static_cast<int>(min(static_cast<size_t>(kTcM), count - m0));
				for (int e = tid; e < rows * 25; e += blockDim.x)
					stage[e] = in[m0 * 25 + e];
				__syncthreads();
				if (tid < rows) {
					float2 v[25];
#pragma unroll
					for (int j = 0; j < 25; ++j)
						v[j] = stage[tid * 25 + j];
					Dft<25, false>::run(v);
#pragma unroll
					for (int j = 0; j < 25; ++j)
						stage[tid * 25 + j] = v[j];
				}
				__syncthreads();
				for (int e = tid; e < rows * 25; e += blockDim.x)
					out[m0 * 25 + e] = stage[e];
				__syncthreads();
			}
		}
	}
}

using namespace ugsdr_gpu;

extern "C" int ugsdr_dft25_batch(ugsdr_ctx* ctx, const void* in, void* out, size_t count, int method, float* kernel_ms) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		require(in && out && count > 0 && count <= (static_cast<size_t>(1) << 32), "null buffer or count out of range");
		require(method == UGSDR_DFT25_CUDA_CORES || method == UGSDR_DFT25_TENSOR_CORES, "unknown method");
		cudaEvent_t e0, e1;
		UG_CUDA(cudaEventCreate(&e0));
		UG_CUDA(cudaEventCreate(&e1));
		DevBuf err;
		err.reserve(sizeof(int));
		UG_CUDA(cudaMemsetAsync(err.ptr, 0, sizeof(int), ctx->stream));
		UG_CUDA(cudaEventRecord(e0, ctx->stream));
		if (method == UGSDR_DFT25_TENSOR_CORES) {
			UG_CUDA(cudaFuncSetAttribute(dft25_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem));
			const size_t tiles = (count + kTcM - 1) / kTcM;
			const int grid = static_cast<int>(std::min<size_t>(tiles, static_cast<size_t>(ctx->sm_count) * 2));
			dft25_tc_kernel<<<grid, kTcThreads, kTcSmem, ctx->stream>>>(static_cast<const float2*>(in), static_cast<float2*>(out),
				count, err.as<int>());
		}
		else {
			const size_t tiles = (count + kTcM - 1) / kTcM;
			const int grid = static_cast<int>(std::min<size_t>(tiles, static_cast<size_t>(ctx->sm_count) * 8));
			dft25_cuda_kernel<<<grid, kTcThreads, 0, ctx->stream>>>(static_cast<const float2*>(in), static_cast<float2*>(out), count);
		}
		note_launch(ctx);
		UG_CUDA(cudaEventRecord(e1, ctx->stream));
		int flag = 0;
		UG_CUDA(cudaMemcpyAsync(&flag, err.ptr, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
		UG_CUDA(cudaStreamSynchronize(ctx->stream));
		float ms = 0.f;
		UG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
		cudaEventDestroy(e0);
		cudaEventDestroy(e1);
		require(flag == 0, "tensor-core DFT: an MMA did not complete within the poll limit", UGSDR_E_TIMEOUT);
		if (kernel_ms)
			*kernel_ms = ms;
	});
}

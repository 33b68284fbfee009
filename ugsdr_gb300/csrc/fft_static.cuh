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
				const float2* wk = tw + k * (R - 1) - 1;  // this pass's table, [k][r - 1]
#pragma unroll
				for (int r = 1; r < R; ++r) {
					const float2 w = wk[r];
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

	// twiddle entries of a pass: W_N^{r k N / (NS R)} for k < NS, 1 <= r < R
	template <int NS, int R>
	constexpr int pass_table_size() {
		return NS > 1 ? NS * (R - 1) : 0;
	}

	template <int N, int NS, bool INV, int R, int... Rest>
	struct StaticPasses<N, NS, INV, R, Rest...> {
		__device__ static float2* run(float2* a, float2* b, const float2* tw, int batch, int ld) {
			static_pass<N, R, NS, INV>(a, b, tw, batch, ld);
			__syncthreads();
			return StaticPasses<N, NS * R, INV, Rest...>::run(b, a, tw + pass_table_size<NS, R>(), batch, ld);
		}
	};

	// Hooked pass: when FIRST, inputs come from load(f, i) (element i of
	// transform f) instead of `in`; when LAST, each butterfly's outputs go to
	// emit.put<R, NS>(f, base, v) — v[r] is output element base + r * NS —
	// instead of `out`.  Fusing the producer and consumer into the first and
	// last passes saves a shared-memory round trip and a barrier each.
	// The threads that run a pass together: the whole CTA (one __syncthreads
	// between passes) or one warp owning its transforms (__syncwarp).
	struct CtaGroup {
		__device__ static int rank() { return threadIdx.x; }
		__device__ static int size() { return blockDim.x; }
		__device__ static void sync() { __syncthreads(); }
	};
	struct WarpGroup {
		__device__ static int rank() { return threadIdx.x & 31; }
		__device__ static int size() { return 32; }
		__device__ static void sync() { __syncwarp(); }
	};

	// A load hook may declare kZeroFrom: its elements i >= kZeroFrom are zero
	// in every transform (a one-sided spectrum's upper half).  Pass 0 then
	// reads only the inputs r < live_inputs() of each butterfly and runs the
	// pruned DFT (the same values but for the sign of exact zeros).
	template <class L, class = void>
	struct ZeroFrom {
		static constexpr int value = 1 << 30;
	};
	template <class L>
	struct ZeroFrom<L, std::void_t<decltype(L::kZeroFrom)>> {
		static constexpr int value = L::kZeroFrom;
	};
	// inputs r of a pass-0 butterfly (element j + r N / R, j < N / R) that
	// may be non-zero: r < ceil(kZeroFrom / (N / R))
	template <class L, int N, int R>
	constexpr int live_inputs() {
		constexpr long zf = ZeroFrom<L>::value, nb = N / R;
		return zf >= N ? R : static_cast<int>((zf + nb - 1) / nb);
	}

	template <int N, int R, int NS, bool INV, bool FIRST, bool LAST, class Load, class Emit, class G = CtaGroup>
	__device__ __forceinline__ void hooked_pass(const float2* __restrict__ in, float2* __restrict__ out,
		const float2* __restrict__ tw, int batch, int ld, Load& load, Emit& emit) {
		constexpr int NB = N / R;
		constexpr int RL = FIRST ? live_inputs<Load, N, R>() : R;
		static_assert(RL >= 1 && RL <= R, "pass 0 reads at least its first input");
		const int total = NB * batch;
		for (int u = G::rank(); u < total; u += G::size()) {
			const int f = u / NB;
			const int j = u - f * NB;
			const int k = NS == 1 ? 0 : j % NS;
			float2 v[R];
			if constexpr (FIRST) {
#pragma unroll
				for (int r = 0; r < RL; ++r)
					v[r] = load(f, j + r * NB);
			}
			else {
				const float2* src = in + f * ld + j;
#pragma unroll
				for (int r = 0; r < R; ++r)
					v[r] = src[r * NB];
			}
			if constexpr (NS > 1) {
				const float2* wk = tw + k * (R - 1) - 1;  // this pass's table, [k][r - 1]
#pragma unroll
				for (int r = 1; r < R; ++r) {
					const float2 w = wk[r];
					v[r] = INV ? cmulc(v[r], w) : cmul(v[r], w);
				}
			}
			if constexpr (RL < R)
				DftPruned<R, INV, RL>::run(v);
			else
				Dft<R, INV>::run(v);
			if constexpr (LAST) {
				emit.template put<R, NS>(f, (j - k) * R + k, v);
			}
			else {
				float2* dst = out + f * ld + (j - k) * R + k;
#pragma unroll
				for (int r = 0; r < R; ++r)
					dst[r * NS] = v[r];
			}
		}
	}

	// a between-passes hook that does nothing
	struct NoMid {
		__device__ void operator()() const {}
	};

	template <class G, int N, int NS, bool INV, bool FIRST, int... Rs>
	struct HookedPasses;

	template <class G, int N, int NS, bool INV, bool FIRST, int R, int... Rest>
	struct HookedPasses<G, N, NS, INV, FIRST, R, Rest...> {
		template <class Load, class Emit, class Mid>
		__device__ static void run(float2* a, float2* b, const float2* tw, int batch, int ld, Load& load, Emit& emit, Mid& mid) {
			constexpr bool LAST = sizeof...(Rest) == 0;
			hooked_pass<N, R, NS, INV, FIRST, LAST, Load, Emit, G>(a, b, tw, batch, ld, load, emit);
			if constexpr (!LAST) {
				G::sync();
				if constexpr (NS == 1)
					mid();  // pass 0's input tile is free from here on
				HookedPasses<G, N, NS * R, INV, false, Rest...>::run(b, a, tw + pass_table_size<NS, R>(), batch, ld, load, emit, mid);
			}
		}
	};

	template <int... Rs>
	constexpr int radix_product() {
		return (1 * ... * Rs);
	}

	// Per-pass twiddle tables, pass after pass, entry [k][r - 1] = tw[r k N / (NS R)]
	// (tw: the N-point table exp(-2 pi i m / N)); a fixed r is a stride-(R - 1)
	// read across lanes, free of the bank conflicts of tw[r k] itself.
	template <int N, int NS, int R, int... Rest>
	__device__ __forceinline__ void build_pass_tables(float2* dst, const float2* __restrict__ tw) {
		if constexpr (NS > 1) {
			constexpr int STEP = N / (NS * R);
			for (int e = threadIdx.x; e < NS * (R - 1); e += blockDim.x) {
				const int k = e / (R - 1);
				const int r = e - k * (R - 1) + 1;
				dst[e] = __ldg(tw + r * k * STEP);
			}
		}
		if constexpr (sizeof...(Rest) > 0)
			build_pass_tables<N, NS * R, Rest...>(dst + pass_table_size<NS, R>(), tw);
	}

	template <int NS, int R, int... Rest>
	constexpr int tables_size() {
		if constexpr (sizeof...(Rest) > 0)
			return pass_table_size<NS, R>() + tables_size<NS * R, Rest...>();
		else
			return pass_table_size<NS, R>();
	}

	template <int... Rs>
	constexpr int radix_last() {
		int l = 1;
		((l = Rs), ...);
		return l;
	}

	template <int R, int... Rest>
	constexpr int radix_first() {
		return R;
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
		static constexpr bool kHooked = true;  // kernels fuse their producer/consumer into the first/last pass
		static constexpr int kPasses = sizeof...(Rs);
		// stride of the last pass (its butterflies start at base = j < kLastNS)
		static constexpr int kLastNS = N_ / radix_last<Rs...>();
		// butterflies of pass 0 per transform (its inputs j + r kFirstNB)
		static constexpr int kFirstNB = N_ / radix_first<Rs...>();
		// inverse row kernel launch bounds: a hooked two-pass plan whose widest
		// pass over 8 rows fits 224 threads runs one shared tile and four CTAs
		// per SM (72 registers), other plans two tiles and three CTAs
		static constexpr bool kRowsCompact = kPasses == 2 && 8 * (N_ / radix_min<Rs...>()) <= 224;
		static constexpr int kRowsMaxThreads = kRowsCompact ? 224 : 256;
		static constexpr int kRowsMinBlocks = kRowsCompact ? 4 : 3;
		// inverse column kernel: a hooked two-pass plan of the same width
		// prefetches the next block into the input tile once pass 0 has read it
		// (two tiles + accumulator, three CTAs per SM, four for N <= 256 whose
		// tiles are small); other plans keep a third prefetch tile and run two
		static constexpr bool kColsCompact = kRowsCompact;
		static constexpr int kColsMaxThreads = kColsCompact ? 224 : 256;
		static constexpr int kColsMinBlocks = kColsCompact ? (N_ <= 256 ? 4 : 3) : 2;
		// forward column kernel (one item per CTA, two tiles): four CTAs per SM
		// for a compact plan
		static constexpr int kFwdColsMinBlocks = kColsCompact ? 4 : 3;
		// most butterflies of one pass over `batch` transforms
		static constexpr int most_butterflies(int batch) { return batch * (N_ / radix_min<Rs...>()); }
		static_assert(tables_size<1, Rs...>() <= N_, "pass tables fit the N-entry table space");
		// Builds the pass tables at `dst` (16-byte aligned, room for N entries)
		// from the plan's N-point table (global memory); returns the plan
		// pointing at them.  Call before the CTA's first barrier.
		__device__ static FftPlanDev prepare(const FftPlanDev& plan, void* dst) {
			float2* t = reinterpret_cast<float2*>((reinterpret_cast<uintptr_t>(dst) + 15) & ~static_cast<uintptr_t>(15));
			build_pass_tables<N_, 1, Rs...>(t, plan.tw);
			FftPlanDev out = plan;
			out.tw = t;
			return out;
		}
		template <bool INV>
		__device__ static float2* run(float2* a, float2* b, const FftPlanDev& plan, int batch, int ld) {
			return StaticPasses<N_, 1, INV, Rs...>::run(a, b, plan.tw, batch, ld);
		}
		// Pass 0 reads `a` (or gathers through `load` when FIRST), intermediate
		// passes ping-pong between the tiles, the last pass emits.  With FIRST and
		// two radices only one tile (`b`) is used.
		// `mid()` runs after the barrier that ends pass 0.
		template <bool INV, bool FIRST, class Load, class Emit, class Mid>
		__device__ static void run_hooked(float2* a, float2* b, const FftPlanDev& plan, int batch, int ld, Load& load, Emit& emit, Mid& mid) {
			HookedPasses<CtaGroup, N_, 1, INV, FIRST, Rs...>::run(a, b, plan.tw, batch, ld, load, emit, mid);
		}
		// the same passes run by one warp over its own transforms (tiles private
		// to the warp; the pass tables shared by the CTA)
		template <bool INV, bool FIRST, class Load, class Emit, class Mid>
		__device__ static void run_hooked_warp(float2* a, float2* b, const FftPlanDev& plan, int batch, int ld, Load& load, Emit& emit,
			Mid& mid) {
			HookedPasses<WarpGroup, N_, 1, INV, FIRST, Rs...>::run(a, b, plan.tw, batch, ld, load, emit, mid);
		}
		template <bool INV, bool FIRST, class Load, class Emit>
		__device__ static void run_hooked(float2* a, float2* b, const FftPlanDev& plan, int batch, int ld, Load& load, Emit& emit) {
			NoMid mid{};
			run_hooked<INV, FIRST>(a, b, plan, batch, ld, load, emit, mid);
		}
	};

	// The same plan with the kernels' separate load / epilogue loops (for
	// plans whose fused first pass would hold too many registers).
	template <int N_, int... Rs>
	struct StaticFftPlain : StaticFft<N_, Rs...> {
		static constexpr bool kHooked = false;
		static constexpr bool kRowsCompact = false;
		static constexpr int kRowsMaxThreads = 256;
		static constexpr int kRowsMinBlocks = 3;
		static constexpr bool kColsCompact = false;
		static constexpr int kColsMaxThreads = 256;
		static constexpr int kColsMinBlocks = 2;
		static constexpr int kFwdColsMinBlocks = 3;
	};

	// a load hook for plans that read their first pass from shared memory
	struct NoLoad {
		__device__ float2 operator()(int, int) const { return c2(0.f, 0.f); }
	};
}

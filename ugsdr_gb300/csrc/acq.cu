// Batched acquisition engine: FFT planning, code-spectrum cache, job launch.
// Host side of the kernels in acq_kernels.cuh / acq_large.cuh; C entry points
// ugsdr_code_put / ugsdr_code_release / ugsdr_acquire / ugsdr_acquire_batch.
#include "internal.hpp"
#include "acq_kernels.cuh"
#include "acq_batched.cuh"
#include "acq_cols_warp.cuh"
#include "dfe.cuh"
#include "fft_plan.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <numeric>
#include <tuple>
#include <vector>

namespace ugsdr_gpu {

	namespace {
		constexpr int kThreads = 256;

		void upload_twiddles(ugsdr_ctx* ctx, int n) {
			if (ctx->twiddles.count(n))
				return;
			std::vector<float2> tw(n);
			const double two_pi = 2.0 * 3.14159265358979323846;
			for (int m = 0; m < n; ++m) {
				const double a = two_pi * static_cast<double>(m) / static_cast<double>(n);
				tw[m] = c2(static_cast<float>(std::cos(a)), static_cast<float>(-std::sin(a)));
			}
			auto buf = std::make_unique<DevBuf>();
			buf->reserve(sizeof(float2) * n);
			UG_CUDA(cudaMemcpy(buf->ptr, tw.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
			ctx->twiddles[n] = std::move(buf);
		}

		FftPlanDev to_dev(const FftPlanDesc& d) {
			FftPlanDev p{};
			p.n = d.n;
			p.n_pass = d.n_pass;
			for (int i = 0; i < d.n_pass; ++i)
				p.radix[i] = d.radix[i];
			p.tw = d.tw;
			return p;
		}

		template <typename K>
		void set_smem(K kernel, size_t bytes) {
			static std::mutex mu;
			std::lock_guard<std::mutex> lock(mu);
			UG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)));
		}
	}

	void note_launch(ugsdr_ctx* ctx, int n) {
		ctx->launches += n;
		UG_CUDA(cudaGetLastError());
	}

	const FftPlanDesc& get_plan(ugsdr_ctx* ctx, int n) {
		auto it = ctx->plans.find(n);
		if (it != ctx->plans.end())
			return it->second;
		std::vector<int> r;
		require(n >= 2 && plan_radices(n, r) && static_cast<int>(r.size()) <= kMaxPasses,
			"FFT size " + std::to_string(n) + " has a prime factor above 31", UGSDR_E_UNSUPPORTED);
		upload_twiddles(ctx, n);
		FftPlanDesc d;
		d.n = n;
		d.n_pass = static_cast<int>(r.size());
		for (size_t i = 0; i < r.size(); ++i)
			d.radix[i] = r[i];
		d.tw = ctx->twiddles[n]->as<float2>();
		return ctx->plans[n] = d;
	}

	const float* get_lut(ugsdr_ctx* ctx) {
		if (!ctx->lut.ptr) {
			// TableMixer::GetSinCosTable<6, float> (table_mixer.hpp:31-47):
			// 80 entries sin(i * 5 pi / 80 / 2), computed in double, stored as float
			float t[80];
			const double step = 5 * 3.14159265358979323846 / 80 / 2;
			for (int i = 0; i < 80; ++i)
				t[i] = static_cast<float>(std::sin(static_cast<double>(i) * step));
			ctx->lut.reserve(sizeof(t));
			UG_CUDA(cudaMemcpy(ctx->lut.ptr, t, sizeof(t), cudaMemcpyHostToDevice));
		}
		return ctx->lut.as<float>();
	}

	// Single-CTA path: ping-pong buffers (2 N complex) + accumulator (N floats)
	bool fits_single_cta(ugsdr_ctx* ctx, int n) {
		return static_cast<size_t>(n) * (2 * sizeof(float2) + sizeof(float)) + 1024 <= ctx->smem_optin;
	}

	// ------------------------------------------------------ large-N path
	// Shape of one job as the large path needs it.
	struct JobLaunchShape {
		int n = 0, k = 0, m = 0, rows = 0, fold_mode = 0;
	};

	namespace {
		// N = a x (n / a) with plans for both factors whose kernels' tiles and
		// twiddle tables fit with at least min_cols columns (inverse: 3 tiles +
		// accumulator) and one row (2 tiles)
		bool split_fits(ugsdr_ctx* ctx, int n, int a, int min_cols) {
			std::vector<int> r;
			if (a < 2 || n % a || n / a < 2 || !plan_radices(a, r) || !plan_radices(n / a, r))
				return false;
			const size_t budget = ctx->smem_optin - 2048;
			const size_t cols = (3 * sizeof(float2) + sizeof(float)) * min_cols * static_cast<size_t>(a | 1) + sizeof(float2) * a + 16;
			const size_t rows = 3 * sizeof(float2) * static_cast<size_t>(n / a) + 16;
			return cols <= budget && rows <= budget;
		}
	}

	// The built-in split: the largest N1 <= sqrt(N) that fits with 4 columns
	// per CTA; the largest sizes (beyond ~1.8e7 points) fall back to single
	// columns.
	int rule_split(ugsdr_ctx* ctx, int n) {
		for (const int min_cols : {4, 1}) {
			int best1 = 0;
			for (int a = 2; static_cast<long>(a) * a <= n; ++a)
				if (split_fits(ctx, n, a, min_cols))
					best1 = a;  // increasing a -> closest to sqrt(n) last
			if (best1 > 0)
				return best1;
		}
		return 0;
	}

	const LargePlan& get_large_plan(ugsdr_ctx* ctx, int n) {
		auto it = ctx->large_plans.find(n);
		if (it != ctx->large_plans.end())
			return it->second;
		const auto t = ctx->tiles.find(n);
		const int best1 = t != ctx->tiles.end() && t->second.n1 > 0 ? t->second.n1 : rule_split(ctx, n);
		require(best1 > 0, "no four-step split for FFT size " + std::to_string(n), UGSDR_E_UNSUPPORTED);
		LargePlan lp;
		lp.n = n;
		lp.n1 = best1;
		lp.n2 = n / best1;
		lp.p1 = get_plan(ctx, lp.n1);
		lp.p2 = get_plan(ctx, lp.n2);
		return ctx->large_plans[n] = lp;
	}

	namespace {
		constexpr int kBatchedThreads = 256;

		// Threads for a CTA running `batch` FFTs of `plan`: enough for the
		// pass with the most butterflies, rounded to whole warps (<= 256, the
		// kernels' launch bound), so no pass leaves more than a warp idle.
		int threads_for(const FftPlanDev& plan, int batch) {
			int most = 0;
			for (int s = 0; s < plan.n_pass; ++s)
				most = std::max(most, batch * plan.n / plan.radix[s]);
			return std::min(kBatchedThreads, std::max(64, (most + 31) / 32 * 32));
		}
		template <class F>
		int threads_of(const FftPlanDev& plan, int batch) {
			if constexpr (F::N > 0)
				return std::min(kBatchedThreads, std::max(64, (F::most_butterflies(batch) + 31) / 32 * 32));
			else
				return threads_for(plan, batch);
		}

		// Compile-time sub-FFT plans for the N1 x N2 splits of the configured
		// block sizes (get_large_plan's choice: the largest N1 <= sqrt(N)),
		// odd radices first; other sizes run the runtime plan.
		template <class Fn>
		void with_large_ffts(int n1, int n2, Fn&& fn) {
			if (n1 == 200 && n2 == 250)
				fn(StaticFft<200, 25, 8>{}, StaticFft<250, 25, 10>{});          // 50,000: 1 ms at 50 MHz
			else if (n1 == 400 && n2 == 500)
				fn(StaticFft<400, 25, 16>{}, StaticFft<500, 25, 20>{});         // 200,000: 4 ms at 50 MHz
			else if (n1 == 440 && n2 == 465)  // 204,600: 10 ms at 20.46 MHz; fusing the radix-31 rows spills
				fn(StaticFft<440, 11, 5, 8>{}, StaticFftPlain<465, 31, 15>{});
			else if (n2 == 1000)  // 0.75 - 1 M points (15 - 20 ms at 50 MHz): compile-time rows
				fn(RuntimeFft{}, StaticFft<1000, 10, 10, 10>{});
			else
				fn(RuntimeFft{}, RuntimeFft{});
		}

		// Sub-transforms per CTA: 8 columns/rows (64-byte runs per k1 row) unless
		// the tiles would exceed a third of shared memory.
		// Sized for inv_cols with three column tiles (input, work, prefetch) and
		// an accumulator at two CTAs per SM (a compact plan drops the prefetch
		// tile and runs three), and for row kernels with two row tiles at three.
		void tile_shape(ugsdr_ctx* ctx, const LargePlan& lp, int& cw, int& rw) {
			const size_t ld = static_cast<size_t>(lp.n1 | 1);
			bool compact = false;  // the column plan's inverse kernel keeps two tiles, not three
			with_large_ffts(lp.n1, lp.n2, [&](auto f1, auto) { compact = decltype(f1)::kColsCompact; });
			auto cols_bytes = [&](int c) { return (3 * sizeof(float2) + sizeof(float)) * c * ld + sizeof(float2) * lp.n1 + 16; };
			cw = 8;
			while (cw > 1 && cols_bytes(cw) > (ctx->smem_optin - 2048) / 2)
				cw /= 2;
			// a three-tile plan whose 8-column tiles leave only two CTAs per SM
			// runs 4-column tiles (more, smaller CTAs: 11 % faster on the
			// 440-point columns of the 204,600-point L5 blocks)
			if (!compact && cw == 8 && cols_bytes(8) > (ctx->smem_optin - 2048) / 3)
				cw = 4;
			rw = 8;
			while (rw > 1 && 2 * sizeof(float2) * rw * static_cast<size_t>(lp.n2) + sizeof(float2) * lp.n2 + 16 > (ctx->smem_optin - 2048) / 3)
				rw /= 2;
			// a set or tuned shape (checked against the kernels' limits when set)
			const auto t = ctx->tiles.find(lp.n);
			if (t != ctx->tiles.end()) {
				if (t->second.cw > 0)
					cw = t->second.cw;
				if (t->second.rw > 0)
					rw = t->second.rw;
			}
		}

		// Column plans of the warp-owned column kernel (unfolded rows): N1 = 400
		// (200,000-point blocks) and 200 (50,000-point blocks), radix 25 last.
		// two warps per CTA (7 CTAs per SM): the default step measured 100.0 ms,
		// against 102.1 with four warps for the 200-point columns and 103.5
		// with four for both
		using ColsWarp400 = ColsWarpPlan<400, 16, 25, 2, 7>;
		using ColsWarp200 = ColsWarpPlan<200, 8, 25, 2, 7>;
		template <class Fn>
		bool with_cols_warp(int n1, int n2, Fn&& fn) {
			if (n1 == 400 && n2 == 500)
				fn(ColsWarp400{});
			else if (n1 == 200 && n2 == 250)
				fn(ColsWarp200{});
			else
				return false;
			return true;
		}

		// warp-owned row kernel (with the warp-owned columns): rows per warp —
		// three 250-point rows (30 of 32 lanes in the radix-25 pass), one
		// 500-point row (20 of 32) — and four warps per CTA
		template <int N2>
		constexpr int kRowsPerWarp = N2 <= 256 ? 3 : 1;
		constexpr int kRowsWarps = 4;
		// 0: CTA row tiles; 1: warp-owned rows (the rule); 2: warp-owned, three
		// rows per warp, code rows through L1 / L2
		int warp_rows_mode(ugsdr_ctx* ctx, int n) {
			const auto t = ctx->tiles.find(n);
			return t == ctx->tiles.end() || t->second.warp_rows < 0 ? 1 : t->second.warp_rows;
		}

		// columns per column-kernel CTA of the blocked layout (0: natural layout)
		int blocked_cw(ugsdr_ctx* ctx, int n, int n1, int n2, int fold_mode) {
			if (fold_mode != 0 || std::getenv("UGSDR_NO_WARP_COLS"))
				return 0;
			const auto t = ctx->tiles.find(n);
			if (t != ctx->tiles.end() && t->second.warp_cols == 0)
				return 0;
			int cw = 0;
			with_cols_warp(n1, n2, [&](auto plan) { cw = decltype(plan)::CW; });
			return cw;
		}

		BatchedParams batched_params(ugsdr_ctx* ctx, const AcqParams& base, int n) {
			const LargePlan& lp = get_large_plan(ctx, n);
			BatchedParams p{};
			p.base = base;
			p.p1 = to_dev(lp.p1);
			p.p2 = to_dev(lp.p2);
			p.n1 = lp.n1;
			p.n2 = lp.n2;
			tile_shape(ctx, lp, p.cw, p.rw);
			p.ld1 = lp.n1 | 1;  // odd column stride: the 8 columns of a tile fall in distinct banks
			p.n2p = lp.n2;
			p.cw_shift = 0;
			while ((1 << p.cw_shift) < p.cw)
				++p.cw_shift;
			return p;
		}

		// fwd_cols: two tiles + the N1-point twiddle table
		size_t smem_cols(const BatchedParams& p) {
			return 2 * sizeof(float2) * static_cast<size_t>(p.cw) * p.ld1 + sizeof(float2) * p.n1 + 16;
		}
		// inv_cols: input, work and (not for a compact plan) prefetch tiles +
		// accumulator + table
		template <class F>
		size_t smem_inv_cols(const BatchedParams& p) {
			return ((F::kColsCompact ? 2 : 3) * sizeof(float2) + sizeof(float)) * static_cast<size_t>(p.cw) * p.ld1
				+ sizeof(float2) * p.n1 + 16;
		}
		// row kernels: two tiles + the N2-point twiddle table
		size_t smem_rows(const BatchedParams& p, bool) {
			return 2 * sizeof(float2) * static_cast<size_t>(p.rw) * p.n2 + sizeof(float2) * p.n2 + 16;
		}
		// inverse rows: work tile(s), the staged X (and code) rows of hooked
		// plans, the twiddle table
		template <class F>
		size_t smem_inv_rows(const BatchedParams& p) {
			return rows_tiles<F>() * sizeof(float2) * static_cast<size_t>(p.rw) * p.n2 + sizeof(float2) * p.n2 + 16 +
				(F::kHooked ? sizeof(float2) * static_cast<size_t>(p.rw) * (F::kLastNS + 1) : 0);  // twiddle seeds
		}

		int chunks_of(int total, int per) { return (total + per - 1) / per; }

		// rows per inverse batch: B (rows x K x N complex) within 8 GiB — large
		// enough that a batch is thousands of CTAs and a search a few hundred
		// launches at most (the host then never waits on a full launch queue)
		int batch_rows(const JobLaunchShape& s, size_t b_points) {
			const size_t per_row = sizeof(float2) * b_points * s.k;
			const size_t budget = static_cast<size_t>(8) << 30;
			return static_cast<int>(std::max<size_t>(1, std::min<size_t>(s.rows, budget / per_row)));
		}

		template <typename K>
		void launch_fwd_cols(ugsdr_ctx* ctx, K kernel, const BatchedParams& p, int items, int threads) {
			const size_t smem = smem_cols(p);
			set_smem(kernel, smem);
			kernel<<<items * chunks_of(p.n2, p.cw), threads, smem, ctx->stream>>>(p);
		}

		void launch_forward(ugsdr_ctx* ctx, int sample_type, const BatchedParams& p, int items) {
			with_large_ffts(p.n1, p.n2, [&](auto f1, auto f2) {
				using F1 = decltype(f1);
				using F2 = decltype(f2);
				const int t1 = threads_of<F1>(p.p1, p.cw);
				switch (sample_type) {
				case UGSDR_SAMPLES_CF32: launch_fwd_cols(ctx, fwd_cols_kernel<UGSDR_SAMPLES_CF32, F1>, p, items, t1); break;
				case UGSDR_SAMPLES_CI8: launch_fwd_cols(ctx, fwd_cols_kernel<UGSDR_SAMPLES_CI8, F1>, p, items, t1); break;
				case UGSDR_SAMPLES_CI16: launch_fwd_cols(ctx, fwd_cols_kernel<UGSDR_SAMPLES_CI16, F1>, p, items, t1); break;
				default: launch_fwd_cols(ctx, fwd_cols_kernel<UGSDR_SAMPLES_RI8, F1>, p, items, t1); break;
				}
				// signal items of the two-pass 250- / 500-point row plans: warp-owned rows
				if constexpr (F2::kHooked && F2::kPasses == 2 && (F2::N == 250 || F2::N == 500)) {
					if (!p.code_mode && !std::getenv("UGSDR_NO_WARP_FWD_ROWS")) {
						constexpr int RPW = kRowsPerWarp<F2::N>, W = kRowsWarps;
						constexpr size_t smem = fwd_rows_warp_smem<F2, RPW, W>();
						set_smem(fwd_rows_warp_kernel<F2, RPW, W>, smem);
						const int groups = (items + kFwdRowItems - 1) / kFwdRowItems;
						fwd_rows_warp_kernel<F2, RPW, W><<<groups * chunks_of(p.n1, RPW * W), 32 * W, smem, ctx->stream>>>(p, items);
						return;
					}
				}
				const size_t smem = smem_rows(p, false);
				set_smem(fwd_rows_kernel<F2>, smem);
				const int groups = F2::kRowsCompact ? (items + kFwdRowItems - 1) / kFwdRowItems : items;
				fwd_rows_kernel<F2><<<groups * chunks_of(p.n1, p.rw), threads_of<F2>(p.p2, p.rw), smem, ctx->stream>>>(p, items);
			});
			note_launch(ctx, 2);
		}
	}

	namespace {
		// Scratch layout of one large-path launch (B, partials, sums, counters,
		// fold buffers), each region 256-byte aligned; sizing and carving both
		// walk it, so they agree byte for byte.
		struct ScratchLayout {
			size_t bbuf = 0, partials = 0, sums = 0, counters = 0, accg = 0, zcg = 0, total = 0;
			ScratchLayout(const JobLaunchShape& s, int r_max, int chunks, size_t b_points) {
				auto region = [&](size_t bytes) {
					const size_t at = total;
					total += (bytes + 255) / 256 * 256;
					return at;
				};
				const size_t r = static_cast<size_t>(r_max);
				bbuf = region(sizeof(float2) * r * s.k * b_points);
				partials = region(sizeof(float4) * r * chunks);
				sums = region(sizeof(double2) * r * chunks);
				counters = region(sizeof(unsigned int) * r);
				if (s.fold_mode) {
					accg = region(sizeof(float) * r * s.m);
					if (s.fold_mode == 2)
						zcg = region(sizeof(float2) * r * s.k * s.m);
				}
			}
		};
	}

	// B points per (row, block) and column chunks per row of a job shape
	void inverse_geometry(ugsdr_ctx* ctx, const BatchedParams& p, int fold_mode, int& cw_blocked, size_t& b_points, int& chunks) {
		cw_blocked = blocked_cw(ctx, p.base.n, p.n1, p.n2, fold_mode);
		if (cw_blocked) {
			const int n2p = (p.n2 + cw_blocked - 1) / cw_blocked * cw_blocked;
			b_points = static_cast<size_t>(p.n1) * n2p;
			chunks = n2p / cw_blocked;
		}
		else {
			b_points = static_cast<size_t>(p.n1) * p.n2;
			chunks = chunks_of(p.n2, p.cw);
		}
	}

	size_t batched_scratch_bytes(ugsdr_ctx* ctx, const JobLaunchShape& s) {
		AcqParams base{};
		base.n = s.n;
		const BatchedParams p = batched_params(ctx, base, s.n);
		int cwb = 0, chunks = 0;
		size_t b_points = 0;
		inverse_geometry(ctx, p, s.fold_mode, cwb, b_points, chunks);
		return ScratchLayout(s, batch_rows(s, b_points), chunks, b_points).total;
	}

	void large_code_spectrum(ugsdr_ctx* ctx, CodeEntry& e, const float* chips_dev, size_t n_chips, size_t repeats,
		uint32_t sign_mask, size_t sign_segment) {
		AcqParams base{};
		base.n = static_cast<int>(e.n);
		base.one_sided = e.spectrum_mode == UGSDR_SPECTRUM_ONE_SIDED;
		BatchedParams p = batched_params(ctx, base, base.n);
		DevBuf mask;
		mask.reserve(sizeof(uint32_t));
		UG_CUDA(cudaMemcpyAsync(mask.ptr, &sign_mask, sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream));
		p.code_mode = 1;
		p.chips = chips_dev;
		p.n_chips = static_cast<int>(n_chips);
		p.chip_stride = static_cast<int>(n_chips);
		p.repeats = static_cast<int>(repeats);
		p.sign_segment = static_cast<int>(sign_segment);
		p.sign_masks = mask.as<uint32_t>();
		p.out = e.spectrum.as<float2>();
		launch_forward(ctx, UGSDR_SAMPLES_CF32, p, 1);
		UG_CUDA(cudaStreamSynchronize(ctx->stream));
	}

	// One forward DFT of a whole device array on the batched four-step kernels
	// (one item; the mixer's zero adder multiplies by table[16] + i table[0] =
	// 1 + 0i exactly): output k1-major, X_T[k1][k2] = X[k1 + N1 k2].
	void dft_four_step(ugsdr_ctx* ctx, const float2* in, float2* out_k1, int n, int& n1, int& n2) {
		if (!ctx->zero_adder.ptr) {
			ctx->zero_adder.reserve(sizeof(uint32_t));
			UG_CUDA(cudaMemsetAsync(ctx->zero_adder.ptr, 0, sizeof(uint32_t), ctx->stream));
		}
		AcqParams base{};
		base.n = n;
		base.k_blocks = 1;
		base.samples = in;
		base.lut = get_lut(ctx);
		base.adders = ctx->zero_adder.as<uint32_t>();
		BatchedParams p = batched_params(ctx, base, n);
		p.out = out_k1;
		launch_forward(ctx, UGSDR_SAMPLES_CF32, p, 1);
		n1 = p.n1;
		n2 = p.n2;
	}

	// One Doppler chunk of nd bins (base.d_base first): forward over nd x K
	// blocks, inverse over the chunk's s.rows = codes x nd rows.
	void large_job(ugsdr_ctx* ctx, const ugsdr_acq_job& job, const AcqParams& base, const JobLaunchShape& s, int nd, char* scratch) {
		BatchedParams p = batched_params(ctx, base, s.n);
		const int items = nd * base.k_blocks;
		p.out = base.spectra;
		int cw_blocked = 0, chunks = 0;
		size_t b_points = 0;
		inverse_geometry(ctx, p, s.fold_mode, cw_blocked, b_points, chunks);
		// the warp-owned row kernels' pruned gather (one-sided spectra) reads
		// only the lower part of each signal-spectrum row: only that is stored
		const int wr = warp_rows_mode(ctx, s.n);
		const bool half = base.one_sided != 0 && !std::getenv("UGSDR_NO_PRUNE");
		if (cw_blocked && wr != 0 && half)
			with_large_ffts(p.n1, p.n2, [&](auto, auto f2) {
				using F2 = decltype(f2);
				if constexpr (F2::kHooked && F2::kRowsCompact)
					p.row_keep = half_row_elems<F2>(p.n1);
			});
		{
			KernelTimer timer(ctx, "acq_forward_large");
			launch_forward(ctx, job.sample_type, p, items);
		}
		p.row_keep = 0;
		if (cw_blocked)
			p.n2p = static_cast<int>(b_points / p.n1);
		const int r_max = batch_rows(s, b_points);
		const ScratchLayout lay(s, r_max, chunks, b_points);
		p.bbuf = reinterpret_cast<float2*>(scratch + lay.bbuf);
		p.partials = reinterpret_cast<float4*>(scratch + lay.partials);
		p.sums = reinterpret_cast<double2*>(scratch + lay.sums);
		p.counters = reinterpret_cast<unsigned int*>(scratch + lay.counters);
		if (s.fold_mode) {
			p.accg = reinterpret_cast<float*>(scratch + lay.accg);
			if (s.fold_mode == 2)
				p.zcg = reinterpret_cast<float2*>(scratch + lay.zcg);
		}
		auto run_batches = [&](auto launch_pair) {
			for (int row0 = 0; row0 < s.rows; row0 += r_max) {
				p.row0 = row0;
				p.rows = std::min(r_max, s.rows - row0);
				UG_CUDA(cudaMemsetAsync(p.counters, 0, sizeof(unsigned int) * p.rows, ctx->stream));
				if (s.fold_mode) {
					UG_CUDA(cudaMemsetAsync(p.accg, 0, sizeof(float) * static_cast<size_t>(p.rows) * s.m, ctx->stream));
					if (s.fold_mode == 2)
						UG_CUDA(cudaMemsetAsync(p.zcg, 0, sizeof(float2) * static_cast<size_t>(p.rows) * s.k * s.m, ctx->stream));
				}
				launch_pair();
				note_launch(ctx, 2);
				if (s.fold_mode) {
					fold_finish_kernel<<<p.rows, kBatchedThreads, 0, ctx->stream>>>(p);
					note_launch(ctx);
				}
			}
		};
		if (cw_blocked) {
			// static row plan + warp-owned columns over the blocked B layout
			with_large_ffts(p.n1, p.n2, [&](auto, auto f2) {
				using F2 = decltype(f2);
				with_cols_warp(p.n1, p.n2, [&](auto plan) {
					using P = decltype(plan);
					constexpr int CW = P::CW;
					// the row plan that pairs with the column plan: N = N1 x N2
					if constexpr (F2::kHooked && ((P::N1 == 400 && F2::N == 500) || (P::N1 == 200 && F2::N == 250))) {
						void (*const cols_kernel)(BatchedParams) = p.base.stat ? inv_cols_warp_kernel<P, 1> : inv_cols_warp_kernel<P, 0>;
						if (wr != 0) {
							// warp-owned rows, four warps per CTA: RPW rows per warp with
							// the code rows staged (mode 1), or three rows per warp with
							// the code rows read through L1 / L2 (mode 2)
							auto launch_rows = [&](auto rows_kernel, int rpw, size_t smem_r) {
								set_smem(rows_kernel, smem_r);
								set_smem(cols_kernel, P::smem_bytes());
								KernelTimer timer(ctx, "acq_inverse_large");
								run_batches([&] {
									rows_kernel<<<p.rows * chunks_of(p.n1, rpw * kRowsWarps), 32 * kRowsWarps, smem_r, ctx->stream>>>(p);
									cols_kernel<<<p.rows * chunks, 32 * P::WARPS, P::smem_bytes(), ctx->stream>>>(p);
								});
							};
							// one-sided code spectra: the gather reads only the rows' lower
							// halves (the rest of Z is zero) and pass 0 runs pruned DFTs
							constexpr int RPW = kRowsPerWarp<F2::N>, W = kRowsWarps;
							if (wr == 2 && half)
								launch_rows(inv_rows_warp_kernel<F2, CW, P::N1, 3, W, false, true>, 3,
									rows_warp_smem<F2, P::N1, 3, W, false, true>());
							else if (wr == 2)
								launch_rows(inv_rows_warp_kernel<F2, CW, P::N1, 3, W, false, false>, 3,
									rows_warp_smem<F2, P::N1, 3, W, false, false>());
							else if (half)
								launch_rows(inv_rows_warp_kernel<F2, CW, P::N1, RPW, W, true, true>, RPW,
									rows_warp_smem<F2, P::N1, RPW, W, true, true>());
							else
								launch_rows(inv_rows_warp_kernel<F2, CW, P::N1, RPW, W, true, false>, RPW,
									rows_warp_smem<F2, P::N1, RPW, W, true, false>());
							return;
						}
						const size_t smem_r = smem_inv_rows<F2>(p);
						set_smem(inv_rows_kernel<F2, CW, P::N1>, smem_r);
						set_smem(cols_kernel, P::smem_bytes());
						const int t_rows = threads_of<F2>(p.p2, p.rw);
						require(t_rows <= F2::kRowsMaxThreads, "row kernel needs more threads than its launch bound");
						KernelTimer timer(ctx, "acq_inverse_large");
						run_batches([&] {
							inv_rows_kernel<F2, CW, P::N1><<<p.rows * chunks_of(p.n1, p.rw), t_rows, smem_r, ctx->stream>>>(p);
							cols_kernel<<<p.rows * chunks, 32 * P::WARPS, P::smem_bytes(), ctx->stream>>>(p);
						});
					}
				});
			});
			return;
		}
		with_large_ffts(p.n1, p.n2, [&](auto f1, auto f2) {
			using F1 = decltype(f1);
			using F2 = decltype(f2);
			const size_t smem_c = smem_inv_cols<F1>(p);
			const size_t smem_r = smem_inv_rows<F2>(p);
			set_smem(inv_rows_kernel<F2>, smem_r);
			set_smem(inv_cols_kernel<F1>, smem_c);
			const int t_rows = threads_of<F2>(p.p2, p.rw), t_cols = threads_of<F1>(p.p1, p.cw);
			require(t_rows <= F2::kRowsMaxThreads, "row kernel needs more threads than its launch bound");
			require(t_cols <= F1::kColsMaxThreads, "column kernel needs more threads than its launch bound");
			KernelTimer timer(ctx, "acq_inverse_large");
			run_batches([&] {
				const int row_items = F2::kHooked ? p.rows : p.rows * s.k;  // hooked: each CTA loops over the K blocks
				inv_rows_kernel<F2><<<row_items * chunks_of(p.n1, p.rw), t_rows, smem_r, ctx->stream>>>(p);
				inv_cols_kernel<F1><<<p.rows * chunks, t_cols, smem_c, ctx->stream>>>(p);
			});
		});
	}

	namespace {
		void build_code_spectrum(ugsdr_ctx* ctx, CodeEntry& e, const float* chips_host, size_t n_chips, size_t repeats,
			uint32_t sign_mask, size_t sign_segment) {
			const int n = static_cast<int>(e.n);
			DevBuf chips;
			chips.reserve(sizeof(float) * n_chips);
			UG_CUDA(cudaMemcpyAsync(chips.ptr, chips_host, sizeof(float) * n_chips, cudaMemcpyHostToDevice, ctx->stream));
			e.spectrum.reserve(sizeof(float2) * n);
			if (!e.large) {
				CodeSpecParams p{};
				p.chips = chips.as<float>();
				p.n_chips = static_cast<int>(n_chips);
				p.repeats = static_cast<int>(repeats);
				p.sign_mask = sign_mask;
				p.sign_segment = static_cast<int>(sign_segment);
				p.one_sided = e.spectrum_mode == UGSDR_SPECTRUM_ONE_SIDED;
				p.out = e.spectrum.as<float2>();
				p.plan = to_dev(get_plan(ctx, n));
				const size_t smem = 2 * sizeof(float2) * n;
				set_smem(code_spectrum_kernel, smem);
				code_spectrum_kernel<<<1, kThreads, smem, ctx->stream>>>(p);
				note_launch(ctx);
			}
			else {
				large_code_spectrum(ctx, e, chips.as<float>(), n_chips, repeats, sign_mask, sign_segment);
				e.n1 = get_large_plan(ctx, n).n1;
			}
			UG_CUDA(cudaStreamSynchronize(ctx->stream));
		}
	}

	// --------------------------------------------------------------- jobs
	struct JobLaunch {
		std::vector<double> grid;
		std::vector<uint32_t> adders;
		int n = 0, k = 0, m = 0, n_codes = 0, fold_mode = 0;
		bool large = false;
		bool front = false;   // device front end (mix at the input rate + resample) first
		ResamplePlan rs{};
	};

	namespace {
		JobLaunchShape shape_of(const JobLaunch& L) {
			JobLaunchShape s;
			s.n = L.n;
			s.k = L.k;
			s.m = L.m;
			s.rows = static_cast<int>(L.grid.size()) * L.n_codes;
			s.fold_mode = L.fold_mode;
			return s;
		}

		JobLaunch validate(ugsdr_ctx* ctx, const ugsdr_acq_job& job) {
			JobLaunch L;
			require(job.samples != nullptr, "null samples");
			require(job.sample_type >= 0 && job.sample_type <= UGSDR_SAMPLES_NT1065_4, "unknown sample type");
			require(job.block_samples >= 2 && job.block_samples <= (1u << 24), "block size out of range");
			require(job.n_blocks >= 1, "n_blocks must be >= 1");
			require(job.sampling_rate > 0, "sampling rate must be positive");
			L.front = job.input_sampling_rate != 0.0 && job.input_sampling_rate != job.sampling_rate;
			if (!L.front && is_packed(job.sample_type)) {
				// packed captures are decoded by the front end, at the same rate
				L.front = true;
				L.rs = ResamplePlan{1, 1, job.n_samples, job.n_samples};
				require(job.n_samples >= job.block_samples * job.n_blocks, "not enough samples for n_blocks blocks");
			}
			else if (L.front) {
				const double fi = job.input_sampling_rate, fo = job.sampling_rate;
				require(fi > 0 && fi == std::floor(fi) && fo == std::floor(fo) && fi < 1e15 && fo < 1e15,
					"resampling needs positive integer rates in Hz");
				const uint64_t in = static_cast<uint64_t>(fi), out = static_cast<uint64_t>(fo);
				const uint64_t g = std::gcd(in, out);
				const unsigned __int128 lcm = static_cast<unsigned __int128>(in / g) * out;
				const uint64_t l = static_cast<uint64_t>(lcm / in), m = static_cast<uint64_t>(lcm / out);
				require(m <= 65536 && l <= (1u << 20), "resampling ratio too large (lcm / rate above 65536)");
				require(job.n_samples >= 1 && job.n_samples < (static_cast<size_t>(1) << 40), "input length out of range");
				L.rs.l = l;
				L.rs.m = m;
				L.rs.up = l * job.n_samples;
				L.rs.n_out = m == 1 ? L.rs.up : (L.rs.up + m - 1) / m;
				require(L.rs.n_out >= job.block_samples * job.n_blocks, "not enough resampled samples for n_blocks blocks");
			}
			else {
				require(job.n_samples >= job.block_samples * job.n_blocks, "not enough samples for n_blocks blocks");
			}
			require(job.codes != nullptr && job.n_codes >= 1, "no codes");
			require(job.statistic == UGSDR_STAT_ABS || job.statistic == UGSDR_STAT_ABS2, "unknown statistic");
			L.n = static_cast<int>(job.block_samples);
			L.k = static_cast<int>(job.n_blocks);
			L.n_codes = job.n_codes;
			if (job.fold_samples) {
				// ReshapeAndSum::CheckBlockSize (reshape_and_sum.hpp:15-18)
				require(job.block_samples % job.fold_samples == 0, "Signal size is not divided by block size");
				L.m = static_cast<int>(job.fold_samples);
				L.fold_mode = job.fold_coherent ? 1 : 2;
			}
			else {
				L.m = L.n;
				L.fold_mode = 0;
			}
			L.grid = doppler_grid(job.doppler_range, job.doppler_step);
			for (double d : L.grid)
				L.adders.push_back(nco_adder(job.sampling_rate, -d));  // Translate(signal, fs, -doppler)
			for (int c = 0; c < job.n_codes; ++c) {
				auto it = ctx->codes.find(job.codes[c]);
				require(it != ctx->codes.end(), "unknown code handle " + std::to_string(job.codes[c]), UGSDR_E_NOT_FOUND);
				require(it->second->n == job.block_samples, "code length differs from block_samples");
				require(it->second->spectrum_mode == job.spectrum_mode, "code spectrum mode differs from the job's");
			}
			if (is_packed(job.sample_type))
				require(capture_bytes(job.sample_type, job.input_sampling_rate != 0.0 ? job.input_sampling_rate : job.sampling_rate,
					job.n_samples) > 0, "BBP DDC captures need a whole-kHz rate and whole 1 ms epochs");
			L.large = !fits_single_cta(ctx, L.n);
			return L;
		}

		// bytes of the job's capture (packed formats: with their framing)
		size_t job_bytes(const ugsdr_acq_job& job) {
			return capture_bytes(job.sample_type, job.input_sampling_rate != 0.0 ? job.input_sampling_rate : job.sampling_rate,
				job.n_samples);
		}
	}

	// Doppler bins per launch: mixed spectra (bins x K x N complex) within 4 GB
	// (UGSDR_SPECTRA_BUDGET_MB overrides, e.g. to exercise chunking in tests).
	int chunk_bins(const JobLaunch& L) {
		const size_t per_bin = sizeof(float2) * static_cast<size_t>(L.n) * L.k;
		size_t budget = static_cast<size_t>(4) << 30;
		if (const char* env = std::getenv("UGSDR_SPECTRA_BUDGET_MB"))
			budget = std::max<size_t>(1, std::strtoull(env, nullptr, 10)) << 20;
		return static_cast<int>(std::max<size_t>(1, std::min<size_t>(L.grid.size(), budget / per_bin)));
	}

	void launch_chunk(ugsdr_ctx* ctx, const ugsdr_acq_job& job, const JobLaunch& L, AcqParams& p, int nd, char* scratch);

	// Launches one job on ctx->stream; cells stay on the device.
	void launch_job(ugsdr_ctx* ctx, const ugsdr_acq_job& job, const JobLaunch& L, const void* dev_samples,
		AcqCellDev* cells, int* best_bin, uint32_t* adders_dev, const float2** code_ptrs_dev, float2* spectra,
		char* scratch) {
		AcqParams p{};
		p.samples = dev_samples;
		p.n = L.n;
		p.k_blocks = L.k;
		p.n_doppler = static_cast<int>(L.grid.size());
		p.n_codes = L.n_codes;
		p.m = L.m;
		p.fold_mode = L.fold_mode;
		p.stat = job.statistic;
		p.one_sided = job.spectrum_mode == UGSDR_SPECTRUM_ONE_SIDED;
		p.adders = adders_dev;
		p.phase0 = 0;
		// const Translate (mixer.hpp:44-51) has no zero-frequency shortcut, but a
		// zero adder multiplies by table[16] + i table[0] = 1 + 0i: skipping is equal
		p.fe_on = job.frontend_frequency != 0.0;
		p.fe_adder = p.fe_on ? nco_adder(job.sampling_rate, job.frontend_frequency) : 0u;
		p.lut = get_lut(ctx);
		p.spectra = spectra;
		p.codes = code_ptrs_dev;
		p.cells = cells;
		// the Doppler grid runs in chunks whose spectra fit the spectra budget
		const int n_bins = static_cast<int>(L.grid.size());
		const int chunk = chunk_bins(L);
		for (int d0 = 0; d0 < n_bins; d0 += chunk) {
			p.d_base = d0;
			launch_chunk(ctx, job, L, p, std::min(chunk, n_bins - d0), scratch);
		}
		(void)best_bin;
	}

	namespace {
		// single-CTA block sizes with a compile-time plan (4000: 1 ms at 4 MHz)
		template <class Fn>
		bool with_small_fft(int n, Fn&& fn) {
			if (n == 4000) {
				fn(StaticFft<4000, 25, 10, 16>{});
				return true;
			}
			return false;
		}

		template <class F>
		void launch_small_static(ugsdr_ctx* ctx, const ugsdr_acq_job& job, const AcqParams& p, int nd, int k, int n_codes) {
			const size_t smem_f = 3 * sizeof(float2) * F::N + 16;
			const int grid_f = nd * k;
			{
				KernelTimer timer(ctx, "acq_forward");
				switch (job.sample_type) {
				case UGSDR_SAMPLES_CF32:
					set_smem(acq_forward_static_kernel<UGSDR_SAMPLES_CF32, F>, smem_f);
					acq_forward_static_kernel<UGSDR_SAMPLES_CF32, F><<<grid_f, kThreads, smem_f, ctx->stream>>>(p);
					break;
				case UGSDR_SAMPLES_CI8:
					set_smem(acq_forward_static_kernel<UGSDR_SAMPLES_CI8, F>, smem_f);
					acq_forward_static_kernel<UGSDR_SAMPLES_CI8, F><<<grid_f, kThreads, smem_f, ctx->stream>>>(p);
					break;
				case UGSDR_SAMPLES_CI16:
					set_smem(acq_forward_static_kernel<UGSDR_SAMPLES_CI16, F>, smem_f);
					acq_forward_static_kernel<UGSDR_SAMPLES_CI16, F><<<grid_f, kThreads, smem_f, ctx->stream>>>(p);
					break;
				default:
					set_smem(acq_forward_static_kernel<UGSDR_SAMPLES_RI8, F>, smem_f);
					acq_forward_static_kernel<UGSDR_SAMPLES_RI8, F><<<grid_f, kThreads, smem_f, ctx->stream>>>(p);
					break;
				}
			}
			note_launch(ctx);
			// a, b, the N-float accumulator, the pass tables (N entries)
			const size_t smem_i = 2 * sizeof(float2) * F::N + sizeof(float) * F::N + sizeof(float2) * F::N + 16;
			KernelTimer timer(ctx, "acq_inverse");
			auto inverse = [&](auto kernel) {
				set_smem(kernel, smem_i);
				kernel<<<nd * n_codes, kThreads, smem_i, ctx->stream>>>(p);
			};
			// one-sided spectra: pass 0 reads only the lower half of Z
			if (p.one_sided && !std::getenv("UGSDR_NO_PRUNE"))
				inverse(acq_inverse_static_kernel<F, true>);
			else
				inverse(acq_inverse_static_kernel<F>);
			note_launch(ctx);
		}
	}

	void launch_chunk(ugsdr_ctx* ctx, const ugsdr_acq_job& job, const JobLaunch& L, AcqParams& p, int nd, char* scratch) {
		if (!L.large && L.fold_mode == 0 && L.m == L.n && L.n == 4000) {
			p.plan = to_dev(get_plan(ctx, L.n));
			with_small_fft(L.n, [&](auto f) { launch_small_static<decltype(f)>(ctx, job, p, nd, L.k, L.n_codes); });
			return;
		}
		if (!L.large) {
			p.plan = to_dev(get_plan(ctx, L.n));
			const size_t smem_f = 2 * sizeof(float2) * L.n;
			const int grid_f = nd * L.k;
			{
			KernelTimer timer(ctx, "acq_forward");
			switch (job.sample_type) {
			case UGSDR_SAMPLES_CF32:
				set_smem(acq_forward_kernel<UGSDR_SAMPLES_CF32>, smem_f);
				acq_forward_kernel<UGSDR_SAMPLES_CF32><<<grid_f, kThreads, smem_f, ctx->stream>>>(p);
				break;
			case UGSDR_SAMPLES_CI8:
				set_smem(acq_forward_kernel<UGSDR_SAMPLES_CI8>, smem_f);
				acq_forward_kernel<UGSDR_SAMPLES_CI8><<<grid_f, kThreads, smem_f, ctx->stream>>>(p);
				break;
			case UGSDR_SAMPLES_CI16:
				set_smem(acq_forward_kernel<UGSDR_SAMPLES_CI16>, smem_f);
				acq_forward_kernel<UGSDR_SAMPLES_CI16><<<grid_f, kThreads, smem_f, ctx->stream>>>(p);
				break;
			default:
				set_smem(acq_forward_kernel<UGSDR_SAMPLES_RI8>, smem_f);
				acq_forward_kernel<UGSDR_SAMPLES_RI8><<<grid_f, kThreads, smem_f, ctx->stream>>>(p);
				break;
			}
			}
			note_launch(ctx);
			const size_t smem_i = 2 * sizeof(float2) * L.n + sizeof(float) * L.m;
			set_smem(acq_inverse_kernel, smem_i);
			KernelTimer timer(ctx, "acq_inverse");
			acq_inverse_kernel<<<nd * L.n_codes, kThreads, smem_i, ctx->stream>>>(p);
			note_launch(ctx);
		}
		else {
			JobLaunchShape s = shape_of(L);
			s.rows = nd * L.n_codes;
			large_job(ctx, job, p, s, nd, scratch);
		}
	}

	// Mixes at the input rate and resamples the first n*K outputs into `out`.
	void launch_front_end(ugsdr_ctx* ctx, const ugsdr_acq_job& job, const JobLaunch& L, const void* samples, float2* out) {
		FrontEndParams f{};
		f.samples = samples;
		f.n_in = job.n_samples;
		const double fs_in = job.input_sampling_rate != 0.0 ? job.input_sampling_rate : job.sampling_rate;
		f.layout.spm = static_cast<uint32_t>(fs_in / 1e3);
		f.layout.epoch_bytes = static_cast<uint32_t>(bbp_epoch_bytes(fs_in));
		f.rs = L.rs;
		f.fe_on = job.frontend_frequency != 0.0;
		f.fe_adder = f.fe_on ? nco_adder(fs_in, job.frontend_frequency) : 0u;
		f.lut = get_lut(ctx);
		f.out = out;
		f.n = static_cast<uint64_t>(L.n) * L.k;
		const int blocks = static_cast<int>(std::min<uint64_t>((f.n + 255) / 256, static_cast<uint64_t>(ctx->sm_count) * 8));
		KernelTimer timer(ctx, "front_end");
		switch (job.sample_type) {
		case UGSDR_SAMPLES_CF32: front_end_kernel<UGSDR_SAMPLES_CF32><<<blocks, 256, 0, ctx->stream>>>(f); break;
		case UGSDR_SAMPLES_CI8: front_end_kernel<UGSDR_SAMPLES_CI8><<<blocks, 256, 0, ctx->stream>>>(f); break;
		case UGSDR_SAMPLES_CI16: front_end_kernel<UGSDR_SAMPLES_CI16><<<blocks, 256, 0, ctx->stream>>>(f); break;
		case UGSDR_SAMPLES_RI8: front_end_kernel<UGSDR_SAMPLES_RI8><<<blocks, 256, 0, ctx->stream>>>(f); break;
		case UGSDR_SAMPLES_BBP_DDC: front_end_kernel<UGSDR_SAMPLES_BBP_DDC><<<blocks, 256, 0, ctx->stream>>>(f); break;
		case UGSDR_SAMPLES_NT1065_1: front_end_kernel<UGSDR_SAMPLES_NT1065_1><<<blocks, 256, 0, ctx->stream>>>(f); break;
		case UGSDR_SAMPLES_NT1065_2: front_end_kernel<UGSDR_SAMPLES_NT1065_2><<<blocks, 256, 0, ctx->stream>>>(f); break;
		case UGSDR_SAMPLES_NT1065_3: front_end_kernel<UGSDR_SAMPLES_NT1065_3><<<blocks, 256, 0, ctx->stream>>>(f); break;
		default: front_end_kernel<UGSDR_SAMPLES_NT1065_4><<<blocks, 256, 0, ctx->stream>>>(f); break;
		}
		note_launch(ctx);
	}

	size_t spectra_bytes(const JobLaunch& L) {
		return sizeof(float2) * static_cast<size_t>(L.n) * L.k * chunk_bins(L);
	}

	namespace {
		struct BatchSizes {
			std::vector<JobLaunch> launches;
			size_t samples = 0, spectra = 0, cells = 0, params = 0, slab = 0, front = 0;
		};

		size_t front_bytes(const JobLaunch& L) {
			return L.front ? (sizeof(float2) * static_cast<size_t>(L.n) * L.k + 255) / 256 * 256 : 0;
		}

		BatchSizes size_batch(ugsdr_ctx* ctx, const ugsdr_acq_job* jobs, int n_jobs) {
			require(jobs != nullptr && n_jobs >= 1, "no jobs");
			BatchSizes s;
			std::map<std::pair<const void*, size_t>, bool> seen;
			for (int j = 0; j < n_jobs; ++j) {
				s.launches.push_back(validate(ctx, jobs[j]));
				const auto& L = s.launches.back();
				if (!jobs[j].samples_on_device) {
					const size_t bytes = job_bytes(jobs[j]);
					if (!seen[{jobs[j].samples, bytes}])
						s.samples += (bytes + 255) / 256 * 256;
					seen[{jobs[j].samples, bytes}] = true;
				}
				s.spectra = std::max(s.spectra, spectra_bytes(L));
				s.cells += static_cast<size_t>(L.n_codes) * L.grid.size();
				s.front += front_bytes(L);
				s.params += (L.grid.size() * sizeof(uint32_t) + L.n_codes * sizeof(void*) + L.n_codes * sizeof(int) + 512) / 256 * 256;
				if (L.large)
					s.slab = std::max(s.slab, batched_scratch_bytes(ctx, shape_of(L)));
			}
			s.samples = std::max<size_t>(s.samples, 256);
			return s;
		}

		struct StreamSwap {  // route the launch helpers (which use ctx->stream) to `stream`
			ugsdr_ctx* ctx;
			cudaStream_t saved;
			StreamSwap(ugsdr_ctx* c, cudaStream_t s) : ctx(c), saved(c->stream) { c->stream = s; }
			~StreamSwap() { ctx->stream = saved; }
		};
	}

	size_t jobs_device_bytes(ugsdr_ctx* ctx, const ugsdr_acq_job* jobs, int n_jobs) {
		const BatchSizes s = size_batch(ctx, jobs, n_jobs);
		return s.samples + s.spectra + sizeof(AcqCellDev) * s.cells + s.params + s.slab + s.front;
	}

	EnqueuedBatch enqueue_jobs(ugsdr_ctx* ctx, Workspace& ws, cudaStream_t stream, const ugsdr_acq_job* jobs, int n_jobs,
		void* host_cells) {
		BatchSizes sizes = size_batch(ctx, jobs, n_jobs);
		const std::vector<JobLaunch>& launches = sizes.launches;
		const size_t params_b = sizes.params;
		ws.samples.reserve(sizes.samples);
		ws.spectra.reserve(sizes.spectra);
		ws.cells.reserve(sizeof(AcqCellDev) * sizes.cells);
		ws.params.reserve(params_b);
		if (sizes.slab)
			ws.slab.reserve(sizes.slab);
		if (sizes.front)
			ws.front.reserve(sizes.front);
		StreamSwap swap(ctx, stream);

		// stage parameters and host samples
		std::vector<char> host_params(params_b);
		size_t s_off = 0, p_off = 0, c_off = 0;
		std::vector<const void*> dev_samples(n_jobs);
		std::map<std::pair<const void*, size_t>, const void*> staged;  // one upload per host buffer
		std::vector<size_t> p_offsets(n_jobs), c_offsets(n_jobs);
		for (int j = 0; j < n_jobs; ++j) {
			const auto& job = jobs[j];
			const auto& L = launches[j];
			if (job.samples_on_device) {
				dev_samples[j] = job.samples;
			}
			else {
				const size_t bytes = job_bytes(job);
				auto key = std::make_pair(job.samples, bytes);
				auto it = staged.find(key);
				if (it != staged.end()) {
					dev_samples[j] = it->second;
				}
				else {
					char* dst = ws.samples.as<char>() + s_off;
					UG_CUDA(cudaMemcpyAsync(dst, job.samples, bytes, cudaMemcpyHostToDevice, ctx->stream));
					dev_samples[j] = dst;
					staged[key] = dst;
					s_off += (bytes + 255) / 256 * 256;
				}
			}
			p_offsets[j] = p_off;
			char* hp = host_params.data() + p_off;
			std::memcpy(hp, L.adders.data(), L.adders.size() * sizeof(uint32_t));
			size_t o = (L.adders.size() * sizeof(uint32_t) + 15) / 16 * 16;
			for (int c = 0; c < L.n_codes; ++c) {
				const float2* ptr = ctx->codes[job.codes[c]]->spectrum.as<float2>();
				std::memcpy(hp + o + c * sizeof(void*), &ptr, sizeof(void*));
			}
			o += L.n_codes * sizeof(void*);
			o = (o + 15) / 16 * 16;
			p_off += (L.grid.size() * sizeof(uint32_t) + L.n_codes * sizeof(void*) + L.n_codes * sizeof(int) + 512) / 256 * 256;
			c_offsets[j] = c_off;
			c_off += static_cast<size_t>(L.n_codes) * L.grid.size();
		}
		UG_CUDA(cudaMemcpyAsync(ws.params.ptr, host_params.data(), params_b, cudaMemcpyHostToDevice, ctx->stream));

		size_t f_off = 0;
		for (int j = 0; j < n_jobs; ++j) {
			const auto& L = launches[j];
			ugsdr_acq_job job = jobs[j];
			const void* samples = dev_samples[j];
			if (L.front) {
				// the search then reads complex float at sampling_rate, front end done
				float2* out = reinterpret_cast<float2*>(ws.front.as<char>() + f_off);
				f_off += front_bytes(L);
				launch_front_end(ctx, job, L, samples, out);
				samples = out;
				job.sample_type = UGSDR_SAMPLES_CF32;
				job.frontend_frequency = 0.0;
			}
			char* dp = ws.params.as<char>() + p_offsets[j];
			auto* adders = reinterpret_cast<uint32_t*>(dp);
			size_t o = (L.adders.size() * sizeof(uint32_t) + 15) / 16 * 16;
			auto* code_ptrs = reinterpret_cast<const float2**>(dp + o);
			o += L.n_codes * sizeof(void*);
			o = (o + 15) / 16 * 16;
			auto* best = reinterpret_cast<int*>(dp + o);
			launch_job(ctx, job, L, samples, ws.cells.as<AcqCellDev>() + c_offsets[j], best, adders,
				code_ptrs, ws.spectra.as<float2>(), ws.slab.as<char>());
		}
		UG_CUDA(cudaMemcpyAsync(host_cells, ws.cells.ptr, sizeof(AcqCellDev) * c_off, cudaMemcpyDeviceToHost, ctx->stream));
		EnqueuedBatch b;
		for (const auto& L : launches)
			b.grids.push_back(L.grid);
		b.cell_offsets = c_offsets;
		b.n_cells = c_off;
		return b;
	}

	void finish_jobs(const EnqueuedBatch& b, const ugsdr_acq_job* jobs, int n_jobs, const void* host_cells,
		ugsdr_acq_result* const* results, ugsdr_acq_cell* cells_out) {
		const auto* cells = static_cast<const AcqCellDev*>(host_cells);
		for (int j = 0; j < n_jobs; ++j) {
			const auto& job = jobs[j];
			const auto& grid = b.grids[j];
			const size_t nd = grid.size();
			for (int c = 0; c < job.n_codes; ++c) {
				const AcqCellDev* row = cells + b.cell_offsets[j] + static_cast<size_t>(c) * nd;
				// first strictly greater level wins (fse.hpp:265), recomputed on the host
				size_t bd = 0;
				for (size_t d = 1; d < nd; ++d)
					if (row[bd].level < row[d].level)
						bd = d;
				ugsdr_acq_result& r = results[j][c];
				r.code = job.codes[c];
				r.doppler_bin = static_cast<int>(bd);
				r.index = row[bd].index;
				r.n_doppler = static_cast<uint32_t>(nd);
				r.doppler = grid[bd] + job.intermediate_frequency;
				r.code_offset = job.code_offset_ratio * static_cast<double>(row[bd].index);
				r.level = row[bd].level;
				r.mean = row[bd].mean;
				r.std = row[bd].std;
				r.sigma = static_cast<double>(row[bd].std + row[bd].mean);
				r.snr = r.level / r.sigma;
			}
		}
		if (cells_out && n_jobs == 1)
			std::memcpy(cells_out, cells, sizeof(AcqCellDev) * b.n_cells);
	}

	void run_jobs(ugsdr_ctx* ctx, const ugsdr_acq_job* jobs, int n_jobs, ugsdr_acq_result* const* results,
		ugsdr_acq_cell* cells_out) {
		// cells land in host memory; pageable is fine here since the call waits
		size_t n_cells = 0;
		{
			const BatchSizes s = size_batch(ctx, jobs, n_jobs);
			n_cells = s.cells;
		}
		std::vector<AcqCellDev> cells(std::max<size_t>(n_cells, 1));
		const EnqueuedBatch b = enqueue_jobs(ctx, ctx->ws, ctx->stream, jobs, n_jobs, cells.data());
		UG_CUDA(cudaStreamSynchronize(ctx->stream));
		finish_jobs(b, jobs, n_jobs, cells.data(), results, cells_out);
	}

	// ------------------------------------------------------------ tile tuning
	namespace {
		// complex points (rows x K x N) of one tuning search, 0.1 - 0.2 s on the
		// device: many full inverse batches, so that a shape that only wins on
		// a short search's tail does not get picked (a 4e9-point cut of the
		// 204,600-point L5 search picked 2-column tiles that ran its full
		// search 3.5 % slower than the rule)
		constexpr double kTunePoints = 1.6e10;
		// a tuned shape replaces the rule only when it is this much faster
		constexpr double kTuneMargin = 0.97;

		ugsdr_tile_shape effective_shape(ugsdr_ctx* ctx, int n) {
			const LargePlan& lp = get_large_plan(ctx, n);
			ugsdr_tile_shape t{};
			tile_shape(ctx, lp, t.cols, t.rows);
			t.n1 = lp.n1;
			t.warp_cols = blocked_cw(ctx, n, lp.n1, lp.n2, 0) ? 1 : 0;
			// the warp-owned row kernel runs with the warp-owned columns of the
			// 200 x 250 and 400 x 500 splits
			t.warp_rows = t.warp_cols ? warp_rows_mode(ctx, n) : 0;
			t.block_samples = n;
			return t;
		}

		// every kernel of the block size's current shape within its shared
		// memory and launch bounds (checked on the host, before any launch)
		void check_shape(ugsdr_ctx* ctx, int n) {
			AcqParams base{};
			base.n = n;
			const BatchedParams p = batched_params(ctx, base, n);
			with_large_ffts(p.n1, p.n2, [&](auto f1, auto f2) {
				using F1 = decltype(f1);
				using F2 = decltype(f2);
				const size_t cap = ctx->smem_optin;
				require(smem_cols(p) <= cap && smem_rows(p, false) <= cap && smem_inv_cols<F1>(p) <= cap &&
					smem_inv_rows<F2>(p) <= cap, "tile shape exceeds shared memory", UGSDR_E_UNSUPPORTED);
				require(threads_of<F1>(p.p1, p.cw) <= F1::kColsMaxThreads && threads_of<F2>(p.p2, p.rw) <= F2::kRowsMaxThreads,
					"tile shape exceeds a kernel's launch bound", UGSDR_E_UNSUPPORTED);
			});
		}

		// rebuilds the cached code spectra of block size n whose four-step
		// layout an earlier split built
		void refresh_codes(ugsdr_ctx* ctx, int n) {
			const int n1 = get_large_plan(ctx, n).n1;
			bool synced = false;
			for (auto& kv : ctx->codes) {
				CodeEntry& e = *kv.second;
				if (!e.large || static_cast<int>(e.n) != n || e.n1 == n1)
					continue;
				if (!synced) {
					UG_CUDA(cudaStreamSynchronize(ctx->stream));  // no search reads the old layout any more
					synced = true;
				}
				build_code_spectrum(ctx, e, e.chips.data(), e.chips.size(), e.repeats, e.sign_mask, e.sign_segment);
			}
		}

		// Sets block size n's shape; an unusable shape leaves the old one.
		void apply_tiles(ugsdr_ctx* ctx, int n, const TileChoice& t) {
			require(!fits_single_cta(ctx, n), "block size runs on the single-CTA path (no four-step tiles)", UGSDR_E_INVALID);
			auto pow2 = [](int v) { return v == 0 || v == 1 || v == 2 || v == 4 || v == 8; };
			require(pow2(t.cw) && pow2(t.rw) && t.warp_cols >= -1 && t.warp_cols <= 1 && t.warp_rows >= -1 && t.warp_rows <= 2,
				"tile shape out of range");
			require(t.n1 == 0 || split_fits(ctx, n, t.n1, 1), "no four-step split " + std::to_string(t.n1) + " for FFT size " +
				std::to_string(n), UGSDR_E_UNSUPPORTED);
			const auto it = ctx->tiles.find(n);
			const TileChoice old = it != ctx->tiles.end() ? it->second : TileChoice{};
			ctx->tiles[n] = t;
			ctx->large_plans.erase(n);
			try {
				check_shape(ctx, n);
			}
			catch (...) {
				ctx->tiles[n] = old;
				ctx->large_plans.erase(n);
				throw;
			}
			refresh_codes(ctx, n);
		}

		struct EventPair {
			cudaEvent_t a = nullptr, b = nullptr;
			EventPair() {
				UG_CUDA(cudaEventCreate(&a));
				UG_CUDA(cudaEventCreate(&b));
			}
			~EventPair() {
				cudaEventDestroy(a);
				cudaEventDestroy(b);
			}
		};

		// best of `reps` device times (ms) of the jobs as one batch, after one
		// untimed run (plans, kernel attributes, scratch growth)
		double time_jobs(ugsdr_ctx* ctx, const std::vector<ugsdr_acq_job>& jobs, int reps) {
			std::vector<std::vector<ugsdr_acq_result>> res(jobs.size());
			std::vector<ugsdr_acq_result*> ptrs(jobs.size());
			for (size_t j = 0; j < jobs.size(); ++j) {
				res[j].resize(jobs[j].n_codes);
				ptrs[j] = res[j].data();
			}
			const int n_jobs = static_cast<int>(jobs.size());
			run_jobs(ctx, jobs.data(), n_jobs, ptrs.data(), nullptr);
			EventPair ev;
			double best = 1e300;
			for (int r = 0; r < reps; ++r) {
				UG_CUDA(cudaEventRecord(ev.a, ctx->stream));
				run_jobs(ctx, jobs.data(), n_jobs, ptrs.data(), nullptr);
				UG_CUDA(cudaEventRecord(ev.b, ctx->stream));
				UG_CUDA(cudaEventSynchronize(ev.b));
				float ms = 0.f;
				UG_CUDA(cudaEventElapsedTime(&ms, ev.a, ev.b));
				best = std::min(best, static_cast<double>(ms));
			}
			return best;
		}

		// splits tried besides the rule's: the next smaller divisor that fits
		// and the rule's split transposed (N1 above sqrt N)
		std::vector<int> other_splits(ugsdr_ctx* ctx, int n, int rule) {
			std::vector<int> out;
			for (int a = rule - 1; a >= 2; --a)
				if (split_fits(ctx, n, a, 4)) {
					out.push_back(a);
					break;
				}
			if (n / rule != rule && split_fits(ctx, n, n / rule, 4))
				out.push_back(n / rule);
			return out;
		}

		// The jobs of block size n with their Doppler grids cut so that one
		// search is about kTunePoints points.
		std::vector<ugsdr_acq_job> tuning_jobs(std::vector<ugsdr_acq_job> js, int n) {
			double pts = 0;
			for (const auto& j : js)
				pts += static_cast<double>(j.n_codes) * doppler_grid(j.doppler_range, j.doppler_step).size() * j.n_blocks * n;
			if (pts <= kTunePoints)
				return js;
			const double scale = kTunePoints / pts;
			for (auto& j : js) {
				const double nd = static_cast<double>(doppler_grid(j.doppler_range, j.doppler_step).size());
				const int half = static_cast<int>(std::max(0.0, (nd * scale - 1.0) / 2.0));
				j.doppler_range = half * j.doppler_step;
			}
			return js;
		}
	}

	// Times the candidate shapes of each large block size among `jobs` on those
	// jobs (Doppler grids cut to ~kTunePoints points) and keeps the fastest:
	// the split first, then the column kernel and its tile width, then the
	// row kernel (warp-owned or CTA tiles) and the rows per row CTA, each
	// stage from the best so far.
	void autotune(ugsdr_ctx* ctx, const ugsdr_acq_job* jobs, int n_jobs, std::vector<ugsdr_tile_shape>& tried) {
		require(jobs != nullptr && n_jobs >= 1, "no jobs");
		std::map<int, std::vector<ugsdr_acq_job>> by_size;
		for (int j = 0; j < n_jobs; ++j) {
			const JobLaunch L = validate(ctx, jobs[j]);
			if (L.large)
				by_size[L.n].push_back(jobs[j]);
		}
		for (const auto& [n, all] : by_size) {
			const std::vector<ugsdr_acq_job> js = tuning_jobs(all, n);
			std::map<std::tuple<int, int, int, int, int>, double> seen;
			auto measure = [&](const TileChoice& t) {
				try {
					apply_tiles(ctx, n, t);
				}
				catch (const Error&) {
					return 1e300;  // outside the kernels' limits: never launched
				}
				ugsdr_tile_shape eff = effective_shape(ctx, n);
				const auto key = std::make_tuple(eff.n1, eff.cols, eff.rows, eff.warp_cols, eff.warp_rows);
				const auto hit = seen.find(key);
				if (hit != seen.end())
					return hit->second;
				eff.ms = time_jobs(ctx, js, 2);
				seen[key] = eff.ms;
				tried.push_back(eff);
				return eff.ms;
			};
			const TileChoice rule{};
			const double rule_ms = measure(rule);
			TileChoice best = rule;
			double best_ms = rule_ms;
			auto consider = [&](const TileChoice& t) {
				const double ms = measure(t);
				if (ms < best_ms) {
					best = t;
					best_ms = ms;
				}
			};
			for (const int a : other_splits(ctx, n, effective_shape(ctx, n).n1)) {
				TileChoice t = rule;
				t.n1 = a;
				consider(t);
			}
			const TileChoice split = best;
			for (const int wc : {1, 0})
				for (const int cw : {8, 4, 2}) {
					TileChoice t = split;
					t.warp_cols = wc;
					t.cw = cw;
					consider(t);
				}
			const TileChoice cols = best;
			for (const int wr : {1, 2, 0})
				for (const int rw : {8, 4, 2}) {
					TileChoice t = cols;
					t.warp_rows = wr;
					t.rw = rw;
					consider(t);
				}
			apply_tiles(ctx, n, best_ms < kTuneMargin * rule_ms ? best : rule);
		}
	}
}

using namespace ugsdr_gpu;

extern "C" {

int ugsdr_code_put(ugsdr_ctx* ctx, const float* chips, size_t n_chips, size_t repeats, size_t samples,
	uint32_t sign_mask, size_t sign_segment, int spectrum_mode, int* handle) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		require(chips && handle && n_chips > 0 && repeats > 0, "null chips/handle or empty code");
		require(samples >= 2 && samples <= (1u << 24), "code samples out of range");
		require(spectrum_mode == UGSDR_SPECTRUM_ONE_SIDED || spectrum_mode == UGSDR_SPECTRUM_TWO_SIDED, "bad spectrum mode");
		auto e = std::make_unique<CodeEntry>();
		e->n = samples;
		e->spectrum_mode = spectrum_mode;
		e->large = !fits_single_cta(ctx, static_cast<int>(samples));
		build_code_spectrum(ctx, *e, chips, n_chips, repeats, sign_mask, sign_segment);
		e->chips.assign(chips, chips + n_chips);
		e->repeats = repeats;
		e->sign_mask = sign_mask;
		e->sign_segment = sign_segment;
		const int h = ctx->next_code++;
		ctx->codes[h] = std::move(e);
		*handle = h;
	});
}

int ugsdr_code_release(ugsdr_ctx* ctx, int handle) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		auto it = ctx->codes.find(handle);
		require(it != ctx->codes.end(), "unknown code handle", UGSDR_E_NOT_FOUND);
		UG_CUDA(cudaStreamSynchronize(ctx->stream));
		ctx->codes.erase(it);
	});
}

int ugsdr_acquire(ugsdr_ctx* ctx, const ugsdr_acq_job* job, ugsdr_acq_result* results, ugsdr_acq_cell* cells) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		require(job && results, "null job/results");
		ugsdr_acq_result* const rs[1] = {results};
		run_jobs(ctx, job, 1, rs, cells);
	});
}

int ugsdr_acquire_batch(ugsdr_ctx* ctx, const ugsdr_acq_job* jobs, int n_jobs, ugsdr_acq_result* const* results) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		require(results != nullptr, "null results");
		run_jobs(ctx, jobs, n_jobs, results, nullptr);
	});
}
int ugsdr_tile_get(ugsdr_ctx* ctx, size_t block_samples, ugsdr_tile_shape* shape) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		require(shape != nullptr, "null shape");
		require(block_samples >= 2 && block_samples <= (1u << 24), "block size out of range");
		const int n = static_cast<int>(block_samples);
		require(!fits_single_cta(ctx, n), "block size runs on the single-CTA path (no four-step tiles)", UGSDR_E_INVALID);
		*shape = effective_shape(ctx, n);
	});
}

int ugsdr_tile_set(ugsdr_ctx* ctx, size_t block_samples, const ugsdr_tile_shape* shape) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		require(block_samples >= 2 && block_samples <= (1u << 24), "block size out of range");
		TileChoice t{};
		if (shape) {
			t.n1 = shape->n1;
			t.cw = shape->cols;
			t.rw = shape->rows;
			t.warp_cols = shape->warp_cols;
			t.warp_rows = shape->warp_rows;
		}
		apply_tiles(ctx, static_cast<int>(block_samples), t);
	});
}

int ugsdr_autotune(ugsdr_ctx* ctx, const ugsdr_acq_job* jobs, int n_jobs, ugsdr_tile_shape* tried, int max_tried, int* n_tried) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::lock_guard<std::mutex> lock(ctx->mutex);
	return guarded(ctx, [&] {
		require(max_tried >= 0 && (tried != nullptr || max_tried == 0), "null tried list");
		std::vector<ugsdr_tile_shape> all;
		autotune(ctx, jobs, n_jobs, all);
		const int n = static_cast<int>(std::min<size_t>(all.size(), static_cast<size_t>(max_tried)));
		std::copy(all.begin(), all.begin() + n, tried);
		if (n_tried)
			*n_tried = static_cast<int>(all.size());
	});
}
}

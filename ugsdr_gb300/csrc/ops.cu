// Per-op entry points: one C function per reference policy so that each
// Cuda* adapter (include/ugsdr_cuda_policies.hpp) is a drop-in for the
// Sequential*/Ipp*/Af* implementation it replaces.  Host buffers in and out;
// every call stages through the context's device scratch on its stream.
#include "internal.hpp"
#include "acq_kernels.cuh"
#include "dfe.cuh"
#include "packed.cuh"
#include "fft_plan.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <numeric>

namespace ugsdr_gpu {
	namespace {
		constexpr int kT = 256;

		int blocks_for(size_t n, int per = kT) {
			return static_cast<int>(std::min<size_t>((n + per - 1) / per, 152 * 32));
		}

		FftPlanDev dev_plan(const FftPlanDesc& d) {
			FftPlanDev p{};
			p.n = d.n;
			p.n_pass = d.n_pass;
			for (int i = 0; i < d.n_pass; ++i)
				p.radix[i] = d.radix[i];
			p.tw = d.tw;
			return p;
		}

		template <typename K>
		void smem_attr(K kernel, size_t bytes) {
			UG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)));
		}

		// ------------------------------------------------------- kernels
		__global__ void mix_kernel(float2* x, size_t n, uint32_t adder, uint32_t phase0, const float* lut_g) {
			__shared__ float lut[80];
			for (int i = threadIdx.x; i < 80; i += blockDim.x)
				lut[i] = lut_g[i];
			__syncthreads();
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x)
				x[i] = table_mix(x[i], i, adder, phase0, lut);
		}

		// single-CTA complex DFT; conj_in/conj_out implement the inverse by conjugation
		__global__ void dft_small_kernel(const float2* in, float2* out, FftPlanDev plan, int inverse, float scale) {
			extern __shared__ float2 sm[];
			float2* a = sm;
			float2* b = sm + plan.n;
			for (int i = threadIdx.x; i < plan.n; i += blockDim.x)
				a[i] = in[i];
			__syncthreads();
			const float2* y = inverse ? fft_passes<true>(a, b, plan) : fft_passes<false>(a, b, plan);
			for (int i = threadIdx.x; i < plan.n; i += blockDim.x)
				out[i] = scale == 1.0f ? y[i] : cscale(y[i], scale);
		}

		// k1-major (X_T[k1][k2] = X[k1 + N1 k2]) -> natural order, optional conj and scale
		__global__ void untranspose_kernel(const float2* t, float2* out, int n1, int n2, int conj_out, float scale) {
			const size_t n = static_cast<size_t>(n1) * n2;
			for (size_t e = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; e < n; e += static_cast<size_t>(gridDim.x) * blockDim.x) {
				const size_t k1 = e / n2, k2 = e % n2;
				float2 v = t[e];
				if (conj_out)
					v.y = -v.y;
				out[k1 + static_cast<size_t>(n1) * k2] = scale == 1.0f ? v : cscale(v, scale);
			}
		}

		__global__ void conj_kernel(const float2* in, float2* out, size_t n) {
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x)
				out[i] = c2(in[i].x, -in[i].y);
		}

		__global__ void cmul_kernel(float2* x, const float2* s, size_t n) {
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x)
				x[i] = cmul(x[i], s[i]);
		}

		__global__ void real_to_complex_kernel(const float* in, float2* out, size_t n) {
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x)
				out[i] = c2(in[i], 0.f);
		}

		__global__ void conj_mask_kernel(float2* x, size_t n, int one_sided) {
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x)
				x[i] = (one_sided && i > n / 2) ? c2(0.f, 0.f) : c2(x[i].x, -x[i].y);
		}

		// (v / N) * 2 as the reference's FFTW inverse (dft.hpp:194-198), or v / N
		__global__ void inverse_scale_kernel(float2* x, size_t n, int one_sided) {
			const float fn = static_cast<float>(n);
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x) {
				float2 v = c2(__fdiv_rn(x[i].x, fn), __fdiv_rn(x[i].y, fn));
				if (one_sided)
					v = c2(v.x * 2.0f, v.y * 2.0f);
				x[i] = v;
			}
		}

		__global__ void abs_kernel(const float2* x, float* out, size_t n) {
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x)
				out[i] = hypotf(x[i].x, x[i].y);
		}

		template <typename V>
		__global__ void fold_kernel(const V* in, V* out, size_t n, size_t block) {
			const size_t folds = n / block;
			for (size_t j = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; j < block; j += static_cast<size_t>(gridDim.x) * blockDim.x) {
				V s = in[j];
				for (size_t f = 1; f < folds; ++f) {
					const V v = in[j + f * block];
					if constexpr (std::is_same_v<V, float2>)
						s = cadd(s, v);
					else
						s += v;
				}
				out[j] = s;
			}
		}

		struct Partial {
			float max_v;
			uint32_t max_i_lo, max_i_hi;
			double sum;
		};

		// grid-stride first-max + sum partials, one per block
		__global__ void max_sum_kernel(const float* x, size_t n, Partial* parts) {
			__shared__ float s_v[32];
			__shared__ unsigned long long s_i[32];
			__shared__ double s_s[32];
			float bv = -INFINITY;
			unsigned long long bi = ~0ull;
			double sum = 0;
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x) {
				const float v = x[i];
				if (v > bv) {
					bv = v;
					bi = i;
				}
				sum += v;
			}
			for (int o = 16; o > 0; o >>= 1) {
				const float ov = __shfl_down_sync(0xffffffffu, bv, o);
				const unsigned long long oi = __shfl_down_sync(0xffffffffu, bi, o);
				if (ov > bv || (ov == bv && oi < bi)) {
					bv = ov;
					bi = oi;
				}
				sum += __shfl_down_sync(0xffffffffu, sum, o);
			}
			const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
			if (lane == 0) {
				s_v[w] = bv;
				s_i[w] = bi;
				s_s[w] = sum;
			}
			__syncthreads();
			if (threadIdx.x == 0) {
				for (int k = 1; k < (blockDim.x + 31) / 32; ++k) {
					if (s_v[k] > bv || (s_v[k] == bv && s_i[k] < bi)) {
						bv = s_v[k];
						bi = s_i[k];
					}
					sum += s_s[k];
				}
				parts[blockIdx.x] = Partial{bv, static_cast<uint32_t>(bi), static_cast<uint32_t>(bi >> 32), sum};
			}
		}

		__global__ void sq_dev_kernel(const float* x, size_t n, double mean, double* parts) {
			__shared__ double s[32];
			double acc = 0;
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x) {
				const double d = static_cast<double>(x[i]) - mean;
				acc += d * d;
			}
			for (int o = 16; o > 0; o >>= 1)
				acc += __shfl_down_sync(0xffffffffu, acc, o);
			if ((threadIdx.x & 31) == 0)
				s[threadIdx.x >> 5] = acc;
			__syncthreads();
			if (threadIdx.x == 0) {
				for (int k = 1; k < (blockDim.x + 31) / 32; ++k)
					acc += s[k];
				parts[blockIdx.x] = acc;
			}
		}

		template <typename V>
		__global__ void upsample_kernel(const V* in, size_t len, V* out, size_t samples) {
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < samples; i += static_cast<size_t>(gridDim.x) * blockDim.x)
				out[i] = in[(static_cast<unsigned __int128>(i) * len / samples) % len];
		}

		// ZOH to the lcm then boxcar mean over `ratio` (decimator.hpp:144-160), with
		// the reference's sequential float sum (resample_point) for ratios up to
		// 65536.  Beyond that each input is weighted by its overlap instead
		// (input j covers upsampled [ceil(j up/n), ceil((j+1) up/n))), which
		// agrees to float rounding.
		__global__ void resample_kernel(const float2* in, size_t n, uint64_t up, uint64_t ratio, float2* out, size_t n_out) {
			const ResamplePlan rs{up / n, ratio, up, n_out};
			for (size_t k = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; k < n_out; k += static_cast<size_t>(gridDim.x) * blockDim.x) {
				if (ratio <= 65536) {
					out[k] = resample_point(k, rs, [&](uint64_t j) { return in[j]; });
					continue;
				}
				const uint64_t i0 = k * ratio;
				const uint64_t i1 = min(i0 + ratio, up);
				float2 acc = c2(0.f, 0.f);
				if (i0 < i1) {
					uint64_t j = static_cast<uint64_t>((static_cast<unsigned __int128>(i0) * n) / up);
					uint64_t i = i0;
					while (i < i1) {
						// first upsampled index of input j + 1
						const uint64_t next = static_cast<uint64_t>((static_cast<unsigned __int128>(j + 1) * up + n - 1) / n);
						const uint64_t stop = min(next, i1);
						const float w = static_cast<float>(stop - i);
						const float2 v = in[j % n];
						acc = c2(acc.x + w * v.x, acc.y + w * v.y);
						i = stop;
						++j;
					}
				}
				const float r = static_cast<float>(ratio);
				out[k] = c2(acc.x / r, acc.y / r);
			}
		}

		__global__ void dot_kernel(const float2* x, const float* code, size_t n, double* parts) {
			__shared__ double s[2][32];
			double re = 0, im = 0;
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x) {
				re += static_cast<double>(x[i].x) * code[i];
				im += static_cast<double>(x[i].y) * code[i];
			}
			for (int o = 16; o > 0; o >>= 1) {
				re += __shfl_down_sync(0xffffffffu, re, o);
				im += __shfl_down_sync(0xffffffffu, im, o);
			}
			if ((threadIdx.x & 31) == 0) {
				s[0][threadIdx.x >> 5] = re;
				s[1][threadIdx.x >> 5] = im;
			}
			__syncthreads();
			if (threadIdx.x == 0) {
				for (int k = 1; k < (blockDim.x + 31) / 32; ++k) {
					re += s[0][k];
					im += s[1][k];
				}
				parts[2 * blockIdx.x] = re;
				parts[2 * blockIdx.x + 1] = im;
			}
		}

		template <int ST>
		__global__ void convert_kernel(const void* in, float2* out, size_t n) {
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x)
				out[i] = load_sample<ST>(in, i);
		}

		// ------------------------------------------------------- helpers
		void h2d(ugsdr_ctx* ctx, void* d, const void* h, size_t bytes) {
			UG_CUDA(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, ctx->stream));
		}
		void d2h(ugsdr_ctx* ctx, void* h, const void* d, size_t bytes) {
			UG_CUDA(cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, ctx->stream));
			UG_CUDA(cudaStreamSynchronize(ctx->stream));
		}

		// Bluestein chirp-z: X_k = w_k sum_j (x_j w_j) conj(w_{k-j}), w_m = exp(-i pi m^2 / N),
		// the convolution done with M-point FFTs (M >= 2N - 1, all radices supported).
		__global__ void chirp_premul_kernel(const float2* x, const float2* w, float2* a, size_t n, size_t m, int conj_in) {
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < m; i += static_cast<size_t>(gridDim.x) * blockDim.x) {
				if (i < n) {
					float2 v = x[i];
					if (conj_in)
						v.y = -v.y;
					a[i] = cmul(v, w[i]);
				}
				else {
					a[i] = c2(0.f, 0.f);
				}
			}
		}
		__global__ void chirp_postmul_kernel(const float2* conv, const float2* w, float2* out, size_t n, float inv_m, int conj_out) {
			for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n; i += static_cast<size_t>(gridDim.x) * blockDim.x) {
				float2 v = cscale(cmul(conv[i], w[i]), inv_m);
				if (conj_out)
					v.y = -v.y;
				out[i] = v;
			}
		}

		struct Bluestein {
			size_t n = 0, m = 0;
			DevBuf w;      // n chirp values
			DevBuf bf;     // FFT_M of the conjugate chirp, wrapped
			DevBuf a, b;   // M-point work buffers
			DevBuf tmp;
		};

		bool plannable(int n) {
			std::vector<int> r;
			return plan_radices(n, r);
		}

		void dft_device(ugsdr_ctx* ctx, const float2* in, float2* out, size_t n, bool inverse, DevBuf& tmp);

		Bluestein& get_bluestein(ugsdr_ctx* ctx, size_t n) {
			static std::mutex mu;
			static std::map<std::pair<ugsdr_ctx*, size_t>, std::unique_ptr<Bluestein>> cache;
			std::lock_guard<std::mutex> lock(mu);
			auto& slot = cache[{ctx, n}];
			if (slot)
				return *slot;
			auto bl = std::make_unique<Bluestein>();
			bl->n = n;
			size_t m = 2 * n - 1;
			while (!plannable(static_cast<int>(m)))
				++m;
			bl->m = m;
			std::vector<float2> w(n), b(m, c2(0.f, 0.f));
			const double pi = 3.14159265358979323846;
			for (size_t k = 0; k < n; ++k) {
				const uint64_t e = (static_cast<uint64_t>(k) * k) % (2 * n);  // exact m^2 mod 2N
				const double ang = -pi * static_cast<double>(e) / static_cast<double>(n);
				w[k] = c2(static_cast<float>(std::cos(ang)), static_cast<float>(std::sin(ang)));
				const float2 cw = c2(w[k].x, -w[k].y);
				b[k] = cw;
				if (k)
					b[m - k] = cw;
			}
			bl->w.reserve(sizeof(float2) * n);
			bl->bf.reserve(sizeof(float2) * m);
			bl->a.reserve(sizeof(float2) * m);
			bl->b.reserve(sizeof(float2) * m);
			UG_CUDA(cudaMemcpy(bl->w.ptr, w.data(), sizeof(float2) * n, cudaMemcpyHostToDevice));
			UG_CUDA(cudaMemcpy(bl->a.ptr, b.data(), sizeof(float2) * m, cudaMemcpyHostToDevice));
			dft_device(ctx, bl->a.as<float2>(), bl->bf.as<float2>(), m, false, bl->tmp);
			UG_CUDA(cudaStreamSynchronize(ctx->stream));
			slot = std::move(bl);
			return *slot;
		}

		// complex DFT device->device: out = DFT(in) (unnormalised, sign by `inverse`)
		void dft_device(ugsdr_ctx* ctx, const float2* in, float2* out, size_t n, bool inverse, DevBuf& tmp) {
			require(n >= 2 && n <= (1u << 28), "DFT size out of range");
			const int ni = static_cast<int>(n);
			if (!plannable(ni)) {
				// inverse via conj(DFT(conj(x)))
				Bluestein& bl = get_bluestein(ctx, n);
				chirp_premul_kernel<<<blocks_for(bl.m), kT, 0, ctx->stream>>>(in, bl.w.as<float2>(), bl.a.as<float2>(), n, bl.m, inverse ? 1 : 0);
				note_launch(ctx);
				dft_device(ctx, bl.a.as<float2>(), bl.b.as<float2>(), bl.m, false, bl.tmp);
				cmul_kernel<<<blocks_for(bl.m), kT, 0, ctx->stream>>>(bl.b.as<float2>(), bl.bf.as<float2>(), bl.m);
				note_launch(ctx);
				dft_device(ctx, bl.b.as<float2>(), bl.a.as<float2>(), bl.m, true, bl.tmp);
				chirp_postmul_kernel<<<blocks_for(n), kT, 0, ctx->stream>>>(bl.a.as<float2>(), bl.w.as<float2>(), out, n,
					1.0f / static_cast<float>(bl.m), inverse ? 1 : 0);
				note_launch(ctx);
				return;
			}
			if (fits_single_cta(ctx, ni)) {
				FftPlanDev p = dev_plan(get_plan(ctx, ni));
				const size_t smem = 2 * sizeof(float2) * n;
				smem_attr(dft_small_kernel, smem);
				dft_small_kernel<<<1, kT, smem, ctx->stream>>>(in, out, p, inverse ? 1 : 0, 1.0f);
				note_launch(ctx);
				return;
			}
			// the batched four-step kernels over the whole GPU; the inverse as
			// conj(DFT(conj(x)))
			tmp.reserve(2 * sizeof(float2) * n);  // k1-major spectrum, conjugated input
			float2* spec = tmp.as<float2>();
			const float2* src = in;
			if (inverse) {
				float2* c = spec + n;
				conj_kernel<<<blocks_for(n), kT, 0, ctx->stream>>>(in, c, n);
				note_launch(ctx);
				src = c;
			}
			int n1 = 0, n2 = 0;
			dft_four_step(ctx, src, spec, ni, n1, n2);
			untranspose_kernel<<<blocks_for(n), kT, 0, ctx->stream>>>(spec, out, n1, n2, inverse ? 1 : 0, 1.0f);
			note_launch(ctx);
		}
	}

	void dft_scaled(ugsdr_ctx* ctx, const float2* in, float2* out, size_t n, bool inverse, DevBuf& tmp) {
		dft_device(ctx, in, out, n, inverse, tmp);
		if (inverse) {
			inverse_scale_kernel<<<blocks_for(n), kT, 0, ctx->stream>>>(out, n, 1);
			note_launch(ctx);
		}
	}
}

using namespace ugsdr_gpu;

#define UG_ENTRY(ctx) \
	if (!(ctx))       \
		return UGSDR_E_INVALID; \
	std::lock_guard<std::mutex> lock_((ctx)->mutex); \
	return guarded((ctx), [&]

extern "C" {

int ugsdr_mix(ugsdr_ctx* ctx, float* iq, size_t n, double fs, double frequency, double phase) {
	UG_ENTRY(ctx) {
		require(iq != nullptr || n == 0, "null buffer");
		require(fs > 0, "sampling rate must be positive");
		// Mixer::Translate(T&) (mixer.hpp:33-42): FixPhase, zero frequency is a no-op
		const uint32_t phase0 = nco_phase(phase);
		if (std::abs(frequency) == 0.0 || n == 0)
			return;
		const uint32_t adder = nco_adder(fs, frequency);
		ctx->op_a.reserve(sizeof(float2) * n);
		h2d(ctx, ctx->op_a.ptr, iq, sizeof(float2) * n);
		mix_kernel<<<blocks_for(n), kT, 0, ctx->stream>>>(ctx->op_a.as<float2>(), n, adder, phase0, get_lut(ctx));
		note_launch(ctx);
		d2h(ctx, iq, ctx->op_a.ptr, sizeof(float2) * n);
	});
}

int ugsdr_dft(ugsdr_ctx* ctx, const float* in_iq, float* out_iq, size_t n, int inverse) {
	UG_ENTRY(ctx) {
		require(in_iq && out_iq, "null buffer");
		ctx->op_a.reserve(sizeof(float2) * n);
		ctx->op_b.reserve(sizeof(float2) * n);
		h2d(ctx, ctx->op_a.ptr, in_iq, sizeof(float2) * n);
		dft_device(ctx, ctx->op_a.as<float2>(), ctx->op_b.as<float2>(), n, inverse != 0, ctx->op_c);
		if (inverse) {
			inverse_scale_kernel<<<blocks_for(n), kT, 0, ctx->stream>>>(ctx->op_b.as<float2>(), n, 1);
			note_launch(ctx);
		}
		d2h(ctx, out_iq, ctx->op_b.ptr, sizeof(float2) * n);
	});
}

int ugsdr_matched_filter_prepare(ugsdr_ctx* ctx, const float* code, size_t n, int spectrum_mode, float* spectrum_iq) {
	UG_ENTRY(ctx) {
		require(code && spectrum_iq, "null buffer");
		require(spectrum_mode == 0 || spectrum_mode == 1, "bad spectrum mode");
		ctx->op_a.reserve(sizeof(float2) * n);
		ctx->op_b.reserve(sizeof(float2) * n);
		float* staged = reinterpret_cast<float*>(ctx->op_b.as<float2>());
		h2d(ctx, staged, code, sizeof(float) * n);
		real_to_complex_kernel<<<blocks_for(n), kT, 0, ctx->stream>>>(staged, ctx->op_a.as<float2>(), n);
		note_launch(ctx);
		dft_device(ctx, ctx->op_a.as<float2>(), ctx->op_b.as<float2>(), n, false, ctx->op_c);
		conj_mask_kernel<<<blocks_for(n), kT, 0, ctx->stream>>>(ctx->op_b.as<float2>(), n, spectrum_mode == 0);
		note_launch(ctx);
		d2h(ctx, spectrum_iq, ctx->op_b.ptr, sizeof(float2) * n);
	});
}

int ugsdr_matched_filter(ugsdr_ctx* ctx, float* iq, size_t n, const float* spectrum_iq, int spectrum_mode) {
	UG_ENTRY(ctx) {
		require(iq && spectrum_iq, "null buffer");
		ctx->op_a.reserve(sizeof(float2) * n * 2);
		ctx->op_b.reserve(sizeof(float2) * n);
		float2* x = ctx->op_a.as<float2>();
		float2* s = x + n;
		h2d(ctx, x, iq, sizeof(float2) * n);
		h2d(ctx, s, spectrum_iq, sizeof(float2) * n);
		dft_device(ctx, x, ctx->op_b.as<float2>(), n, false, ctx->op_c);
		cmul_kernel<<<blocks_for(n), kT, 0, ctx->stream>>>(ctx->op_b.as<float2>(), s, n);
		note_launch(ctx);
		dft_device(ctx, ctx->op_b.as<float2>(), x, n, true, ctx->op_c);
		inverse_scale_kernel<<<blocks_for(n), kT, 0, ctx->stream>>>(x, n, spectrum_mode == 0);
		note_launch(ctx);
		d2h(ctx, iq, x, sizeof(float2) * n);
	});
}

int ugsdr_abs(ugsdr_ctx* ctx, const float* iq, size_t n, float* out) {
	UG_ENTRY(ctx) {
		require(iq && out, "null buffer");
		ctx->op_a.reserve(sizeof(float2) * n);
		ctx->op_b.reserve(sizeof(float) * n);
		h2d(ctx, ctx->op_a.ptr, iq, sizeof(float2) * n);
		abs_kernel<<<blocks_for(n), kT, 0, ctx->stream>>>(ctx->op_a.as<float2>(), ctx->op_b.as<float>(), n);
		note_launch(ctx);
		d2h(ctx, out, ctx->op_b.ptr, sizeof(float) * n);
	});
}

int ugsdr_reshape_sum(ugsdr_ctx* ctx, const float* in, size_t n, size_t block, int is_complex, float* out) {
	UG_ENTRY(ctx) {
		require(in && out, "null buffer");
		// ReshapeAndSum::CheckBlockSize (reshape_and_sum.hpp:15-18)
		require(block > 0 && n % block == 0, "Signal size is not divided by block size");
		const size_t w = is_complex ? 8 : 4;
		ctx->op_a.reserve(w * n);
		ctx->op_b.reserve(w * block);
		h2d(ctx, ctx->op_a.ptr, in, w * n);
		if (is_complex)
			fold_kernel<float2><<<blocks_for(block), kT, 0, ctx->stream>>>(ctx->op_a.as<float2>(), ctx->op_b.as<float2>(), n, block);
		else
			fold_kernel<float><<<blocks_for(block), kT, 0, ctx->stream>>>(ctx->op_a.as<float>(), ctx->op_b.as<float>(), n, block);
		note_launch(ctx);
		d2h(ctx, out, ctx->op_b.ptr, w * block);
	});
}

int ugsdr_max_index(ugsdr_ctx* ctx, const float* in, size_t n, float* value, size_t* index) {
	UG_ENTRY(ctx) {
		require(in && value && index && n > 0, "null buffer or empty input");
		const int blocks = std::max(1, std::min(blocks_for(n), 1024));
		ctx->op_a.reserve(sizeof(float) * n);
		ctx->op_b.reserve(sizeof(Partial) * blocks);
		h2d(ctx, ctx->op_a.ptr, in, sizeof(float) * n);
		max_sum_kernel<<<blocks, kT, 0, ctx->stream>>>(ctx->op_a.as<float>(), n, ctx->op_b.as<Partial>());
		note_launch(ctx);
		std::vector<Partial> parts(blocks);
		d2h(ctx, parts.data(), ctx->op_b.ptr, sizeof(Partial) * blocks);
		float bv = parts[0].max_v;
		uint64_t bi = parts[0].max_i_lo | (static_cast<uint64_t>(parts[0].max_i_hi) << 32);
		for (int b = 1; b < blocks; ++b) {
			const uint64_t i = parts[b].max_i_lo | (static_cast<uint64_t>(parts[b].max_i_hi) << 32);
			if (parts[b].max_v > bv || (parts[b].max_v == bv && i < bi)) {
				bv = parts[b].max_v;
				bi = i;
			}
		}
		*value = bv;
		*index = static_cast<size_t>(bi);
	});
}

int ugsdr_mean_stddev(ugsdr_ctx* ctx, const float* in, size_t n, float* mean, float* sigma) {
	UG_ENTRY(ctx) {
		require(mean && sigma, "null output");
		// mean_stddev.hpp:30-31: fewer than two samples give {0, 0}
		if (n < 2) {
			*mean = 0;
			*sigma = 0;
			return;
		}
		require(in != nullptr, "null buffer");
		const int blocks = std::max(1, std::min(blocks_for(n), 1024));
		ctx->op_a.reserve(sizeof(float) * n);
		ctx->op_b.reserve(sizeof(Partial) * blocks + sizeof(double) * blocks);
		h2d(ctx, ctx->op_a.ptr, in, sizeof(float) * n);
		max_sum_kernel<<<blocks, kT, 0, ctx->stream>>>(ctx->op_a.as<float>(), n, ctx->op_b.as<Partial>());
		note_launch(ctx);
		std::vector<Partial> parts(blocks);
		d2h(ctx, parts.data(), ctx->op_b.ptr, sizeof(Partial) * blocks);
		double sum = 0;
		for (auto& p : parts)
			sum += p.sum;
		const double m = sum / static_cast<double>(n);
		double* sq = reinterpret_cast<double*>(ctx->op_b.as<char>() + sizeof(Partial) * blocks);
		sq_dev_kernel<<<blocks, kT, 0, ctx->stream>>>(ctx->op_a.as<float>(), n, m, sq);
		note_launch(ctx);
		std::vector<double> sqs(blocks);
		d2h(ctx, sqs.data(), sq, sizeof(double) * blocks);
		const double ss = std::accumulate(sqs.begin(), sqs.end(), 0.0);
		*mean = static_cast<float>(m);
		*sigma = static_cast<float>(std::sqrt(ss / static_cast<double>(n - 1)));
	});
}

int ugsdr_upsample(ugsdr_ctx* ctx, const float* in, size_t n, int is_complex, float* out, size_t samples) {
	UG_ENTRY(ctx) {
		require(in && out && n > 0, "null buffer or empty input");
		const size_t w = is_complex ? 8 : 4;
		ctx->op_a.reserve(w * n);
		ctx->op_b.reserve(w * samples);
		h2d(ctx, ctx->op_a.ptr, in, w * n);
		if (is_complex)
			upsample_kernel<float2><<<blocks_for(samples), kT, 0, ctx->stream>>>(ctx->op_a.as<float2>(), n, ctx->op_b.as<float2>(), samples);
		else
			upsample_kernel<float><<<blocks_for(samples), kT, 0, ctx->stream>>>(ctx->op_a.as<float>(), n, ctx->op_b.as<float>(), samples);
		note_launch(ctx);
		d2h(ctx, out, ctx->op_b.ptr, w * samples);
	});
}

int ugsdr_resample(ugsdr_ctx* ctx, const float* in_iq, size_t n, uint64_t new_fs, uint64_t old_fs, float* out_iq, size_t cap,
	size_t* n_out) {
	UG_ENTRY(ctx) {
		require(n_out != nullptr && new_fs > 0 && old_fs > 0, "null output or zero rate");
		const uint64_t lcm = std::lcm(new_fs, old_fs);
		const unsigned __int128 up128 = static_cast<unsigned __int128>(lcm) * n / old_fs;
		require(up128 < (static_cast<unsigned __int128>(1) << 62), "resampling ratio too large");
		const uint64_t up = static_cast<uint64_t>(up128);
		const uint64_t ratio = lcm / new_fs;
		const uint64_t padded = (up % ratio) ? (up / ratio + 1) * ratio : up;
		const size_t out_n = ratio == 1 ? static_cast<size_t>(up) : static_cast<size_t>(padded / ratio);
		*n_out = out_n;
		if (!out_iq)
			return;
		require(cap >= out_n, "output buffer too small");
		require(in_iq != nullptr && n > 0, "null input");
		ctx->op_a.reserve(sizeof(float2) * n);
		ctx->op_b.reserve(sizeof(float2) * out_n);
		h2d(ctx, ctx->op_a.ptr, in_iq, sizeof(float2) * n);
		resample_kernel<<<blocks_for(out_n), kT, 0, ctx->stream>>>(ctx->op_a.as<float2>(), n, up, ratio, ctx->op_b.as<float2>(), out_n);
		note_launch(ctx);
		d2h(ctx, out_iq, ctx->op_b.ptr, sizeof(float2) * out_n);
	});
}

int ugsdr_correlate(ugsdr_ctx* ctx, const float* iq, const float* code, size_t n, float* out_iq) {
	UG_ENTRY(ctx) {
		require(iq && code && out_iq, "null buffer");
		const int blocks = std::max(1, std::min(blocks_for(n), 1024));
		ctx->op_a.reserve(sizeof(float2) * n + sizeof(float) * n);
		ctx->op_b.reserve(2 * sizeof(double) * blocks);
		float2* x = ctx->op_a.as<float2>();
		float* c = reinterpret_cast<float*>(x + n);
		h2d(ctx, x, iq, sizeof(float2) * n);
		h2d(ctx, c, code, sizeof(float) * n);
		dot_kernel<<<blocks, kT, 0, ctx->stream>>>(x, c, n, ctx->op_b.as<double>());
		note_launch(ctx);
		std::vector<double> parts(2 * blocks);
		d2h(ctx, parts.data(), ctx->op_b.ptr, sizeof(double) * 2 * blocks);
		double re = 0, im = 0;
		for (int b = 0; b < blocks; ++b) {
			re += parts[2 * b];
			im += parts[2 * b + 1];
		}
		out_iq[0] = static_cast<float>(re);
		out_iq[1] = static_cast<float>(im);
	});
}

int ugsdr_convert_samples(ugsdr_ctx* ctx, const void* in, int sample_type, size_t n, float* out_iq) {
	UG_ENTRY(ctx) {
		require(in && out_iq, "null buffer");
		size_t w = 0;
		switch (sample_type) {
		case UGSDR_SAMPLES_CF32: w = 8; break;
		case UGSDR_SAMPLES_CI8: w = 2; break;
		case UGSDR_SAMPLES_CI16: w = 4; break;
		case UGSDR_SAMPLES_RI8: w = 1; break;
		default: require(false, "unknown sample type");
		}
		ctx->op_a.reserve(w * n + 16);
		ctx->op_b.reserve(sizeof(float2) * n);
		h2d(ctx, ctx->op_a.ptr, in, w * n);
		const int g = blocks_for(n);
		switch (sample_type) {
		case UGSDR_SAMPLES_CF32: convert_kernel<UGSDR_SAMPLES_CF32><<<g, kT, 0, ctx->stream>>>(ctx->op_a.ptr, ctx->op_b.as<float2>(), n); break;
		case UGSDR_SAMPLES_CI8: convert_kernel<UGSDR_SAMPLES_CI8><<<g, kT, 0, ctx->stream>>>(ctx->op_a.ptr, ctx->op_b.as<float2>(), n); break;
		case UGSDR_SAMPLES_CI16: convert_kernel<UGSDR_SAMPLES_CI16><<<g, kT, 0, ctx->stream>>>(ctx->op_a.ptr, ctx->op_b.as<float2>(), n); break;
		default: convert_kernel<UGSDR_SAMPLES_RI8><<<g, kT, 0, ctx->stream>>>(ctx->op_a.ptr, ctx->op_b.as<float2>(), n); break;
		}
		note_launch(ctx);
		d2h(ctx, out_iq, ctx->op_b.ptr, sizeof(float2) * n);
	});
}

int ugsdr_unpack_samples(ugsdr_ctx* ctx, const void* in, size_t in_bytes, int sample_type, double sampling_rate,
	size_t n_samples, float* out_iq) {
	UG_ENTRY(ctx) {
		require(in && out_iq, "null buffer");
		require(sample_type >= 0 && sample_type <= UGSDR_SAMPLES_NT1065_4, "unknown sample type");
		const size_t bytes = capture_bytes(sample_type, sampling_rate, n_samples);
		require(bytes > 0 || n_samples == 0, "BBP DDC captures need a whole-kHz rate and whole 1 ms epochs");
		require(in_bytes >= bytes, "input holds fewer bytes than n_samples need");
		if (n_samples == 0)
			return;
		PackedLayout l;
		l.spm = static_cast<uint32_t>(sampling_rate / 1e3);
		l.epoch_bytes = static_cast<uint32_t>(bbp_epoch_bytes(sampling_rate));
		ctx->op_a.reserve(bytes + 16);
		ctx->op_b.reserve(sizeof(float2) * n_samples);
		h2d(ctx, ctx->op_a.ptr, in, bytes);
		unpack_kernel<<<blocks_for(n_samples), kT, 0, ctx->stream>>>(ctx->op_a.ptr, sample_type, l, n_samples, ctx->op_b.as<float2>());
		note_launch(ctx);
		d2h(ctx, out_iq, ctx->op_b.ptr, sizeof(float2) * n_samples);
	});
}
}

// ugsdr_acquire_static: the single-CTA acquisition kernels run with their
// scratch in a file-scope device array instead of context allocations, for
// callers that must not call cudaMalloc (see include/ugsdr_cuda.h).
//
// Scratch layout (256-byte aligned regions of g_static_scratch):
//   twiddles  N float2          W_N^m, computed on the device
//   adders    D uint32          TableMixer NCO adder per Doppler bin
//   code ptrs P pointers        into the code-spectrum region
//   codes     P * N float2      conj(FFT(code))
//   spectra   D * K * N float2  mixed forward spectra
#include "internal.hpp"
#include "acq_kernels.cuh"
#include "fft_plan.hpp"

#include <cmath>
#include <mutex>

namespace ugsdr_gpu {
	namespace {
		static __device__ __align__(256) unsigned char g_static_scratch[UGSDR_STATIC_SCRATCH_BYTES];
		static __device__ float g_static_lut[80];

		constexpr int kMaxDevices = 64;
		std::mutex g_setup_mutex;
		unsigned char* g_scratch_ptr[kMaxDevices] = {};
		float* g_lut_ptr[kMaxDevices] = {};

		size_t align256(size_t x) { return (x + 255) / 256 * 256; }

		// once per device, with that device current: device addresses of the
		// file-scope arrays (the host-side names are only stand-ins) and the
		// mixer table (TableMixer::GetSinCosTable<6, float>, table_mixer.hpp:31-47).
		// A synchronous copy from pageable memory may return before its DMA has
		// landed, and a caller's non-blocking stream is not ordered after the
		// legacy stream, so the set-up waits for the copy before it publishes the
		// addresses.  The cached addresses belong to the device's primary
		// context: resetting the device between calls invalidates them.
		int setup_device(int dev) {
			std::lock_guard<std::mutex> lock(g_setup_mutex);
			if (g_scratch_ptr[dev])
				return UGSDR_OK;
			auto fail = [] {
				cudaGetLastError();
				return UGSDR_E_CUDA;
			};
			void* p = nullptr;
			if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess)
				return fail();
			void* l = nullptr;
			if (cudaGetSymbolAddress(&l, g_static_lut) != cudaSuccess)
				return fail();
			float t[80];
			const double step = 5 * 3.14159265358979323846 / 80 / 2;
			for (int i = 0; i < 80; ++i)
				t[i] = static_cast<float>(std::sin(static_cast<double>(i) * step));
			if (cudaMemcpyToSymbol(g_static_lut, t, sizeof(t)) != cudaSuccess)
				return fail();
			if (cudaDeviceSynchronize() != cudaSuccess)
				return fail();
			g_lut_ptr[dev] = static_cast<float*>(l);
			g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
			return UGSDR_OK;
		}

		// W_N^m = exp(-2 pi i m / N) from sincospi in double, rounded to float
		__global__ void static_twiddle_kernel(float2* tw, int n) {
			for (int m = blockIdx.x * blockDim.x + threadIdx.x; m < n; m += gridDim.x * blockDim.x) {
				double s, c;
				sincospi(2.0 * static_cast<double>(m) / static_cast<double>(n), &s, &c);
				tw[m] = c2(static_cast<float>(c), static_cast<float>(-s));
			}
		}

		// Doppler grid (fse.hpp:250-252, accumulated in double as the reference)
		// and the NCO adder of Translate(signal, fs, -d) (mixer.hpp:46-47, nco.hpp:17-20);
		// code-spectrum pointer table.
		__global__ void static_tables_kernel(uint32_t* adders, int n_doppler, double range, double step, double fs,
			const float2** code_ptrs, float2* codes, int n_codes, int n) {
			if (blockIdx.x == 0 && threadIdx.x == 0) {
				double d = -range;
				for (int i = 0; i < n_doppler; ++i, d += step) {
					double f = -d;
					if (f < 0)
						f = fs + f;
					adders[i] = static_cast<uint32_t>(static_cast<uint64_t>(4294967296.0 * f / fs));
				}
			}
			for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n_codes; c += gridDim.x * blockDim.x)
				code_ptrs[c] = codes + static_cast<size_t>(c) * n;
		}

		// one CTA per code: conj(FFT(code samples)), one-sided mask (matched_filter.hpp:49-54)
		__global__ void static_code_spectra_kernel(const float* code_samples, float2* codes, FftPlanDev plan, int one_sided) {
			extern __shared__ float2 smem[];
			float2* a = smem;
			float2* b = smem + plan.n;
			const int n = plan.n;
			const float* src = code_samples + static_cast<size_t>(blockIdx.x) * n;
			for (int i = threadIdx.x; i < n; i += blockDim.x)
				a[i] = c2(src[i], 0.f);
			__syncthreads();
			const float2* y = fft_passes<false>(a, b, plan);
			float2* out = codes + static_cast<size_t>(blockIdx.x) * n;
			for (int i = threadIdx.x; i < n; i += blockDim.x) {
				const float2 v = y[i];
				out[i] = (one_sided && i > n / 2) ? c2(0.f, 0.f) : c2(v.x, -v.y);
			}
		}

		template <typename K>
		bool smem_ok(K kernel, size_t bytes) {
			return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)) == cudaSuccess;
		}
	}
}

using namespace ugsdr_gpu;

extern "C" int ugsdr_acquire_static(void* cuda_stream, const ugsdr_static_job* job, ugsdr_acq_cell* cells_device,
	size_t* scratch_needed) {
	if (!job || !cells_device || !job->samples || !job->code_samples || job->n_codes < 1)
		return UGSDR_E_INVALID;
	if (job->sample_type < 0 || job->sample_type > 3 || job->block_samples < 2 || job->n_blocks < 1 ||
		job->n_samples < job->block_samples * job->n_blocks || job->sampling_rate <= 0 || job->doppler_step <= 0 ||
		job->doppler_range < 0 || (job->statistic != UGSDR_STAT_ABS && job->statistic != UGSDR_STAT_ABS2) ||
		(job->spectrum_mode != UGSDR_SPECTRUM_ONE_SIDED && job->spectrum_mode != UGSDR_SPECTRUM_TWO_SIDED))
		return UGSDR_E_INVALID;
	if (job->fold_samples && job->block_samples % job->fold_samples != 0)
		return UGSDR_E_INVALID;
	const int n = static_cast<int>(job->block_samples);
	const int m = job->fold_samples ? static_cast<int>(job->fold_samples) : n;
	int n_doppler = 0;
	for (double d = -job->doppler_range; d <= job->doppler_range; d += job->doppler_step)
		if (++n_doppler > 1000000)
			return UGSDR_E_INVALID;
	// launch grids: Doppler bins x blocks (forward), Doppler bins x codes (inverse)
	const size_t grid_fwd = static_cast<size_t>(n_doppler) * job->n_blocks;
	const size_t grid_inv = static_cast<size_t>(n_doppler) * static_cast<size_t>(job->n_codes);
	if (grid_fwd > 0x7fffffffu || grid_inv > 0x7fffffffu)
		return UGSDR_E_INVALID;

	// scratch bytes, checked before anything is launched
	const size_t tw_b = align256(sizeof(float2) * n);
	const size_t ad_b = align256(sizeof(uint32_t) * n_doppler);
	const size_t cp_b = align256(sizeof(void*) * job->n_codes);
	const size_t cs_b = align256(sizeof(float2) * static_cast<size_t>(n) * job->n_codes);
	const size_t sp_b = align256(sizeof(float2) * static_cast<size_t>(n) * job->n_blocks * n_doppler);
	const size_t need = tw_b + ad_b + cp_b + cs_b + sp_b;
	if (scratch_needed)
		*scratch_needed = need;
	if (need > UGSDR_STATIC_SCRATCH_BYTES)
		return UGSDR_E_NOMEM;

	int dev = 0;
	if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
		cudaGetLastError();
		return UGSDR_E_CUDA;
	}
	int optin = 0;
	if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
		cudaGetLastError();
		return UGSDR_E_CUDA;
	}
	const size_t smem_f = 2 * sizeof(float2) * n;
	const size_t smem_i = smem_f + sizeof(float) * m;
	if (smem_i + 1024 > static_cast<size_t>(optin))
		return UGSDR_E_UNSUPPORTED;  // block too large for the single-CTA kernels
	std::vector<int> radices;
	if (!plan_radices(n, radices) || radices.size() > 12)
		return UGSDR_E_UNSUPPORTED;
	if (const int st = setup_device(dev); st != UGSDR_OK)
		return st;

	unsigned char* base = g_scratch_ptr[dev];
	auto* tw = reinterpret_cast<float2*>(base);
	auto* adders = reinterpret_cast<uint32_t*>(base + tw_b);
	auto* code_ptrs = reinterpret_cast<const float2**>(base + tw_b + ad_b);
	auto* codes = reinterpret_cast<float2*>(base + tw_b + ad_b + cp_b);
	auto* spectra = reinterpret_cast<float2*>(base + tw_b + ad_b + cp_b + cs_b);
	cudaStream_t stream = static_cast<cudaStream_t>(cuda_stream);

	FftPlanDev plan{};
	plan.n = n;
	plan.n_pass = static_cast<int>(radices.size());
	for (size_t i = 0; i < radices.size(); ++i)
		plan.radix[i] = radices[i];
	plan.tw = tw;

	// every kernel's shared-memory opt-in is set before the first launch
	bool smem_set = smem_ok(static_code_spectra_kernel, smem_f) && smem_ok(acq_inverse_kernel, smem_i);
	switch (job->sample_type) {
	case UGSDR_SAMPLES_CF32: smem_set = smem_set && smem_ok(acq_forward_kernel<UGSDR_SAMPLES_CF32>, smem_f); break;
	case UGSDR_SAMPLES_CI8: smem_set = smem_set && smem_ok(acq_forward_kernel<UGSDR_SAMPLES_CI8>, smem_f); break;
	case UGSDR_SAMPLES_CI16: smem_set = smem_set && smem_ok(acq_forward_kernel<UGSDR_SAMPLES_CI16>, smem_f); break;
	default: smem_set = smem_set && smem_ok(acq_forward_kernel<UGSDR_SAMPLES_RI8>, smem_f); break;
	}
	if (!smem_set) {
		cudaGetLastError();
		return UGSDR_E_CUDA;
	}

	constexpr int kThreads = 256;
	static_twiddle_kernel<<<(n + kThreads - 1) / kThreads, kThreads, 0, stream>>>(tw, n);
	static_tables_kernel<<<(job->n_codes + kThreads - 1) / kThreads, kThreads, 0, stream>>>(
		adders, n_doppler, job->doppler_range, job->doppler_step, job->sampling_rate, code_ptrs, codes, job->n_codes, n);
	static_code_spectra_kernel<<<job->n_codes, kThreads, smem_f, stream>>>(job->code_samples, codes, plan,
		job->spectrum_mode == UGSDR_SPECTRUM_ONE_SIDED);

	AcqParams p{};
	p.samples = job->samples;
	p.n = n;
	p.k_blocks = static_cast<int>(job->n_blocks);
	p.n_doppler = n_doppler;
	p.n_codes = job->n_codes;
	p.m = m;
	p.fold_mode = job->fold_samples ? (job->fold_coherent ? 1 : 2) : 0;
	p.stat = job->statistic;
	p.one_sided = job->spectrum_mode == UGSDR_SPECTRUM_ONE_SIDED;
	p.adders = adders;
	p.phase0 = 0;
	p.fe_on = job->frontend_frequency != 0.0;
	p.fe_adder = p.fe_on ? nco_adder(job->sampling_rate, job->frontend_frequency) : 0u;
	p.lut = g_lut_ptr[dev];
	p.spectra = spectra;
	p.codes = code_ptrs;
	p.cells = reinterpret_cast<AcqCellDev*>(cells_device);
	p.plan = plan;

	const int grid_f = static_cast<int>(grid_fwd);
	switch (job->sample_type) {
	case UGSDR_SAMPLES_CF32: acq_forward_kernel<UGSDR_SAMPLES_CF32><<<grid_f, kThreads, smem_f, stream>>>(p); break;
	case UGSDR_SAMPLES_CI8: acq_forward_kernel<UGSDR_SAMPLES_CI8><<<grid_f, kThreads, smem_f, stream>>>(p); break;
	case UGSDR_SAMPLES_CI16: acq_forward_kernel<UGSDR_SAMPLES_CI16><<<grid_f, kThreads, smem_f, stream>>>(p); break;
	default: acq_forward_kernel<UGSDR_SAMPLES_RI8><<<grid_f, kThreads, smem_f, stream>>>(p); break;
	}
	acq_inverse_kernel<<<static_cast<int>(grid_inv), kThreads, smem_i, stream>>>(p);
	if (cudaGetLastError() != cudaSuccess)
		return UGSDR_E_CUDA;
	return UGSDR_OK;
}

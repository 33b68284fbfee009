// Host-side internals shared by the translation units of libugsdr_cuda.so.
#pragma once

#include "../../include/ugsdr_cuda.h"

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

namespace ugsdr_gpu {

	// Thrown inside the library, converted to a status at the C boundary.
	struct Error : std::runtime_error {
		int status;
		Error(int s, const std::string& msg) : std::runtime_error(msg), status(s) {}
	};

	inline void check_cuda(cudaError_t e, const char* what) {
		if (e != cudaSuccess)
			throw Error(UGSDR_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
	}
#define UG_CUDA(call) ::ugsdr_gpu::check_cuda((call), #call)

	inline void require(bool cond, const std::string& msg, int status = UGSDR_E_INVALID) {
		if (!cond)
			throw Error(status, msg);
	}

	// Device buffer that only grows (scratch reused across calls).  With a
	// stream it allocates and frees stream-ordered (cudaMallocAsync /
	// cudaFreeAsync), which, unlike cudaFree, does not wait for the whole device.
	struct DevBuf {
		void* ptr = nullptr;
		size_t bytes = 0;
		cudaStream_t stream = nullptr;  // set: stream-ordered allocation on it
		void reserve(size_t n) {
			if (n <= bytes)
				return;
			release();
			const cudaError_t e = stream ? cudaMallocAsync(&ptr, n, stream) : cudaMalloc(&ptr, n);
			if (e != cudaSuccess) {
				cudaGetLastError();
				ptr = nullptr;
				throw Error(UGSDR_E_NOMEM, "device allocation of " + std::to_string(n) + " bytes failed");
			}
			bytes = n;
		}
		template <typename T>
		T* as() const { return static_cast<T*>(ptr); }
		void release() {
			if (ptr) {
				if (stream)
					cudaFreeAsync(ptr, stream);
				else
					cudaFree(ptr);
			}
			ptr = nullptr;
			bytes = 0;
		}
		~DevBuf() { release(); }
		DevBuf() = default;
		DevBuf(const DevBuf&) = delete;
		DevBuf& operator=(const DevBuf&) = delete;
	};

	// FFT plan for one size: radix sequence and the device twiddle table
	// W_N^m = exp(-2 pi i m/N), m < N (double-precision angles, rounded to float).
	constexpr int kMaxPasses = 12;
	struct FftPlanDesc {
		int n = 0;
		int n_pass = 0;
		int radix[kMaxPasses] = {};
		const float2* tw = nullptr;
	};

	// Four-step split N = N1 * N2 for sizes above the single-CTA limit.
	struct LargePlan {
		int n = 0;
		int n1 = 0, n2 = 0;
		FftPlanDesc p1, p2;    // N1-point and N2-point plans (the inter-step twiddles are computed in the kernels)
	};

	// Tile shape of the four-step path for one block size, as set by
	// ugsdr_tile_set or chosen by ugsdr_autotune (0 / -1: the built-in rule).
	struct TileChoice {
		int n1 = 0;         // split N = n1 x N / n1
		int cw = 0;         // columns per column-kernel CTA (natural layout)
		int rw = 0;         // rows per row-kernel CTA
		int warp_cols = -1; // 1: warp-owned column kernel where one is compiled, 0: natural layout
		int warp_rows = -1; // 1: warp-owned row kernel with the warp-owned columns, 0: CTA row tiles
	};

	struct CodeEntry {
		size_t n = 0;
		int spectrum_mode = 0;
		bool large = false;           // stored in the four-step (k1-major) layout
		int n1 = 0;                   // large: the split the layout was built with
		DevBuf spectrum;              // N complex
		// what built the spectrum, so that a new split can rebuild the layout
		std::vector<float> chips;
		size_t repeats = 0, sign_segment = 0;
		uint32_t sign_mask = 0;
	};

	struct Plans;  // fft planning (acq.cu)

	// Device scratch of one in-flight batch of acquisition jobs (grow-only).
	// The context owns one; each serving slot owns its own so batches overlap.
	// tracking banks for the server (track.cu)
	void track_bank_shape(const ugsdr_track_bank* bank, ugsdr_ctx** ctx, int* n_channels, size_t* spm, double* fs);
	void track_enqueue_on(ugsdr_track_bank* bank, const void* dev_samples, int sample_type, int n_epochs,
		ugsdr_track_output* dev_out, cudaStream_t stream);

	struct Workspace {
		DevBuf samples;    // staged host samples
		DevBuf spectra;    // forward spectra X[d][b][N]
		DevBuf slab;       // large-path scratch (B, partials, counters, fold buffers)
		DevBuf cells;      // per (code, doppler) records
		DevBuf params;     // per-job parameter arrays
		DevBuf front;      // front-end output (resampled complex float) of jobs that need one
		size_t reserved() const {
			return samples.bytes + spectra.bytes + slab.bytes + cells.bytes + params.bytes + front.bytes;
		}
		void set_stream(cudaStream_t s) {
			samples.stream = spectra.stream = slab.stream = cells.stream = params.stream = front.stream = s;
		}
		void release() {
			front.release();
			samples.release();
			spectra.release();
			slab.release();
			cells.release();
			params.release();
		}
	};
}

struct ugsdr_ctx {
	int device = 0;
	cudaStream_t own_stream = nullptr;
	cudaStream_t stream = nullptr;
	std::string last_error;
	std::atomic<uint64_t> launches{0};
	std::mutex mutex;

	// twiddle tables and plans per size
	std::map<int, std::unique_ptr<ugsdr_gpu::DevBuf>> twiddles;
	std::map<int, ugsdr_gpu::FftPlanDesc> plans;
	std::map<int, ugsdr_gpu::LargePlan> large_plans;
	std::map<int, ugsdr_gpu::TileChoice> tiles;  // per block size (ugsdr_tile_set / ugsdr_autotune)

	// code spectra
	std::map<int, std::unique_ptr<ugsdr_gpu::CodeEntry>> codes;
	int next_code = 1;

	// scratch
	ugsdr_gpu::DevBuf lut;        // float[80] TableMixer sine table
	ugsdr_gpu::DevBuf zero_adder; // uint32 0: an NCO that leaves samples unchanged
	ugsdr_gpu::Workspace ws;      // acquisition scratch of the synchronous entry points
	ugsdr_gpu::DevBuf op_a, op_b, op_c;  // per-op entry staging
	// interference stage: staged samples, STFT spectra, inverse columns /
	// whole-signal spectrum, per-column candidates, DFT scratch, window
	ugsdr_gpu::DevBuf jam_x, jam_s, jam_t, jam_cand, jam_tmp, jam_window;
	int jam_window_len = 0;
	// tracking banks' staging (host captures, decoded packed captures, host
	// outputs): shared by the context's banks, whose calls the context
	// serialises on its stream, and kept between banks
	ugsdr_gpu::DevBuf track_samples, track_unpacked, track_out;
	// observables: staged bank outputs (host callers), observables, scratch
	ugsdr_gpu::DevBuf obs_in, obs_out, obs_tmp;
	// copies of host-buffer calls that overlap the context stream's kernels
	// (created on first use): a stream and per-slot events
	cudaStream_t copy_stream = nullptr;
	cudaEvent_t slot_copied[2] = {nullptr, nullptr}, slot_used[2] = {nullptr, nullptr};
	int sm_count = 0;
	size_t smem_optin = 0;

	// per-kernel event timing (ugsdr_ctx_enable_timing)
	bool timing = false;
	struct TimedLaunch {
		std::string name;
		cudaEvent_t start, stop;
	};
	std::vector<TimedLaunch> timed;
	std::map<std::string, std::pair<uint64_t, double>> kernel_totals;
};

namespace ugsdr_gpu {
	// Records a start/stop event pair around the launches in its scope when
	// the context has timing enabled.
	struct KernelTimer {
		ugsdr_ctx* ctx;
		ugsdr_ctx::TimedLaunch t{};
		bool on;
		KernelTimer(ugsdr_ctx* c, const char* name) : ctx(c), on(c->timing) {
			if (!on)
				return;
			t.name = name;
			cudaEventCreate(&t.start);
			cudaEventCreate(&t.stop);
			cudaEventRecord(t.start, ctx->stream);
		}
		~KernelTimer() {
			if (!on)
				return;
			cudaEventRecord(t.stop, ctx->stream);
			ctx->timed.push_back(t);
		}
	};
}

namespace ugsdr_gpu {
	// status wrapper used by every C entry point
	template <typename F>
	int guarded(ugsdr_ctx* ctx, F&& f) {
		try {
			f();
			return UGSDR_OK;
		}
		catch (const Error& e) {
			if (ctx)
				ctx->last_error = e.what();
			return e.status;
		}
		catch (const std::exception& e) {
			if (ctx)
				ctx->last_error = e.what();
			return UGSDR_E_INVALID;
		}
	}

	// forward DFT of a device array (n with a four-step split) on the batched
	// kernels, output k1-major; n1, n2 receive the split (acq.cu)
	void dft_four_step(ugsdr_ctx* ctx, const float2* in, float2* out_k1, int n, int& n1, int& n2);

	// complex DFT device to device with the reference's scaling: forward
	// unnormalised, inverse (v / n) * 2 (ops.cu); `in` and `out` distinct
	void dft_scaled(ugsdr_ctx* ctx, const float2* in, float2* out, size_t n, bool inverse, DevBuf& tmp);

	// plan accessors (acq.cu)
	const FftPlanDesc& get_plan(ugsdr_ctx* ctx, int n);
	const LargePlan& get_large_plan(ugsdr_ctx* ctx, int n);
	bool fits_single_cta(ugsdr_ctx* ctx, int n);
	const float* get_lut(ugsdr_ctx* ctx);
	void note_launch(ugsdr_ctx* ctx, int n = 1);

	// batched acquisition (acq.cu): a batch of jobs is enqueued on `stream` with
	// the scratch of `ws`; cells are copied into host_cells (pinned for overlap);
	// finish_jobs turns them into per-code results once the stream reached them.
	struct EnqueuedBatch {
		std::vector<std::vector<double>> grids;    // Doppler grid per job
		std::vector<size_t> cell_offsets;          // per job, in cells
		size_t n_cells = 0;
	};
	EnqueuedBatch enqueue_jobs(ugsdr_ctx* ctx, Workspace& ws, cudaStream_t stream, const ugsdr_acq_job* jobs, int n_jobs,
		void* host_cells);
	void finish_jobs(const EnqueuedBatch& b, const ugsdr_acq_job* jobs, int n_jobs, const void* host_cells,
		ugsdr_acq_result* const* results, ugsdr_acq_cell* cells_out);
	// Device bytes a batch needs beyond what `ws` already holds (admission control).
	size_t jobs_device_bytes(ugsdr_ctx* ctx, const ugsdr_acq_job* jobs, int n_jobs);

	// capture framing (codes.cpp): bytes of a BBP DDC epoch at fs (0 if fs is not
	// a whole number of kHz), bytes of n samples of any sample type (0 if the
	// count is not whole BBP epochs), whether the type is a packed format
	size_t bbp_epoch_bytes(double fs);
	size_t capture_bytes(int sample_type, double fs, size_t n);
	inline bool is_packed(int sample_type) { return sample_type >= UGSDR_SAMPLES_BBP_DDC && sample_type <= UGSDR_SAMPLES_NT1065_4; }

	// shared host helpers (codes.cpp)
	int prn_code(int signal, int sv, float* out, size_t cap, size_t* len);
	// TableMixer adder for Translate(signal, fs, f): f < 0 -> fs + f (mixer.hpp:46-47)
	uint32_t nco_adder(double fs, double f);
	uint32_t nco_phase(double phase);
	std::vector<double> doppler_grid(double range, double step);
}

/*
 * ugsdr_cuda.h - C ABI of the GB300 (sm_103a) acquisition-and-correlation
 * backend for ugsdr.
 *
 * Plain pointers and sizes only.  Every function returns an int status:
 * UGSDR_OK (0) or a negative UGSDR_E_* code; the message of the last failure
 * on a context is available from ugsdr_last_error().  No C++ exception
 * crosses this boundary; the C++ policy adapters (ugsdr_cuda_policies.hpp)
 * turn a failure into std::runtime_error the way the reference's CPU policies
 * throw (e.g. src/math/reshape_and_sum.hpp:17, src/correlator/correlator.hpp:31).
 *
 * Pointers: unless a function says otherwise, buffers are HOST memory owned
 * by the caller (the reference policies work on std::vector); the context
 * owns all device memory (code-spectrum cache, FFT twiddles, scratch).  The
 * batched acquisition job also accepts device-resident samples.
 *
 * Threading: a context serialises its own calls on its stream; use one
 * context per host thread for concurrency (the reference calls its policies
 * from std::execution::par_unseq lambdas, src/acquisition/fse.hpp:294).
 */
#ifndef UGSDR_CUDA_H
#define UGSDR_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define UGSDR_CUDA_ABI_VERSION 9

enum ugsdr_status {
	UGSDR_OK = 0,
	UGSDR_E_INVALID = -1,      /* bad argument (size, range, null pointer) */
	UGSDR_E_CUDA = -2,         /* CUDA runtime error */
	UGSDR_E_NOMEM = -3,        /* device allocation or admission refused */
	UGSDR_E_UNSUPPORTED = -4,  /* size/radix/signal not handled */
	UGSDR_E_NOT_FOUND = -5,    /* unknown handle */
	UGSDR_E_QUEUE_FULL = -6,   /* serving queue has no free slot */
	UGSDR_E_TIMEOUT = -7       /* a bounded device-side wait gave up */
};

/* Signal ids: the values of ugsdr::Signal (src/common.hpp:40-66). */
enum ugsdr_signal {
	UGSDR_GPS_L1CA = 0,
	UGSDR_GPS_L2CM = 1,
	UGSDR_GPS_L5I = 2,
	UGSDR_GPS_L5Q = 3,
	UGSDR_GLONASS_L1OF = 4,
	UGSDR_GLONASS_L2OF = 5,
	UGSDR_GALILEO_E1B = 6,
	UGSDR_GALILEO_E1C = 7
};

/* Sample formats at the front-end boundary (src/signal_parameters.hpp:150-183). */
enum ugsdr_sample_type {
	UGSDR_SAMPLES_CF32 = 0, /* interleaved float I/Q (std::complex<float>) */
	UGSDR_SAMPLES_CI8 = 1,  /* interleaved int8 I/Q  (FileType::Iq_8_plus_8) */
	UGSDR_SAMPLES_CI16 = 2, /* interleaved int16 I/Q (FileType::Iq_16_plus_16) */
	UGSDR_SAMPLES_RI8 = 3,  /* real int8, imag = 0   (FileType::Real_8) */
	/* Packed front-end captures, decoded on the device as the reference's
	 * readers decode them (signal_parameters.hpp:78-85, 186-246):
	 * BBP DDC: 1 ms epochs of an 8-byte header and fs/1e3 complex samples,
	 * two per byte (bits 0-3 and 4-7: imag then real 2-bit fields, each
	 * read as (field | 1), i.e. +-1; helpers/BbpPackedSpan.hpp), the epoch
	 * padded to an even count of 64-bit words; sample counts are whole epochs. */
	UGSDR_SAMPLES_BBP_DDC = 4,
	/* NT1065 grabber: one byte per sample carrying four channels, 2 bits each
	 * (sign, magnitude) -> (2 sign - 1)(1 + 2 magnitude), real
	 * (helpers/NtlabPackedSpan.hpp); _1 .. _4 = FileType::Nt1065GrabberFirst ..
	 * Fourth, bit offsets 6, 4, 2, 0 */
	UGSDR_SAMPLES_NT1065_1 = 5,
	UGSDR_SAMPLES_NT1065_2 = 6,
	UGSDR_SAMPLES_NT1065_3 = 7,
	UGSDR_SAMPLES_NT1065_4 = 8
};

/* Bytes a capture of n_samples samples of sample_type occupies at
 * sampling_rate (BBP DDC: whole 1 ms epochs with their headers and padding,
 * as SignalParametersBase::OpenFile sizes them, signal_parameters.hpp:78-85). */
int ugsdr_sample_bytes(int sample_type, double sampling_rate, size_t n_samples, size_t* bytes);

/* Matched-filter spectrum convention. */
enum ugsdr_spectrum_mode {
	/* reference FFTW path: code spectrum from an r2c transform, bins
	 * N/2+1..N-1 zero, inverse scaled by 2/N (src/math/dft.hpp:37-46, 124-129) */
	UGSDR_SPECTRUM_ONE_SIDED = 0,
	/* IPP / ArrayFire paths: full conj spectrum, inverse scaled by 1/N */
	UGSDR_SPECTRUM_TWO_SIDED = 1
};

enum ugsdr_statistic {
	UGSDR_STAT_ABS = 0,  /* |y|   (SequentialAbs, src/math/abs.hpp:24-32) */
	UGSDR_STAT_ABS2 = 1  /* |y|^2 */
};

typedef struct ugsdr_ctx ugsdr_ctx;

/* ---------------------------------------------------------------- context */
int ugsdr_ctx_create(int device, ugsdr_ctx** out);
int ugsdr_ctx_destroy(ugsdr_ctx* ctx);
/* Run subsequent work on a caller-owned cudaStream_t (NULL = context's own). */
int ugsdr_ctx_set_stream(ugsdr_ctx* ctx, void* cuda_stream);
int ugsdr_ctx_synchronize(ugsdr_ctx* ctx);
const char* ugsdr_last_error(const ugsdr_ctx* ctx);
/* Number of kernels this context has launched so far. */
int ugsdr_ctx_launch_count(const ugsdr_ctx* ctx, uint64_t* count);
int ugsdr_abi_version(void);
/* CUDA-event timing of the engine's kernels on the stream they are launched
 * on (off by default; a pair of events per launch while on). */
int ugsdr_ctx_enable_timing(ugsdr_ctx* ctx, int on);
/* Launch count and summed device time (ms) of the kernels named `kernel`
 * ("acq_forward", "acq_inverse", "acq_forward_large", "acq_inverse_large",
 * "track_bank", ...) since timing was enabled or last reset.  Synchronises. */
int ugsdr_ctx_kernel_time(ugsdr_ctx* ctx, const char* kernel, uint64_t* launches, double* total_ms);
int ugsdr_ctx_reset_timing(ugsdr_ctx* ctx);

/* ------------------------------------------------------------- PRN codes */
/* Replaces ugsdr::Codegen<Impl>::Get<T>(sv) / PrnGenerator<signal>
 * (src/prn_codes/codegen.hpp:23-36, codegen_wrapper.hpp:32-61): writes the
 * +-1 chips of `sv` (0-based id, as the reference) into out[0..cap).  *len
 * receives the code length even when cap is too small (then UGSDR_E_INVALID).
 * LFSR codes (GPS L1 C/A PRN 1-37, L5I/L5Q PRN 1-32, GLONASS L1OF/L2OF) are
 * generated here; the Galileo E1B/E1C memory codes (sv 0-49, the ICD's
 * tables built into the library) come as 8,184 sine-BOC(1,1) half-chips
 * [c, -c] per chip, as MemoryCodes::DecodeBoc returns them
 * (src/prn_codes/MemoryCodes.hpp:33-40). */
int ugsdr_prn_code(int signal, int sv, float* out, size_t cap, size_t* len);

/* RepeatCodeNTimes + Upsampler::Transform (src/common.hpp:78-85,
 * src/resample/upsampler.hpp:30-37): dst[i] = src[(i*L/S) % L], L = len*repeats. */
int ugsdr_repeat_upsample(const float* chips, size_t len, size_t repeats, float* dst, size_t samples);

/* ------------------------------------------------- code-spectrum cache */
/* Builds conj(FFT(code)) on the device for a code of `samples` samples made
 * from `chips` by RepeatCodeNTimes(repeats) + upsampling, optionally with the
 * sign of segment s (length sign_segment samples) flipped where bit s of
 * sign_mask is set (the per-ms sign permutations of ProcessGalileo,
 * src/acquisition/fse.hpp:374-388).  Replaces MatchedFilter::PrepareCodeSpectrum
 * (src/matched_filter/matched_filter.hpp:27-30) for the batched engine; the
 * spectrum stays resident until released or the context is destroyed. */
int ugsdr_code_put(ugsdr_ctx* ctx, const float* chips, size_t n_chips, size_t repeats, size_t samples,
	uint32_t sign_mask, size_t sign_segment, int spectrum_mode, int* handle);
int ugsdr_code_release(ugsdr_ctx* ctx, int handle);

/* ---------------------------------------------------- batched acquisition */
/* One search = FastSearchEngineBase::ProcessBpsk (src/acquisition/fse.hpp:
 * 242-276) for every code in `codes`, over K = n_blocks consecutive coherent
 * blocks of block_samples samples whose GetOneMsPeak outputs (fse.hpp:201-220)
 * are summed non-coherently (K = 1 is the reference as written).
 * Doppler grid: d = -range; d <= range; d += step (fse.hpp:250-252), each
 * applied with the TableMixer NCO (src/mixer/table_mixer.hpp:78-101). */
typedef struct ugsdr_acq_job {
	const void* samples;       /* n_samples samples of sample_type */
	int sample_type;           /* ugsdr_sample_type */
	int samples_on_device;     /* 1: `samples` is a device pointer */
	size_t n_samples;          /* >= block_samples * n_blocks */
	double sampling_rate;      /* Hz (the acquisition rate, new_sampling_rate) */
	double intermediate_frequency; /* added to the reported Doppler (fse.hpp:263) */
	/* Front-end translation applied before the Doppler mix, as
	 * Mixer::Translate(signal, fs, frontend_frequency) (fse.hpp:289, 348);
	 * 0 = none.  For a signal at IF f_if the reference passes -f_if. */
	double frontend_frequency;
	double code_offset_ratio;  /* signal_fs / acquisition_fs (fse.hpp:247, 262) */
	size_t block_samples;      /* N: coherent block = FFT size */
	size_t n_blocks;           /* K */
	size_t fold_samples;       /* 0: no reshape; else samples per ms (fse.hpp:203) */
	int fold_coherent;         /* 1: |.| then fold; 0: fold complex then |.| (fse.hpp:209-218) */
	double doppler_range;
	double doppler_step;
	const int* codes;          /* n_codes handles from ugsdr_code_put (same N, mode) */
	int n_codes;
	int statistic;             /* ugsdr_statistic */
	int spectrum_mode;         /* ugsdr_spectrum_mode, must match the codes */
	/* Rate of `samples` when it differs from sampling_rate (0 = the same).  The
	 * front end then runs on the device before the search, as AcquireL5 /
	 * AcquireGoldCodesL1 do on the host (fse.hpp:289-291, 312-314):
	 * frontend_frequency is applied at this rate, and the result is resampled
	 * to sampling_rate by SequentialResampler (resampler.hpp:39-46; ZOH to the
	 * lcm, boxcar mean, same float rounding).  Both rates must be integers in
	 * Hz with lcm/sampling_rate <= 65536; n_samples counts input samples, and
	 * the resampled length must cover block_samples * n_blocks. */
	double input_sampling_rate;
} ugsdr_acq_job;

/* Per-code result: the AcquisitionResult<T> fields (src/acquisition/acquisition_result.hpp:11-19). */
typedef struct ugsdr_acq_result {
	int code;            /* handle */
	int doppler_bin;     /* index into the Doppler grid of the kept maximum */
	uint32_t index;      /* peak sample index in the (folded) output */
	uint32_t n_doppler;  /* Doppler bins searched */
	double doppler;      /* grid Doppler + intermediate_frequency */
	double code_offset;  /* code_offset_ratio * index */
	double level;        /* peak value */
	double sigma;        /* std + mean, as AcquisitionResult::sigma (fse.hpp:261) */
	double mean;
	double std;
	double snr;          /* level / sigma (GetSnr) */
} ugsdr_acq_result;

/* Per (code, Doppler) cell record, optional output. */
typedef struct ugsdr_acq_cell {
	float level;
	uint32_t index;
	float mean;
	float std;
} ugsdr_acq_cell;

/* Runs one job; results[n_codes]; cells (optional, may be NULL) receives
 * n_codes x n_doppler records, code-major. */
int ugsdr_acquire(ugsdr_ctx* ctx, const ugsdr_acq_job* job, ugsdr_acq_result* results, ugsdr_acq_cell* cells);
/* Runs several jobs back to back on the context's stream (one persistent set
 * of launches per job, no host synchronisation in between). */
int ugsdr_acquire_batch(ugsdr_ctx* ctx, const ugsdr_acq_job* jobs, int n_jobs, ugsdr_acq_result* const* results);
/* Number of Doppler bins the reference loop visits for (range, step). */
int ugsdr_doppler_bins(double range, double step, uint32_t* n);

/* ------------------------------------------------ four-step tile shapes */
/* No counterpart in the reference (FFTW plans its own transforms): block
 * sizes above the single-CTA limit run as N = n1 x (N / n1) four-step
 * transforms, and these calls read, pin or tune the shape of one size.
 * A shape changes the kernels' tiling and, through n1, the order of the
 * float sums: results agree with another shape's within float rounding,
 * and peaks and Doppler bins are the same on any signal above threshold. */
typedef struct ugsdr_tile_shape {
	int n1;          /* split (0 in ugsdr_tile_set: the built-in rule, the largest n1 <= sqrt N that fits) */
	int cols;        /* columns per column-kernel CTA: 1, 2, 4 or 8 (0: rule) */
	int rows;        /* rows per row-kernel CTA: 1, 2, 4 or 8 (0: rule) */
	int warp_cols;   /* 1: warp-owned column kernel where one is compiled for the split, 0: one tile of
	                    `cols` columns per CTA, -1: rule (the warp-owned kernel where compiled) */
	int warp_rows;   /* 1: warp-owned row kernel (with the warp-owned columns; each warp takes whole rows through
	                    both passes, code rows staged), 2: the same with three rows per warp and the code rows read
	                    through L1 / L2, 0: rows in CTA tiles of `rows` rows, -1: rule (1 where compiled) */
	int block_samples; /* N the shape is for (filled by ugsdr_tile_get / ugsdr_autotune, ignored by ugsdr_tile_set) */
	double ms;       /* ugsdr_autotune: device time of the tuning search with this shape */
} ugsdr_tile_shape;
/* The shape block_samples runs with now (every field resolved). */
int ugsdr_tile_get(ugsdr_ctx* ctx, size_t block_samples, ugsdr_tile_shape* shape);
/* Pins block_samples' shape (NULL: back to the rule), e.g. one an earlier
 * ugsdr_autotune chose; a shape outside the kernels' shared-memory or launch
 * limits returns UGSDR_E_UNSUPPORTED and leaves the old one.  A new n1
 * rebuilds the context's cached code spectra of that size: call it while no
 * search of that size is in flight. */
int ugsdr_tile_set(ugsdr_ctx* ctx, size_t block_samples, const ugsdr_tile_shape* shape);
/* Autotuner: for every block size above the single-CTA limit among `jobs`,
 * runs those jobs (Doppler grids cut to about 1.6e10 complex points per search)
 * with candidate shapes and keeps the fastest: the split (the rule's, the
 * next smaller divisor, the rule's transposed), then the column kernel and
 * its width, then the row kernel and the rows per row CTA, each stage from
 * the best so far; the rule's shape stays unless another is 3 % faster.
 * Each candidate runs once untimed and twice timed with CUDA events (the
 * best counts).  tried
 * receives up to max_tried measured shapes, n_tried (may be NULL) their
 * number.  Same caveat as ugsdr_tile_set for in-flight searches. */
int ugsdr_autotune(ugsdr_ctx* ctx, const ugsdr_acq_job* jobs, int n_jobs, ugsdr_tile_shape* tried, int max_tried,
	int* n_tried);

/* ------------------------------------------- allocation-free acquisition */
/* No counterpart in the reference: an extra entry point of this library.
 *
 * ugsdr_acquire_static runs the same search as ugsdr_acquire (single-CTA block
 * sizes: block_samples up to about 11,000) without allocating any device
 * memory.  It is meant for callers that must not call cudaMalloc: real-time
 * receiver loops, where an allocation can synchronise the device and take an
 * unbounded time, and host applications whose device memory is owned by
 * another allocator or pool that reserves HBM up front, so an extra cudaMalloc
 * would fail or fragment it.  Such callers allocate inputs and outputs
 * themselves and pass device pointers.
 *
 * Scratch (code spectra, mixed spectra, twiddles, Doppler table) lives in one
 * file-scope device array of UGSDR_STATIC_SCRATCH_BYTES, which every GPU that
 * loads the library holds until the process exits.  A job needing more is
 * rejected with UGSDR_E_NOMEM and *scratch_needed set to the bytes it needs.
 * The first call on a device (with that device current) resolves the array's
 * device address and uploads the mixer table, waiting for the upload to land
 * (it synchronises the device once); make that first call before any stream
 * capture.  The resolved addresses are kept for the life of the process: do
 * not reset the device (cudaDeviceReset) between calls.  All calls share the
 * one array: calls that overlap on the
 * GPU (different streams or host threads without ordering) race on it.
 * Nothing in it needs to start at zero; each call rewrites what it reads. */
#define UGSDR_STATIC_SCRATCH_BYTES (16u << 20)

typedef struct ugsdr_static_job {
	const void* samples;       /* DEVICE pointer: n_samples samples of sample_type */
	int sample_type;           /* ugsdr_sample_type */
	size_t n_samples;          /* >= block_samples * n_blocks */
	double sampling_rate;      /* Hz */
	double frontend_frequency; /* as ugsdr_acq_job::frontend_frequency (0 = none) */
	size_t block_samples;      /* N */
	size_t n_blocks;           /* K */
	size_t fold_samples;       /* as ugsdr_acq_job */
	int fold_coherent;
	double doppler_range;
	double doppler_step;
	const float* code_samples; /* DEVICE pointer: n_codes x block_samples code samples (+-1) */
	int n_codes;
	int statistic;             /* ugsdr_statistic */
	int spectrum_mode;         /* ugsdr_spectrum_mode */
} ugsdr_static_job;

/* cells_device: DEVICE pointer to n_codes x n_doppler records (code-major),
 * written on `cuda_stream` (a cudaStream_t; NULL = legacy default stream).
 * Returns after enqueueing; synchronise the stream before reading the cells.
 * scratch_needed (optional) receives the scratch bytes the job uses. */
int ugsdr_acquire_static(void* cuda_stream, const ugsdr_static_job* job, ugsdr_acq_cell* cells_device,
	size_t* scratch_needed);

/* ---------------------------------------------- per-op policy entries */
/* Each replaces one reference policy implementation; host buffers. */

/* Mixer<Impl>::Translate(T& src_dst, fs, f, phase) with TableMixer arithmetic
 * (src/mixer/mixer.hpp:33-42, src/mixer/table_mixer.hpp:78-101). In place. */
int ugsdr_mix(ugsdr_ctx* ctx, float* iq, size_t n, double fs, double frequency, double phase);
/* SequentialDft::Transform on complex data (src/math/dft.hpp:114-135, 211-220):
 * forward unnormalised, inverse scaled 2/N (FFTW path). */
int ugsdr_dft(ugsdr_ctx* ctx, const float* in_iq, float* out_iq, size_t n, int inverse);
/* No counterpart in the reference: a measurement entry.  `count` 25-point
 * forward DFTs (the radix-25 butterfly of the four-step inverse) of device
 * complex-float data, in[i * 25 + j] -> out[i * 25 + k], computed on the CUDA
 * cores (the butterfly the transforms use) or on the tensor cores (tcgen05,
 * 3xTF32 split, one 128 x 64 x 56 product per 128 transforms); kernel_ms
 * (may be NULL) receives the kernel's CUDA-event time. */
enum ugsdr_dft25_method { UGSDR_DFT25_CUDA_CORES = 0, UGSDR_DFT25_TENSOR_CORES = 1 };
int ugsdr_dft25_batch(ugsdr_ctx* ctx, const void* in, void* out, size_t count, int method, float* kernel_ms);
/* MatchedFilter::PrepareCodeSpectrum (src/matched_filter/matched_filter.hpp:27-30, 49-54). */
int ugsdr_matched_filter_prepare(ugsdr_ctx* ctx, const float* code, size_t n, int spectrum_mode, float* spectrum_iq);
/* MatchedFilter::FilterOptimized (matched_filter.hpp:32-35, 56-61), in place. */
int ugsdr_matched_filter(ugsdr_ctx* ctx, float* iq, size_t n, const float* spectrum_iq, int spectrum_mode);
/* Abs::Transform (src/math/abs.hpp:13-17). */
int ugsdr_abs(ugsdr_ctx* ctx, const float* iq, size_t n, float* out);
/* ReshapeAndSum::Transform (src/math/reshape_and_sum.hpp:20-30): real (is_complex=0)
 * or complex data folded to `block` values; UGSDR_E_INVALID when n % block != 0. */
int ugsdr_reshape_sum(ugsdr_ctx* ctx, const float* in, size_t n, size_t block, int is_complex, float* out);
/* MaxIndex::Transform (src/math/max_index.hpp:15-24): first maximum. */
int ugsdr_max_index(ugsdr_ctx* ctx, const float* in, size_t n, float* value, size_t* index);
/* MeanStdDev::Calculate (src/math/mean_stddev.hpp:13-22): mean, unbiased sigma. */
int ugsdr_mean_stddev(ugsdr_ctx* ctx, const float* in, size_t n, float* mean, float* sigma);
/* Upsampler::Transform (src/resample/upsampler.hpp:13-23), real or complex. */
int ugsdr_upsample(ugsdr_ctx* ctx, const float* in, size_t n, int is_complex, float* out, size_t samples);
/* Resampler::Transform (src/resample/resampler.hpp:15-25; ZOH to the lcm then
 * boxcar mean, decimator.hpp:144-160), complex samples.  *n_out receives the
 * output length; pass out = NULL to query it. */
int ugsdr_resample(ugsdr_ctx* ctx, const float* in_iq, size_t n, uint64_t new_fs, uint64_t old_fs,
	float* out_iq, size_t cap, size_t* n_out);
/* Correlator::Correlate (src/correlator/correlator.hpp:16-20, 27-34). */
int ugsdr_correlate(ugsdr_ctx* ctx, const float* iq, const float* code, size_t n, float* out_iq);
/* SignalParametersBase::GetPartialSignal int -> complex<float> conversion
 * (src/signal_parameters.hpp:150-183). */
int ugsdr_convert_samples(ugsdr_ctx* ctx, const void* in, int sample_type, size_t n, float* out_iq);
/* SignalParametersBase::GetSeveralMs for any sample type (signal_parameters.hpp:
 * 150-246, 262-273): decodes n_samples samples (whole epochs for BBP DDC) of
 * `in` (in_bytes bytes, host) captured at sampling_rate into out_iq
 * (n_samples complex floats, host). */
int ugsdr_unpack_samples(ugsdr_ctx* ctx, const void* in, size_t in_bytes, int sample_type, double sampling_rate,
	size_t n_samples, float* out_iq);

/* ------------------------------------------------------ tracking bank */
/* Correlator bank for many channels per 1 ms epoch (Tracker::Track,
 * src/tracking/tracker.hpp:186-197): per channel and epoch the carrier
 * wipe-off (TableMixer, 6-bit LUT, with the NCO phase held as a 64-bit
 * fixed-point accumulator), five taps VE/E/P/L/VL each computed as
 * TrackingParameters::CorrelateSplit (two dot products split at the code
 * period, combined by AddWithPhase; tracking_parameters.hpp:89-98, 472-493),
 * then Pll(prompt) and Dll(early, late) in FP64 (tracking_parameters.hpp:
 * 495-528; Tracker::GetEpl order, tracker.hpp:119-177).  One launch advances
 * every channel over many epochs; the state stays on the device between calls. */
typedef struct ugsdr_track_channel {
	int code;                 /* index into the bank's code table */
	double sampling_rate;     /* Hz (all channels of a bank share it) */
	double code_frequency;    /* chips/s, base (BOC: half-chips, 2.046e6 for E1B) */
	double code_length;       /* chips per code period (period = length / frequency, in ms) */
	double code_phase;        /* samples, TrackingParameters::code_phase semantics */
	double carrier_frequency; /* Hz (Doppler + IF) */
	double carrier_phase;     /* rad */
	int boc;                  /* informational: VE/VL taps are for BOC signals */
} ugsdr_track_channel;

typedef struct ugsdr_track_config {
	double early_late_spacing;      /* chips from prompt to E and L (reference: 0.25) */
	double very_early_late_spacing; /* chips from prompt to VE and VL */
	double pll_bandwidth;           /* Hz (reference 25) */
	double dll_bandwidth;           /* Hz (reference 0.7) */
	double fll_bandwidth;           /* Hz, FLL assist; 0 = off (reference 250) */
	double integration_time;        /* s; 0.001 (one epoch) is supported */
	/* Carrier NCO: 0 = 64-bit fixed-point phase, continuous across epochs
	 * (cycles * 2^64, top 6 bits index the 64-entry LUT); 1 = the reference's:
	 * the carrier phase in double radians (UpdatePhase, Pll), each epoch's
	 * wipe-off a fresh 32-bit TableMixer NCO from it (Mixer::Translate,
	 * src/mixer/mixer.hpp:33-42, nco.hpp:17-20) and the PLL discriminator's
	 * atan in double, as tracking_parameters.hpp:495-511 computes it. */
	int nco_mode;
} ugsdr_track_config;

/* Per channel per epoch output: taps VE, E, P, L, VL as I/Q and loop state. */
typedef struct ugsdr_track_output {
	float taps[5][2];
	double carrier_frequency;
	double carrier_phase;       /* rad: wrapped (nco_mode 0), the reference's unwrapped phase (nco_mode 1) */
	double code_phase;          /* samples (TrackingParameters::code_phases) */
	double code_frequency;
	double phase_error;         /* PLL discriminator, cycles */
	double code_error;          /* DLL discriminator */
} ugsdr_track_output;

typedef struct ugsdr_track_bank ugsdr_track_bank;

/* codes: n_codes x code_len_max chips (+-1), code_lens[n_codes]. */
int ugsdr_track_create(ugsdr_ctx* ctx, const ugsdr_track_config* cfg, const ugsdr_track_channel* channels, int n_channels,
	const float* codes, const int* code_lens, int n_codes, int code_len_max, ugsdr_track_bank** bank);
/* Advances every channel by n_epochs epochs of samples (n_epochs * samples_per_epoch,
 * one shared sampling rate), writing n_epochs x n_channels outputs (host or NULL). */
int ugsdr_track_run(ugsdr_track_bank* bank, const void* samples, int sample_type, int samples_on_device,
	size_t samples_per_epoch, int n_epochs, ugsdr_track_output* outputs);
/* Device-resident variant: `samples` and `outputs` (n_epochs x n_channels, or
 * NULL) are device pointers; enqueued on the context stream without waiting
 * (ugsdr_ctx_synchronize or the caller's stream order completes it).  No
 * reference counterpart: Tracker::Track (tracker.hpp:185-200) works on host
 * vectors; this is the form a device-resident caller chains behind its own
 * front end. */
int ugsdr_track_run_device(ugsdr_track_bank* bank, const void* samples, int sample_type, size_t samples_per_epoch,
	int n_epochs, ugsdr_track_output* outputs);
int ugsdr_track_destroy(ugsdr_track_bank* bank);

/* Acquisition -> tracking hand-off: TrackingParameters::AddSignalImpl's
 * code-phase refinement (src/tracking/tracking_parameters.hpp:297-357) for
 * n_channels channels at once, on the device.  Per channel: the first three
 * code periods of `samples` (n_samples >= 3 periods at the channel's rate),
 * translated by -carrier_frequency, matched-filtered against one code period
 * upsampled, zero-padded to three periods and rotated right by
 * (integer) code_phase; |.| folded to one period; the first maximum's offset
 * (wrapped to +-period / 2) goes to offsets[c] (may be NULL), and when it is
 * within 1e-6 fs samples of a whole number of ms, accepted[c] = 1 and the
 * channel's code_phase += offset (else accepted[c] = 0, code_phase kept).
 * codes: n_codes x code_len_max chips as for ugsdr_track_create.  All
 * channels' filters run as one batch of one-row acquisition jobs.  (An
 * arbitrary replica given as samples is ugsdr_code_put with repeats 1 and
 * samples = its length.) */
int ugsdr_track_refine(ugsdr_ctx* ctx, ugsdr_track_channel* channels, int n_channels, const float* codes,
	const int* code_lens, int n_codes, int code_len_max, const void* samples, int sample_type, int samples_on_device,
	size_t n_samples, int* accepted, int* offsets);

/* ------------------------------------------------------- observables */
/* Tracking outputs -> measurements (src/measurements/observable.hpp), for
 * every channel of a bank at once.  `outputs` is the n_epochs x n_channels
 * array ugsdr_track_run / ugsdr_track_run_device wrote ([epoch][channel]),
 * on the device when outputs_on_device, else host. */

/* Navigation message whose preamble ugsdr_preamble_search looks for. */
typedef enum ugsdr_nav_message {
	UGSDR_NAV_GPS_LNAV = 0,     /* 8-bit preamble, 20 ms bits (observable.hpp:90-98) */
	UGSDR_NAV_GLONASS = 1       /* 40-symbol time mark, 10 ms (observable.hpp:141-151) */
} ugsdr_nav_message;

/* FindPreambleGps / FindPreambleGlonass's candidate search
 * (observable.hpp:204-220, 260-277): per channel the navigation symbols
 * sign(prompt I) (+1 when > 0, else -1) over all n_epochs epochs are
 * circularly matched-filtered against the preamble upsampled to 1 ms (the
 * reference's FFT matched filter, 2/N inverse scale, so |y| is twice the
 * +-1 correlation) and every epoch with |y| above the reference's threshold
 * (153 GPS, 370 GLONASS) is listed in ascending order.  The correlation is
 * computed exactly in integers, so the list equals the reference's float
 * one (|y| is a multiple of 4, the thresholds are not).  messages[c]: a
 * ugsdr_nav_message per channel.  counts[c] = the number of candidates
 * (may exceed cap); indexes: n_channels x cap epochs (host), the first
 * min(counts[c], cap) of row c valid. */
int ugsdr_preamble_search(ugsdr_ctx* ctx, const ugsdr_track_output* outputs, int outputs_on_device, int n_epochs,
	int n_channels, const int* messages, int* counts, int* indexes, int cap);

/* Per channel: Observable's constructor inputs (observable.hpp:75-88) and
 * UpdatePseudoranges' term (327-336). */
typedef struct ugsdr_observable_channel {
	double sampling_rate;          /* Hz */
	double intermediate_frequency; /* Hz */
	double carrier_frequency;      /* Hz, the tracking channel's value before epoch 0 */
	double carrier_phase;          /* rad, the tracking channel's value before epoch 0 */
	long long preamble_position;   /* epoch whose code phase gives the integer-ms offset */
	double range_correction_ms;    /* added to every pseudorange: UpdatePseudorangeGps/Glonass's
	                                  time_scale[i] - (i - preamble_position + tow_ms + 2), which
	                                  does not depend on i; 0 before the time scale is known */
} ugsdr_observable_channel;

/* One channel-epoch measurement. */
typedef struct ugsdr_observable {
	double pseudorange; /* ms: code_phases[i] * 1000 / fs - int32(code_phases[pos] * 1000 / fs) + correction */
	double pseudophase; /* cycles: -carrier_phase[i] / 2 pi + (i + 1) * IF / 1000 */
	double doppler;     /* Hz: frequencies[i] - IF */
	double snr;         /* dB-Hz: 27 + 20 log10(|I_P[i]| / sigma(Q_P)) (CalculateSnr, 55-72) */
} ugsdr_observable;

/* Observable's per-epoch arithmetic for all channels.  The carrier phase
 * is the tracking loop's unwrapped phase (carrier_phase before epoch 0, plus
 * each epoch's carrier_frequency / 1000 and phase_error / 4 cycles), which
 * the bank outputs wrapped; sigma is SequentialMeanStdDev over the
 * channel's prompt Q in float, in epoch order.  out: n_epochs x n_channels
 * ([epoch][channel]), on the device when outputs_on_device, else host. */
int ugsdr_observables(ugsdr_ctx* ctx, const ugsdr_track_output* outputs, int outputs_on_device, int n_epochs,
	int n_channels, const ugsdr_observable_channel* channels, ugsdr_observable* out);

/* --------------------------------------------- interference mitigation */
/* The antijamming stage the digital front end runs after resampling when
 * mitigation is enabled (src/dfe/dfe.hpp:199-202). */

/* ShortTimeFourierTransform<SequentialStft>::Transform(src, window_length,
 * overlap_length) (src/math/stft.hpp:19-21, 42-61): column i is samples
 * [i * hop, i * hop + window_length), hop = window_length - overlap_length,
 * times the periodic Hann window 0.5 (1 - cos(2 pi j / window_length)),
 * forward unnormalised DFT; n_columns = (n - overlap_length) / hop.
 * out_iq (may be NULL: count only) receives n_columns x window_length
 * complex.  Needs n >= window_length > overlap_length >= 0.  The reference's
 * defaults are 128 and 96. */
int ugsdr_stft(ugsdr_ctx* ctx, const float* in_iq, size_t n, int window_length, int overlap_length, float* out_iq,
	size_t* n_columns);
/* The container-of-containers overload, OverlapAndAdd (stft.hpp:63-75):
 * each column's inverse DFT scaled 2 / window_length (the reference's FFTW
 * inverse) added at i * hop into window_length + (n_columns - 1) * hop
 * samples, in column order. */
int ugsdr_istft(ugsdr_ctx* ctx, const float* in_iq, size_t n_columns, int window_length, int overlap_length,
	float* out_iq);

/* JammingDetector::DetectionResult::InterferenceType
 * (src/antijamming/jamming_detection.hpp:30-34) */
enum ugsdr_interference_type {
	UGSDR_INTERFERENCE_NONE = 0,
	UGSDR_INTERFERENCE_NARROWBAND = 1,
	UGSDR_INTERFERENCE_WIDEBAND = 2
};
/* JammingDetector::DetectionResult (jamming_detection.hpp:29-48) */
typedef struct ugsdr_jamming_detection {
	int type;                /* ugsdr_interference_type */
	int frequency_bin;       /* STFT bin (of 128) */
	double frequency;        /* Hz: frequency_bin * fs / 128 */
	double jammer_to_noise;  /* candidate peak / sigma, averaged over the columns */
} ugsdr_jamming_detection;

/* JammingDetector(fs).Process(src) (jamming_detection.hpp:196-201): STFT
 * (128 / 96), per column the 8 strongest bins (each nulled +-3 bins after it
 * is taken) kept when peak / sigma of the nulled magnitudes >= 6, then the
 * occupation analysis (AnalyzeStftData, 130-189).  iq: n complex samples,
 * host or (samples_on_device) device memory.  Up to `cap` detections go to
 * `out`; *n_detections receives their count. */
int ugsdr_jamming_detect(ugsdr_ctx* ctx, const float* iq, size_t n, double fs, int samples_on_device,
	ugsdr_jamming_detection* out, int cap, int* n_detections);
/* JammingSuppressionEngine<complex<float>>(fs).Process(src_dst)
 * (src/antijamming/jse.hpp:89-102), in place: no detection leaves the
 * samples unchanged; narrowband detections only null +-128 bins of the
 * whole-signal DFT around each jammer (inverse scaled 2 / n); any wideband
 * detection zeroes every STFT bin with |.| >= 20 and resynthesises by
 * OverlapAndAdd, truncated or zero-padded to n.  Detections as for
 * ugsdr_jamming_detect. */
int ugsdr_jamming_suppress(ugsdr_ctx* ctx, float* iq, size_t n, double fs, int samples_on_device,
	ugsdr_jamming_detection* out, int cap, int* n_detections);

/* ------------------------------------------------------------ serving */
/* Continuous-batching acquisition and tracking server.  A worker thread admits queued jobs
 * into `max_inflight` slots, each with its own CUDA stream and scratch, as
 * soon as a slot is free and the job's device-memory estimate fits the
 * budget; admitted jobs run concurrently on the device while later requests
 * keep arriving.  Code spectra (ugsdr_code_put handles) stay resident across
 * requests; do not release a handle that a pending job uses. */
typedef struct ugsdr_server ugsdr_server;
/* Admission order of pending requests. */
enum ugsdr_serve_policy {
	UGSDR_SERVE_FIFO = 0,       /* oldest first */
	/* highest response ratio next: (wait + estimated service) / estimated
	 * service, the service estimated from the request's cell-blocks (codes x
	 * Doppler bins x block samples x blocks) and the server's measured
	 * throughput — short searches go first, long ones age to the front.  A
	 * search estimated below 20 ms (the latency target) is short: it runs on
	 * its slot's highest-priority CUDA stream, so its blocks are dispatched
	 * ahead of running long searches, and one slot (with max_inflight >= 2)
	 * admits only short searches, so long ones cannot hold every slot */
	UGSDR_SERVE_RESPONSE_RATIO = 1
};

typedef struct ugsdr_server_config {
	int max_inflight;          /* concurrent jobs on the device (0 = 4) */
	size_t memory_budget;      /* device bytes the slots' scratch may hold (0 = 80 % of free memory) */
	int queue_capacity;        /* pending requests before UGSDR_E_QUEUE_FULL (0 = 1024) */
	int policy;                /* ugsdr_serve_policy */
} ugsdr_server_config;

typedef struct ugsdr_server_stats {
	uint64_t submitted, completed, failed;
	int inflight;              /* jobs on the device now */
	int max_inflight_seen;     /* most jobs on the device at once so far */
	size_t device_bytes;       /* scratch the slots hold */
	double busy_seconds;       /* wall time with at least one job on the device */
} ugsdr_server_stats;

int ugsdr_server_create(ugsdr_ctx* ctx, const ugsdr_server_config* cfg, ugsdr_server** server);
/* Copies the job description (and the host samples) and returns a ticket;
 * UGSDR_E_QUEUE_FULL when queue_capacity requests are pending. */
int ugsdr_server_submit(ugsdr_server* server, const ugsdr_acq_job* job, uint64_t* ticket);
/* Tracking request: advances `bank` (created on the server's context) by
 * n_epochs epochs of host samples (samples_per_epoch = the bank's rate / 1000;
 * CF32, CI8, CI16 or RI8), copied at submit; n_epochs x n_channels outputs are
 * written to `outputs` (host, kept valid by the caller until the ticket is
 * polled done).  The bank's channels keep their loop and NCO state on the
 * device between requests, as Tracker::Track keeps its TrackingParameters
 * between epochs (src/tracking/tracker.hpp:186-197); a bank's requests run one
 * at a time in submission order, interleaved with acquisition jobs on the
 * other slots.  Poll the ticket with results = NULL. */
int ugsdr_server_submit_track(ugsdr_server* server, ugsdr_track_bank* bank, const void* samples, int sample_type,
	size_t samples_per_epoch, int n_epochs, ugsdr_track_output* outputs, uint64_t* ticket);
/* Non-blocking: *done = 1 and results[n_codes] filled when the job finished
 * (the ticket is then retired), 0 while pending; a failed job returns its
 * error status (UGSDR_E_NOMEM when its estimate exceeds the budget). */
int ugsdr_server_poll(ugsdr_server* server, uint64_t ticket, ugsdr_acq_result* results, int* done);
/* Blocks until every submitted job finished. */
int ugsdr_server_drain(ugsdr_server* server);
int ugsdr_server_get_stats(ugsdr_server* server, ugsdr_server_stats* stats);
int ugsdr_server_destroy(ugsdr_server* server);

#ifdef __cplusplus
}
#endif

#endif

// Acquisition -> tracking hand-off (ugsdr_track_refine).
//
// TrackingParameters::AddSignalImpl (src/tracking/tracking_parameters.hpp:
// 321-357) refines each acquired channel's code phase before tracking starts:
// the first three code periods are translated by -carrier_frequency
// (MatchedFilterTranslated, 297-318) and matched-filtered against the code,
// one period upsampled, zero-padded to three periods and rotated right by the
// code phase; |.| is folded to one period and the first maximum gives the
// offset (wrapped to +-period / 2).  The channel is kept, with code_phase +=
// offset, when the offset is within 1e-6 fs samples of a whole number of ms.
//
// Here every channel's matched filter is one row of the batched acquisition
// engine — a job of one code (the rotated replica, put as samples), one
// Doppler bin (0; the translation is the job's front-end frequency) and one
// block of three periods folded to one period — and all channels go in one
// batch on the device.
#include "internal.hpp"

#include <cmath>
#include <vector>

using namespace ugsdr_gpu;

extern "C" int ugsdr_track_refine(ugsdr_ctx* ctx, ugsdr_track_channel* channels, int n_channels, const float* codes,
	const int* code_lens, int n_codes, int code_len_max, const void* samples, int sample_type, int samples_on_device,
	size_t n_samples, int* accepted, int* offsets) {
	if (!ctx)
		return UGSDR_E_INVALID;
	std::vector<int> handles;
	auto release = [&] {
		for (int h : handles)
			ugsdr_code_release(ctx, h);
	};
	const int st = guarded(ctx, [&] {
		require(channels && n_channels > 0 && codes && code_lens && n_codes > 0 && code_len_max > 0 && samples && accepted,
			"null or empty hand-off description");
		std::vector<ugsdr_acq_job> jobs(n_channels);
		std::vector<size_t> period(n_channels), spm(n_channels);
		for (int c = 0; c < n_channels; ++c) {
			const ugsdr_track_channel& ch = channels[c];
			require(ch.code >= 0 && ch.code < n_codes, "channel code index out of range");
			const int len = code_lens[ch.code];
			require(len > 0 && len <= code_len_max && static_cast<double>(len) == ch.code_length, "code length mismatch");
			require(ch.sampling_rate > 0 && std::fmod(ch.sampling_rate, 1e3) == 0.0, "sampling rate must be a whole number of kHz");
			const double period_ms = ch.code_length / ch.code_frequency * 1000.0;
			require(std::fabs(period_ms - std::round(period_ms)) < 1e-9 && period_ms >= 1, "code period must be a whole number of ms");
			spm[c] = static_cast<size_t>(ch.sampling_rate / 1e3);
			period[c] = spm[c] * static_cast<size_t>(std::lround(period_ms));  // samples_period
			const size_t n = 3 * period[c];                                     // ms_cnt = 3 periods
			require(n_samples >= n, "fewer samples than three code periods");
			// SequentialUpsampler over one period, zero-padded to the epoch, rotated right by code_phase
			std::vector<float> replica(n, 0.0f);
			const float* chips = codes + static_cast<size_t>(ch.code) * code_len_max;
			for (size_t i = 0; i < period[c]; ++i)
				replica[i] = chips[(i * static_cast<size_t>(len) / period[c]) % static_cast<size_t>(len)];
			const long long shift = static_cast<long long>(ch.code_phase);  // static_cast<ptrdiff_t>(code_phase)
			const size_t r = static_cast<size_t>(((shift % static_cast<long long>(n)) + static_cast<long long>(n)) % static_cast<long long>(n));
			std::vector<float> rotated(n);
			for (size_t i = 0; i < n; ++i)
				rotated[(i + r) % n] = replica[i];
			int h = 0;
			const int ps = ugsdr_code_put(ctx, rotated.data(), n, 1, n, 0, 0, UGSDR_SPECTRUM_ONE_SIDED, &h);
			if (ps != UGSDR_OK)
				throw Error(ps, ctx->last_error);
			handles.push_back(h);
			ugsdr_acq_job& j = jobs[c];
			j.samples = samples;
			j.sample_type = sample_type;
			j.samples_on_device = samples_on_device;
			j.n_samples = n_samples;
			j.sampling_rate = ch.sampling_rate;
			j.frontend_frequency = -ch.carrier_frequency;  // Translate(epoch, fs, -carrier_frequency)
			j.code_offset_ratio = 1.0;
			j.block_samples = n;
			j.n_blocks = 1;
			j.fold_samples = period[c];  // ReshapeAndSum(Abs(...), batch_size)
			j.fold_coherent = 1;
			j.doppler_range = 0.0;        // a single bin at 0 Hz
			j.doppler_step = 1.0;
			j.codes = &handles.back();
			j.n_codes = 1;
			j.statistic = UGSDR_STAT_ABS;
			j.spectrum_mode = UGSDR_SPECTRUM_ONE_SIDED;
		}
		std::vector<ugsdr_acq_result> res(n_channels);
		std::vector<ugsdr_acq_result*> rp(n_channels);
		for (int c = 0; c < n_channels; ++c) {
			jobs[c].codes = &handles[c];
			rp[c] = &res[c];
		}
		const int as = ugsdr_acquire_batch(ctx, jobs.data(), n_channels, rp.data());
		if (as != UGSDR_OK)
			throw Error(as, ctx->last_error);
		for (int c = 0; c < n_channels; ++c) {
			const long long batch = static_cast<long long>(period[c]);
			long long offset = static_cast<long long>(res[c].index);
			if (offset > batch / 2)
				offset -= batch;
			long long mod = (offset + batch) % static_cast<long long>(spm[c]);
			if (mod > static_cast<long long>(spm[c]) / 2)
				mod -= static_cast<long long>(spm[c]);
			accepted[c] = std::fabs(static_cast<double>(mod)) < 1e-6 * channels[c].sampling_rate ? 1 : 0;
			if (offsets)
				offsets[c] = static_cast<int>(offset);
			if (accepted[c])
				channels[c].code_phase += static_cast<double>(offset);
		}
	});
	release();
	return st;
}

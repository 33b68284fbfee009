// ORACLE / TEST INFRASTRUCTURE ONLY.
//
// The reference's OWN tracking arithmetic, compiled into
// oracle/_ref/libugsdr_ref.so for the golden-vector generator
// (tests/golden/make_golden.py).  TrackingParameters comes from the build-time
// copy of src/tracking/tracking_parameters.hpp that oracle/patch_tracking.py
// writes (the non-IPP configuration alias fixed, nothing else), so these
// calls run the reference's code:
//   TableMixer carrier wipe-off with phase   src/mixer/mixer.hpp:33-42, table_mixer.hpp:78-101
//   TrackingParameters::UpdatePhase          tracking_parameters.hpp:163-165
//   TrackingParameters::CorrelateSplit       tracking_parameters.hpp:472-493 (AddWithPhase 89-98)
//   TrackingParameters::Pll / Dll            tracking_parameters.hpp:495-528 (constants 72-87)
//   SequentialMatchedFilter::Filter, SequentialAbs, SequentialReshapeAndSum
//   Observable's constructor and UpdatePseudoranges (measurements/
//   observable.hpp:55-88, 327-336; the build-time copy opens its access)
// Tracker::TrackSingleSatellite / GetEpl (src/tracking/tracker.hpp:119-177)
// and AddSignalImpl's surrounding steps (tracking_parameters.hpp:321-357) are
// private or need a DigitalFrontend, and MatchedFilterTranslated (297-319)
// calls the const Translate that TableMixer lacks without IPP, so their few
// lines of sequencing are restated below around those calls.
// the policies tracking_parameters.hpp names but leaves to its includers
#include "math/abs.hpp"
#include "math/reshape_and_sum.hpp"
#include "matched_filter/matched_filter.hpp"
#include "prn_codes/codegen_wrapper.hpp"
#include "resample/upsampler.hpp"
#include "patched/tracking/tracking_parameters.hpp"
#include "patched/measurements/observable.hpp"

#include <algorithm>
#include <complex>
#include <cstring>
#include <vector>

namespace {
	using Params = ugsdr::TrackingParameters<ugsdr::DefaultTrackingParametersConfig, float>;
	using ugsdr::Signal;

	Signal SignalOf(int id) { return static_cast<Signal>(id); }
}

extern "C" {

// The reference tracker on one channel for n_epochs epochs of spm complex
// float samples: per epoch TrackSingleSatellite (tracker.hpp:156-177) with
// GetEpl's E / P / L at +-0.25 chip (119-139).  full_code: the channel's code
// repeated three times and upsampled to 3 code periods (Codes::FillCodesImpl,
// tracker.hpp:40-50).  out: n_epochs x 12 doubles: E, P, L (re, im),
// carrier_frequency, carrier_phase (rad, unwrapped), code_phase,
// code_frequency, phase residual, code residual.
void ref_track_f32(const float* iq, std::size_t spm, int n_epochs, const float* full_code, std::size_t code_len,
	int signal, double fs, double base_code_frequency, double code_phase, double carrier_frequency, double* out) {
	Params p;
	p.sv.signal = SignalOf(signal);
	p.sampling_rate = fs;
	p.code_period = static_cast<double>(Params::GetCodePeriod(p.sv.signal));
	p.base_code_frequency = base_code_frequency;
	p.code_frequency = base_code_frequency;
	p.code_phase = code_phase;
	p.carrier_frequency = carrier_frequency;
	const std::vector<float> code(full_code, full_code + code_len);
	std::vector<std::complex<float>> translated(spm);
	for (int ep = 0; ep < n_epochs; ++ep) {
		std::memcpy(translated.data(), iq + 2 * static_cast<std::size_t>(ep) * spm, sizeof(float) * 2 * spm);
		const double ph = p.code_phase - p.sampling_rate / 1e3 * static_cast<double>(p.prompt.size() % p.GetCodePeriod());
		// GetEpl
		ugsdr::TableMixer::Translate(translated, p.sampling_rate, -p.carrier_frequency, -p.carrier_phase);
		p.UpdatePhase();
		const double spacing = p.GetSamplesPerChip() * 0.25;
		const auto e = p.CorrelateSplit(translated, code, ph + spacing);
		const auto pr = p.CorrelateSplit(translated, code, ph);
		const auto l = p.CorrelateSplit(translated, code, ph - spacing);
		p.early.push_back(e);
		p.prompt.push_back(pr);
		p.late.push_back(l);
		p.Pll(pr);
		p.Dll(e, l);
		double* o = out + 12 * static_cast<std::size_t>(ep);
		o[0] = e.real();
		o[1] = e.imag();
		o[2] = pr.real();
		o[3] = pr.imag();
		o[4] = l.real();
		o[5] = l.imag();
		o[6] = p.carrier_frequency;
		o[7] = p.carrier_phase;
		o[8] = p.code_phase;
		o[9] = p.code_frequency;
		o[10] = p.phase_residuals.back();
		o[11] = p.code_residuals.back();
	}
}

// One CorrelateSplit of the reference: the tap of `translated` (spm complex
// float samples) against full_code at code phase `phase` (samples).
void ref_correlate_split_f32(const float* translated, std::size_t spm, const float* full_code, std::size_t code_len,
	int signal, double fs, double phase, double* out) {
	Params p;
	p.sv.signal = SignalOf(signal);
	p.sampling_rate = fs;
	p.code_period = static_cast<double>(Params::GetCodePeriod(p.sv.signal));
	std::vector<std::complex<float>> x(spm);
	std::memcpy(x.data(), translated, sizeof(float) * 2 * spm);
	const std::vector<float> code(full_code, full_code + code_len);
	const auto v = p.CorrelateSplit(x, code, phase);
	out[0] = v.real();
	out[1] = v.imag();
}

// AddSignalImpl's refinement (tracking_parameters.hpp:321-357) for a GPS L1
// C/A (signal 0) or Galileo E1B (signal 6) channel: the first three code
// periods of `iq` (complex float at fs), the code of `sv` upsampled to one
// period, resized to three periods and rotated right by the acquisition's
// code phase; MatchedFilterTranslated at the carrier frequency; the offset
// rule.  out: code offset, accepted (0/1), refined code phase, |correlator|.
void ref_refine_f32(const float* iq, std::size_t n, int signal, int sv, double fs, double code_phase,
	double carrier_frequency, double* out) {
	Params p;
	p.sv.signal = SignalOf(signal);
	p.sampling_rate = fs;
	p.code_period = static_cast<double>(Params::GetCodePeriod(p.sv.signal));
	p.code_phase = code_phase;
	p.carrier_frequency = carrier_frequency;
	const auto samples_per_ms = static_cast<std::size_t>(fs / 1e3);
	const std::size_t ms = static_cast<std::size_t>(p.code_period);
	const std::size_t samples_period = samples_per_ms * ms;
	std::vector<std::complex<float>> epoch(3 * samples_period);
	std::memcpy(epoch.data(), iq, sizeof(float) * 2 * std::min(n, epoch.size()));
	std::vector<float> code;
	if (signal == static_cast<int>(Signal::Galileo_E1b))
		code = ugsdr::SequentialUpsampler::Transform(ugsdr::PrnGenerator<Signal::Galileo_E1b>::Get<float>(sv), samples_per_ms * ms);
	else
		code = ugsdr::SequentialUpsampler::Transform(ugsdr::PrnGenerator<Signal::GpsCoarseAcquisition_L1>::Get<float>(sv), samples_per_ms * ms);
	code.resize(epoch.size());
	std::rotate(code.rbegin(), code.rbegin() + static_cast<std::ptrdiff_t>(p.code_phase), code.rend());
	// MatchedFilterTranslated (tracking_parameters.hpp:297-319): translate a
	// copy in place, filter against the code, |.|, fold to one code period,
	// first maximum by magnitude, offset wrapped to +-period / 2
	auto translated = epoch;
	ugsdr::TableMixer::Translate(translated, p.sampling_rate, -p.carrier_frequency);
	const std::vector<float> local_code(code.begin(), code.begin() + translated.size());
	const auto batch_size = static_cast<std::size_t>(p.code_period * p.sampling_rate / 1e3);
	ugsdr::SequentialMatchedFilter::Filter(translated, local_code);
	const auto matched = ugsdr::SequentialReshapeAndSum::Transform(ugsdr::SequentialAbs::Transform(translated), batch_size);
	const auto it = std::max_element(matched.begin(), matched.end(), [](auto& lhs, auto& rhs) { return std::abs(lhs) < std::abs(rhs); });
	auto code_offset = static_cast<std::ptrdiff_t>(std::distance(matched.begin(), it));
	if (code_offset > static_cast<std::ptrdiff_t>(batch_size / 2))
		code_offset = code_offset - static_cast<std::ptrdiff_t>(batch_size);
	const float value = *it;
	auto mod = static_cast<std::ptrdiff_t>((code_offset + static_cast<std::ptrdiff_t>(samples_period)) % static_cast<std::ptrdiff_t>(samples_per_ms));
	if (mod > static_cast<std::ptrdiff_t>(samples_per_ms / 2))
		mod -= static_cast<std::ptrdiff_t>(samples_per_ms);
	const bool accepted = std::abs(static_cast<double>(mod)) < 1e-6 * fs;
	out[0] = static_cast<double>(code_offset);
	out[1] = accepted ? 1.0 : 0.0;
	out[2] = accepted ? p.code_phase + static_cast<double>(code_offset) : p.code_phase;
	out[3] = std::abs(value);
}

// The reference's Observable on one GPS L1 C/A channel's tracking history
// (what TrackingParameters holds after TrackSingleSatellite: prompt, phases =
// -carrier_phase / 2 pi as Pll pushes them (tracking_parameters.hpp:509),
// frequencies, code_phases): the constructor (observable.hpp:75-88) with
// CalculateSnr (55-72), then TimeScale::UpdateScale for a preamble at
// `position` and time of week tow_s (timescale.hpp:22-36) and
// UpdatePseudoranges (UpdatePseudorangeGps, observable.hpp:327-331).
// CalculateSnr keeps thread_local buffers sized by its first call, so every
// call of one process passes the same n.  out: n x 4 (pseudorange ms,
// pseudophase cycles, doppler Hz, snr).
void ref_observable_f64(const float* prompt_iq, const double* carrier_phase, const double* frequencies,
	const double* code_phases, std::size_t n, double fs, double intermediate_frequency, std::size_t position,
	std::size_t tow_s, double* out) {
	Params p;
	p.sv.system = ugsdr::System::Gps;
	p.sv.signal = Signal::GpsCoarseAcquisition_L1;
	p.sampling_rate = fs;
	p.intermediate_frequency = intermediate_frequency;
	for (std::size_t i = 0; i < n; ++i) {
		p.prompt.emplace_back(prompt_iq[2 * i], prompt_iq[2 * i + 1]);
		p.phases.push_back(-carrier_phase[i] / (2 * std::numbers::pi));
		p.frequencies.push_back(frequencies[i]);
		p.code_phases.push_back(code_phases[i]);
	}
	ugsdr::TimeScale time_scale(n);
	time_scale.UpdateScale(position, tow_s * 1000, ugsdr::System::Gps);
	ugsdr::GpsEphemeris eph;
	eph.tow = tow_s;
	ugsdr::Observable obs(p, time_scale, position, eph);
	obs.UpdatePseudoranges(0);
	for (std::size_t i = 0; i < n; ++i) {
		out[4 * i] = obs.pseudorange[i];
		out[4 * i + 1] = obs.pseudophase[i];
		out[4 * i + 2] = obs.doppler[i];
		out[4 * i + 3] = obs.snr[i];
	}
}
}

// ORACLE — FP64 CPU restatement of the tracking correlator bank.
// TEST INFRASTRUCTURE ONLY (tests/, smoke(), bench.py cpu_baseline).
//
// Follows the reference's per-epoch tracking step (the reference Tracker does
// not build without Intel IPP, so this is a restatement, checked by reading):
//   Tracker::TrackSingleSatellite / GetEpl   src/tracking/tracker.hpp:119-177
//   TrackingParameters::CorrelateSplit       tracking_parameters.hpp:472-493
//   AddWithPhase                             tracking_parameters.hpp:89-98
//   Pll / Dll and loop constants             tracking_parameters.hpp:72-87, 495-528
//   TableMixer carrier wipe-off              src/mixer/table_mixer.hpp:78-101
// with the bank's design choices: five taps (VE, E, P, L, VL) at configurable
// offsets, loop bandwidths as parameters, and the carrier phase held as a
// 64-bit fixed-point accumulator (cycles * 2^64) that also drives the mixer's
// 64-bit NCO (top 6 bits index the reference's 64-entry LUT).
// Taps accumulate in double; the mixed samples are formed in float exactly as
// the GPU forms them.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {
	constexpr double kPi = 3.14159265358979323846;
	constexpr double kTwo64 = 18446744073709551616.0;

	using cd = std::complex<double>;

	// AddWithPhase (tracking_parameters.hpp:89-98)
	cd add_with_phase(cd lhs, cd rhs, double rel) {
		if (rel < 0.5)
			std::swap(lhs, rhs);
		const double wl = lhs.real() / rel;
		const double wr = rhs.real() / (1.0 - rel);
		if (std::abs(wl + wr) > std::abs(wl))
			return lhs + rhs;
		return lhs - rhs;
	}

	uint64_t frac_to_fx(double cycles) {
		double f = cycles - std::floor(cycles);
		double v = f * kTwo64;
		if (v >= kTwo64)
			v = 0.0;
		return static_cast<uint64_t>(v);
	}
}

extern "C" {

// Open-loop correlator of ONE epoch: the five taps for the given NCO state
// at the start of the epoch (carrier frequency Hz, carrier phase rad, code
// phase of this epoch in samples), same arithmetic as orc_track_f64's epoch.
// out: 10 doubles (VE, E, P, L, VL re/im) + 5 minor partial magnitudes.
void orc_track_taps_f64(const float* iq, size_t spm, const float* chips, int len, double fs, double base, double code_len,
	double ph, double carrier_freq, double carrier_phase, double el, double vel, double* out) {
	constexpr double kTwo64l = 18446744073709551616.0;
	float table[80];
	const double step = 5 * kPi / 80 / 2;
	for (int i = 0; i < 80; ++i)
		table[i] = static_cast<float>(std::sin(static_cast<double>(i) * step));
	const int period_ms = static_cast<int>(std::lround(code_len / base * 1000.0));
	const size_t samples_per_ms = static_cast<size_t>(fs / 1e3);
	const double period = static_cast<double>(samples_per_ms) * period_ms;
	const uint64_t L3 = 3ull * static_cast<uint64_t>(len);
	const uint64_t S3 = static_cast<uint64_t>(3 * period_ms * fs / 1e3);
	const double spc = fs / base;
	const double offsets[5] = {vel, el, 0.0, -el, -vel};
	const uint64_t phase_fx = frac_to_fx(carrier_phase / (2 * kPi));
	double f = -carrier_freq;
	const bool mix = std::abs(f) != 0.0;
	if (f < 0)
		f = fs + f;
	double av = kTwo64l * f / fs;
	if (av >= kTwo64l)
		av = 0.0;
	const uint64_t adder = static_cast<uint64_t>(av);
	const uint64_t holder0 = 0ull - phase_fx;
	std::vector<cd> mixed(spm);
	for (size_t i = 0; i < spm; ++i) {
		const float a = iq[2 * i], b = iq[2 * i + 1];
		if (!mix) {
			mixed[i] = cd(a, b);
			continue;
		}
		const uint32_t idx = static_cast<uint32_t>((holder0 + static_cast<uint64_t>(i) * adder) >> 58);
		const float c = table[idx + 16], s = table[idx];
		const volatile float re1 = a * c, re2 = b * s, im1 = a * s, im2 = b * c;
		mixed[i] = cd(re1 - re2, im1 + im2);
	}
	for (int t = 0; t < 5; ++t) {
		double p = ph + spc * offsets[t];
		while (p < 0)
			p += period;
		if (p > period)
			p = std::fmod(p, period);
		const size_t first_len = static_cast<size_t>(std::ceil(p)) % samples_per_ms;
		const uint64_t first_phase = static_cast<uint64_t>(std::ceil(2 * period - p));
		cd A(0, 0), B(0, 0);
		for (size_t i = 0; i < spm; ++i) {
			const float cv = chips[(((first_phase + i) * L3) / S3 % L3) % static_cast<uint64_t>(len)];
			if (i < first_len)
				A += mixed[i] * static_cast<double>(cv);
			else
				B += mixed[i] * static_cast<double>(cv);
		}
		const cd tap = add_with_phase(A, B, std::fmod(p, static_cast<double>(samples_per_ms)) / samples_per_ms);
		out[2 * t] = tap.real();
		out[2 * t + 1] = tap.imag();
		out[10 + t] = std::min(std::abs(A), std::abs(B));
	}
}

// One channel over n_epochs epochs of spm samples (complex float I/Q).
// cfg: [el_offset, vel_offset, pll_bw, dll_bw, fll_bw, T]
// ch:  [fs, code_frequency, code_length, code_phase, carrier_frequency, carrier_phase]
// out: n_epochs x 21 doubles: VE, E, P, L, VL (re, im) x 5, carrier_frequency,
//      carrier_phase (rad, [0, 2pi)), code_phase, code_frequency, phase_error, code_error,
//      then per tap the magnitude of the smaller CorrelateSplit partial sum
void orc_track_f64(const float* iq, size_t spm, int n_epochs, const float* chips, int len, const double* cfg,
	const double* ch, double* out) {
	const double el = cfg[0], vel = cfg[1], pll_bw = cfg[2], dll_bw = cfg[3], fll_bw = cfg[4], T = cfg[5];
	const double fs = ch[0], base = ch[1], code_len = ch[2];
	double code_phase = ch[3], carrier_freq = ch[4];
	uint64_t phase_fx = frac_to_fx(ch[5] / (2 * kPi));

	// loop constants (tracking_parameters.hpp:72-87) with the bandwidths as parameters
	const double K1_PLL = T * (pll_bw / 0.53 * (pll_bw / 0.53)) + 1.414 * (pll_bw / 0.53);
	const double K2_PLL = 1.414 * (pll_bw / 0.53);
	const double K3_PLL = T * (fll_bw / 0.25);
	const double zeta = 1.0, gain = 0.1;
	const double WN = dll_bw * 8.0 * zeta / (4.0 * zeta * zeta + 1.0);
	const double TAU1 = gain / (WN * WN), TAU2 = 2.0 * zeta / WN;
	const double K1_DLL = TAU2 / TAU1, K2_DLL = T / TAU1;

	float table[80];
	const double step = 5 * kPi / 80 / 2;
	for (int i = 0; i < 80; ++i)
		table[i] = static_cast<float>(std::sin(static_cast<double>(i) * step));

	const int period_ms = static_cast<int>(std::lround(code_len / base * 1000.0));
	const size_t samples_per_ms = static_cast<size_t>(fs / 1e3);
	const double period = static_cast<double>(samples_per_ms) * period_ms;
	const uint64_t L3 = 3ull * static_cast<uint64_t>(len);
	const uint64_t S3 = static_cast<uint64_t>(3 * period_ms * fs / 1e3);
	const double spc = fs / base;
	const double offsets[5] = {vel, el, 0.0, -el, -vel};

	double carrier_phase_error = 0.0, code_nco = 0.0, code_error = 0.0, code_freq = base;
	cd prev_prompt(0.0, 0.0);
	std::vector<cd> mixed(spm);
	for (int ep = 0; ep < n_epochs; ++ep) {
		const float* x = iq + 2 * static_cast<size_t>(ep) * spm;
		// GetEpl: Translate(signal, fs, -carrier_frequency, -carrier_phase)
		double f = -carrier_freq;
		const bool mix = std::abs(f) != 0.0;
		if (f < 0)
			f = fs + f;
		double av = kTwo64 * f / fs;
		if (av >= kTwo64)
			av = 0.0;
		const uint64_t adder = static_cast<uint64_t>(av);
		const uint64_t holder0 = 0ull - phase_fx;
		for (size_t i = 0; i < spm; ++i) {
			const float a = x[2 * i], b = x[2 * i + 1];
			if (!mix) {
				mixed[i] = cd(a, b);
				continue;
			}
			const uint32_t idx = static_cast<uint32_t>((holder0 + static_cast<uint64_t>(i) * adder) >> 58);
			const float c = table[idx + 16], s = table[idx];
			const volatile float re1 = a * c, re2 = b * s, im1 = a * s, im2 = b * c;
			const float re = re1 - re2, im = im1 + im2;
			mixed[i] = cd(re, im);
		}
		// UpdatePhase (tracking_parameters.hpp:163-165) with the pre-update frequency
		phase_fx += frac_to_fx(carrier_freq / 1000.0);

		// taps (tracker.hpp:169-137: code phase of this epoch, offsets in samples per chip)
		const double ph = code_phase - fs / 1e3 * static_cast<double>(ep % period_ms);
		cd taps[5];
		double minor[5];
		for (int t = 0; t < 5; ++t) {
			double p = ph + spc * offsets[t];
			while (p < 0)
				p += period;
			if (p > period)
				p = std::fmod(p, period);
			const size_t first_len = static_cast<size_t>(std::ceil(p)) % samples_per_ms;
			const uint64_t first_phase = static_cast<uint64_t>(std::ceil(2 * period - p));
			cd A(0, 0), B(0, 0);
			for (size_t i = 0; i < spm; ++i) {
				const uint64_t q = first_phase + i;
				const float cv = chips[((q * L3) / S3 % L3) % static_cast<uint64_t>(len)];
				if (i < first_len)
					A += mixed[i] * static_cast<double>(cv);
				else
					B += mixed[i] * static_cast<double>(cv);
			}
			const double rel = std::fmod(p, static_cast<double>(samples_per_ms)) / samples_per_ms;
			taps[t] = add_with_phase(A, B, rel);
			// AddWithPhase chooses lhs +/- rhs by a comparison that is a near-tie when
			// one partial sum is tiny; report that partial so a checker can allow
			// the sign choice to differ under different rounding
			minor[t] = std::min(std::abs(A), std::abs(B));
		}

		// the reference's taps are std::complex<float> (tracker.hpp:128-137)
		for (auto& t : taps)
			t = cd(static_cast<float>(t.real()), static_cast<float>(t.imag()));
		// Pll(prompt) (tracking_parameters.hpp:495-511), in the reference's types:
		// the prompt is std::complex<float>, so imag/real, cross and dot are float
		// products (not contracted) and std::atan2 takes the float overload; atan
		// of the float ratio and the loop filter are double.
		const float pr = static_cast<float>(taps[2].real()), pi = static_cast<float>(taps[2].imag());
		const float ppr = static_cast<float>(prev_prompt.real()), ppi = static_cast<float>(prev_prompt.imag());
		const volatile float ratio = pi / pr;
		const double err = pr != 0.0f ? std::atan(static_cast<double>(ratio)) / (kPi * 2.0) : 0.0;
		const volatile float c1 = pr * ppi, c2 = ppr * pi, d1 = pr * ppr, d2 = ppi * pi;
		const float cross = c1 - c2;
		const float dot = std::abs(d1 + d2);
		const double ferr = std::atan2(cross, dot) / kPi;
		carrier_freq += K1_PLL * err - K2_PLL * carrier_phase_error - K3_PLL * ferr;
		carrier_phase_error = err;
		// carrier_phase += err * pi / 2 rad = err / 4 cycles; |err| <= 1/4 keeps it below 2^60
		phase_fx += static_cast<uint64_t>(std::llround(err / 4.0 * kTwo64));
		prev_prompt = cd(pr, pi);

		// Dll(early, late) (tracking_parameters.hpp:513-528): std::abs of
		// complex<float> and the normalised difference in float
		const float ea = std::abs(std::complex<float>(static_cast<float>(taps[1].real()), static_cast<float>(taps[1].imag())));
		const float la = std::abs(std::complex<float>(static_cast<float>(taps[3].real()), static_cast<float>(taps[3].imag())));
		double ce = 0.0;
		if (ea + la != 0)
			ce = (ea - la) / (ea + la);
		code_nco += (K1_DLL * (ce - code_error) + K2_DLL * ce) * (base / 1.023e6);
		code_error = ce;
		code_freq = base - code_nco;
		code_phase -= fs / 1000 / 2 * (code_freq / base - 1);

		double* o = out + 21 * static_cast<size_t>(ep);
		for (int t = 0; t < 5; ++t)
			o[16 + t] = minor[t];
		for (int t = 0; t < 5; ++t) {
			o[2 * t] = taps[t].real();
			o[2 * t + 1] = taps[t].imag();
		}
		o[10] = carrier_freq;
		o[11] = static_cast<double>(phase_fx) / kTwo64 * 2 * kPi;
		o[12] = code_phase;
		o[13] = code_freq;
		o[14] = err;
		o[15] = ce;
	}
}
}

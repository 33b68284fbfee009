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
// offsets and loop bandwidths as parameters.  Two carrier NCO modes, as the
// bank has them:
//   0  the carrier phase held as a 64-bit fixed-point accumulator
//      (cycles * 2^64) that also drives the mixer's 64-bit NCO (top 6 bits
//      index the reference's 64-entry LUT);
//   1  the reference's: the phase in double radians, advanced by
//      UpdatePhase (2 pi f / 1000) and Pll (err pi / 2), and each epoch's
//      wipe-off a fresh TableMixer NCO (Mixer::Translate, mixer.hpp:33-42:
//      phase reduced to [0, 2 pi), 32-bit holder 2^32 phase / 2 pi, 32-bit
//      adder 2^32 f / fs, nco.hpp:17-20).
// Taps accumulate in double; the mixed samples are formed in float exactly as
// the GPU forms them.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <utility>
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

	// Loop state between epochs and the loop constants
	// (tracking_parameters.hpp:72-87 with the bandwidths as parameters).
	struct LoopState {
		double carrier_freq, phase_rad, carrier_phase_error, code_nco, code_error, code_freq, code_phase;
		float prev_re, prev_im;
		uint64_t phase_fx;
	};
	struct LoopConst {
		double K1_PLL, K2_PLL, K3_PLL, K1_DLL, K2_DLL, base, fs;
		LoopConst(double pll_bw, double dll_bw, double fll_bw, double T, double base_, double fs_) : base(base_), fs(fs_) {
			K1_PLL = T * (pll_bw / 0.53 * (pll_bw / 0.53)) + 1.414 * (pll_bw / 0.53);
			K2_PLL = 1.414 * (pll_bw / 0.53);
			K3_PLL = T * (fll_bw / 0.25);
			const double zeta = 1.0, gain = 0.1;
			const double WN = dll_bw * 8.0 * zeta / (4.0 * zeta * zeta + 1.0);
			const double TAU1 = gain / (WN * WN), TAU2 = 2.0 * zeta / WN;
			K1_DLL = TAU2 / TAU1;
			K2_DLL = T / TAU1;
		}
	};

	// Pll(prompt) then Dll(early, late) (tracking_parameters.hpp:495-528) on
	// the epoch's float taps, in the reference's types: the prompt is
	// std::complex<float>, so imag/real, cross and dot are float products (not
	// contracted) and std::atan2 takes the float overload; atan of the float
	// ratio and the loop filters are double; |E|, |L| are std::abs of
	// complex<float>.  Returns (phase_error, code_error).
	std::pair<double, double> loop_update(LoopState& s, const LoopConst& k, std::complex<float> e, std::complex<float> p,
		std::complex<float> l) {
		const float pr = p.real(), pi = p.imag();
		const float ppr = s.prev_re, ppi = s.prev_im;
		const volatile float ratio = pi / pr;
		const double err = pr != 0.0f ? std::atan(static_cast<double>(ratio)) / (kPi * 2.0) : 0.0;
		const volatile float c1 = pr * ppi, c2 = ppr * pi, d1 = pr * ppr, d2 = ppi * pi;
		const float cross = c1 - c2;
		const float dot = std::abs(d1 + d2);
		const double ferr = std::atan2(cross, dot) / kPi;
		s.carrier_freq += k.K1_PLL * err - k.K2_PLL * s.carrier_phase_error - k.K3_PLL * ferr;
		s.carrier_phase_error = err;
		// carrier_phase += err * pi / 2 rad = err / 4 cycles; |err| <= 1/4 keeps it below 2^60
		s.phase_fx += static_cast<uint64_t>(std::llround(err / 4.0 * kTwo64));
		{
			const volatile double adv = err * kPi / 2;
			s.phase_rad += adv;
		}
		s.prev_re = pr;
		s.prev_im = pi;
		const float ea = std::abs(e);
		const float la = std::abs(l);
		double ce = 0.0;
		if (ea + la != 0)
			ce = (ea - la) / (ea + la);
		s.code_nco += (k.K1_DLL * (ce - s.code_error) + k.K2_DLL * ce) * (k.base / 1.023e6);
		s.code_error = ce;
		s.code_freq = k.base - s.code_nco;
		s.code_phase -= k.fs / 1000 / 2 * (s.code_freq / k.base - 1);
		return {err, ce};
	}

	// The epoch's carrier wipe-off: mixed[i] = x[i] * LUT(NCO), LUT index the
	// top 6 bits of holder0 + i * adder (64-bit; mode 1 keeps the reference's
	// 32-bit NCO in the upper half, so the index and the wrap are its own).
	// Returns false when the frequency is 0 (Translate does not mix then).
	bool carrier_nco(int mode, double fs, double carrier_freq, uint64_t phase_fx, double phase_rad, uint64_t& holder0,
		uint64_t& adder) {
		double f = -carrier_freq;
		if (std::abs(f) == 0.0)
			return false;
		if (f < 0)
			f = fs + f;
		if (mode == 1) {
			double ph = std::fmod(-phase_rad, 2 * kPi);  // Mixer::FixPhase
			if (ph < 0)
				ph += 2 * kPi;
			const uint64_t a32 = static_cast<uint64_t>(4294967296.0 * f / fs);
			const uint64_t h32 = static_cast<uint64_t>(4294967296.0 * ph / (2 * kPi)) & 0xFFFFFFFFull;
			adder = a32 << 32;
			holder0 = h32 << 32;
			return true;
		}
		double av = kTwo64 * f / fs;
		if (av >= kTwo64)
			av = 0.0;
		adder = static_cast<uint64_t>(av);
		holder0 = 0ull - phase_fx;
		return true;
	}
}

extern "C" {

// Open-loop correlator of ONE epoch: the five taps for the given NCO state
// at the start of the epoch (carrier frequency Hz, carrier phase rad, code
// phase of this epoch in samples), same arithmetic as orc_track_f64's epoch.
// out: 10 doubles (VE, E, P, L, VL re/im) + 5 minor partial magnitudes.
void orc_track_taps_f64(const float* iq, size_t spm, const float* chips, int len, double fs, double base, double code_len,
	double ph, double carrier_freq, double carrier_phase, double el, double vel, int nco_mode, double* out) {
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
	(void)kTwo64l;
	uint64_t holder0 = 0, adder = 0;
	const bool mix = carrier_nco(nco_mode, fs, carrier_freq, frac_to_fx(carrier_phase / (2 * kPi)), carrier_phase, holder0, adder);
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

// The loop update alone, epoch after epoch, on given taps: for each epoch the
// E, P, L taps (re, im; float values) -> the state after Pll and Dll.
// cfg: [pll_bw, dll_bw, fll_bw, T, fs, code_frequency]; init: [carrier_frequency,
// carrier_phase (rad), code_phase].  out: n x 6 doubles: carrier_frequency,
// carrier_phase (rad), code_phase, code_frequency, phase_error, code_error.
void orc_track_loop_f64(const double* taps, int n, const double* cfg, const double* init, double* out) {
	const LoopConst k(cfg[0], cfg[1], cfg[2], cfg[3], cfg[5], cfg[4]);
	LoopState s{init[0], init[1], 0.0, 0.0, 0.0, cfg[5], init[2], 0.0f, 0.0f, 0};
	for (int e = 0; e < n; ++e) {
		const double* t = taps + 6 * static_cast<size_t>(e);
		// UpdatePhase runs in GetEpl before the taps, with the pre-update frequency
		{
			const volatile double adv = 2 * kPi * s.carrier_freq / 1000.0;
			s.phase_rad += adv;
		}
		const auto f = [](double re, double im) { return std::complex<float>(static_cast<float>(re), static_cast<float>(im)); };
		const auto [err, ce] = loop_update(s, k, f(t[0], t[1]), f(t[2], t[3]), f(t[4], t[5]));
		double* o = out + 6 * static_cast<size_t>(e);
		o[0] = s.carrier_freq;
		o[1] = s.phase_rad;
		o[2] = s.code_phase;
		o[3] = s.code_freq;
		o[4] = err;
		o[5] = ce;
	}
}

// One channel over n_epochs epochs of spm samples (complex float I/Q).
// cfg: [el_offset, vel_offset, pll_bw, dll_bw, fll_bw, T, nco_mode]
// ch:  [fs, code_frequency, code_length, code_phase, carrier_frequency, carrier_phase]
// out: n_epochs x 21 doubles: VE, E, P, L, VL (re, im) x 5, carrier_frequency,
//      carrier_phase (rad, [0, 2pi)), code_phase, code_frequency, phase_error, code_error,
//      then per tap the magnitude of the smaller CorrelateSplit partial sum
void orc_track_f64(const float* iq, size_t spm, int n_epochs, const float* chips, int len, const double* cfg,
	const double* ch, double* out) {
	const double el = cfg[0], vel = cfg[1], pll_bw = cfg[2], dll_bw = cfg[3], fll_bw = cfg[4], T = cfg[5];
	const int nco_mode = static_cast<int>(cfg[6]);
	const double fs = ch[0], base = ch[1], code_len = ch[2];
	double code_phase = ch[3], carrier_freq = ch[4];
	uint64_t phase_fx = frac_to_fx(ch[5] / (2 * kPi));
	double phase_rad = ch[5];  // nco_mode 1

	const LoopConst k(pll_bw, dll_bw, fll_bw, T, base, fs);

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
		uint64_t holder0 = 0, adder = 0;
		const bool mix = carrier_nco(nco_mode, fs, carrier_freq, phase_fx, phase_rad, holder0, adder);
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
		{
			const volatile double adv = 2 * kPi * carrier_freq / 1000.0;
			phase_rad += adv;
		}

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
		LoopState ls{carrier_freq, phase_rad, carrier_phase_error, code_nco, code_error, code_freq, code_phase,
			static_cast<float>(prev_prompt.real()), static_cast<float>(prev_prompt.imag()), phase_fx};
		const auto fc = [](cd v) { return std::complex<float>(static_cast<float>(v.real()), static_cast<float>(v.imag())); };
		const auto [err, ce] = loop_update(ls, k, fc(taps[1]), fc(taps[2]), fc(taps[3]));
		carrier_freq = ls.carrier_freq;
		phase_rad = ls.phase_rad;
		carrier_phase_error = ls.carrier_phase_error;
		code_nco = ls.code_nco;
		code_error = ls.code_error;
		code_freq = ls.code_freq;
		code_phase = ls.code_phase;
		phase_fx = ls.phase_fx;
		prev_prompt = cd(ls.prev_re, ls.prev_im);

		double* o = out + 21 * static_cast<size_t>(ep);
		for (int t = 0; t < 5; ++t)
			o[16 + t] = minor[t];
		for (int t = 0; t < 5; ++t) {
			o[2 * t] = taps[t].real();
			o[2 * t + 1] = taps[t].imag();
		}
		o[10] = carrier_freq;
		o[11] = nco_mode == 1 ? phase_rad : static_cast<double>(phase_fx) / kTwo64 * 2 * kPi;
		o[12] = code_phase;
		o[13] = code_freq;
		o[14] = err;
		o[15] = ce;
	}
}
}

// ORACLE / TEST INFRASTRUCTURE ONLY — never linked into the product library.
//
// CPU restatement of the reference's observable generation
// (src/measurements/observable.hpp) from one tracking channel's history:
//   - the preamble candidate search of FindPreambleGps / FindPreambleGlonass
//     (observable.hpp:204-220, 260-277): navigation symbols sign(prompt I),
//     matched-filtered against the upsampled preamble the reference's way
//     (SequentialMatchedFilter::Filter, matched_filter/matched_filter.hpp:
//     64-68: forward DFTs, product with the conjugate preamble spectrum,
//     inverse DFT times 2 / N, src/math/dft.hpp:124-129), |.| above 153 /
//     370;
//   - the Observable constructor (observable.hpp:75-88) with CalculateSnr
//     (55-72) and the i-independent UpdatePseudorange term (327-336).
// Pinned: the candidate search (against the reference's own upsampler,
// matched filter and abs, tests/golden/preamble.npz), and the constructor's
// pseudorange / pseudophase / Doppler / SNR with UpdatePseudoranges, bit for
// bit (SNR within 1e-12) against the reference's own Observable run on its
// own tracker's histories (tests/golden/observables.npz; the harness
// compiles a build-time copy of observable.hpp whose only change opens the
// constructor's access, oracle/patch_tracking.py).
#include "fft64.hpp"

#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <vector>

namespace oracle {
	namespace {
		constexpr double kPi = 3.14159265358979323846;

		// GetPreambleGps (observable.hpp:90-98) and GetPreambleGlonass
		// (141-151): symbols upsampled by SequentialUpsampler (dst[i] =
		// src[i * L / S]), resized to the prompt's length
		std::vector<double> Preamble(int message, std::size_t size) {
			static const int gps[8] = {1, -1, -1, -1, 1, -1, 1, 1};
			static const int glo[40] = {-1, -1, -1, -1, -1, 1, 1, 1, -1, -1, 1, -1, -1, -1, 1, -1, 1, -1, 1, 1,
				1, 1, -1, 1, 1, -1, 1, -1, -1, 1, 1, -1, 1, -1, 1, -1, 1, -1, -1, 1};
			const int* sym = message == 1 ? glo : gps;
			const std::size_t n_sym = message == 1 ? 40 : 8, up = message == 1 ? 10 : 20;
			std::vector<double> p(n_sym * up);
			for (std::size_t i = 0; i < p.size(); ++i)
				p[i] = sym[i * n_sym / p.size()];
			p.resize(size, 0.0);
			return p;
		}
	}
}

extern "C" {

// counts and lists (ascending) the epochs where |matched filter| exceeds the
// message's threshold; returns the count, writes the first `cap` indexes
int orc_preamble_search(const float* prompt_i, std::size_t n, int message, int* indexes, int cap) {
	using oracle::cd;
	std::vector<cd> x(n), X(n), P(n), y(n);
	for (std::size_t i = 0; i < n; ++i)
		x[i] = cd(prompt_i[i] > 0 ? 1.0 : -1.0, 0.0);
	const auto p = oracle::Preamble(message, n);
	std::vector<cd> pc(p.begin(), p.end());
	oracle::Fft64 fwd(n, -1), inv(n, +1);
	fwd.Execute(x.data(), X.data());
	fwd.Execute(pc.data(), P.data());
	for (std::size_t k = 0; k < n; ++k)
		X[k] *= std::conj(P[k]);
	inv.Execute(X.data(), y.data());
	const double threshold = message == 1 ? 370.0 : 153.0;
	int count = 0;
	for (std::size_t k = 0; k < n; ++k) {
		if (std::abs(y[k] / static_cast<double>(n) * 2.0) > threshold) {
			if (count < cap)
				indexes[count] = static_cast<int>(k);
			++count;
		}
	}
	return count;
}

// One channel: the tracking history as the reference's TrackingParameters
// holds it (prompt I/Q, frequencies, code_phases) plus the PLL's
// phase_residuals, from which the reference's unwrapped carrier_phase is
// re-accumulated the reference's way in radians (UpdatePhase, tracking_
// parameters.hpp:163-165, then Pll's += error * pi / 2, 505-509).
// out: n x 4 (pseudorange ms, pseudophase cycles, doppler Hz, snr dB-Hz).
void orc_observables_f64(const float* prompt_i, const float* prompt_q, const double* frequencies,
	const double* phase_errors, const double* code_phases, std::size_t n, double sampling_rate,
	double intermediate_frequency, double carrier_frequency0, double carrier_phase0, std::size_t position,
	double correction, double* out) {
	// CalculateSnr: SequentialMeanStdDev over the prompt Q in float
	float sigma = 0.f;
	if (n >= 2) {
		float q = 0.f, m = 0.f;
		for (std::size_t i = 0; i < n; ++i) {
			q += prompt_q[i] * prompt_q[i];
			m += prompt_q[i];
		}
		const float var = (q - m * m / static_cast<float>(n)) / static_cast<float>(n - 1);
		sigma = std::sqrt(var);
	}
	const double samples_to_ms_rate = 1000 / sampling_rate;
	const auto pseudorange_offset = static_cast<std::int32_t>(code_phases[position] * samples_to_ms_rate);
	const double windup = intermediate_frequency / 1e3;
	double carrier_phase = carrier_phase0, f = carrier_frequency0;
	for (std::size_t i = 0; i < n; ++i) {
		carrier_phase += 2 * oracle::kPi * f / 1000.0;
		carrier_phase += phase_errors[i] * oracle::kPi / 2;
		f = frequencies[i];
		const double phase = -carrier_phase / (2 * oracle::kPi);
		double* o = out + 4 * i;
		o[0] = code_phases[i] * samples_to_ms_rate - pseudorange_offset + correction;
		o[1] = phase + static_cast<double>(i + 1) * windup;
		o[2] = frequencies[i] - intermediate_frequency;
		o[3] = 27 + 20 * std::log10(std::abs(prompt_i[i]) / sigma);
	}
}
}

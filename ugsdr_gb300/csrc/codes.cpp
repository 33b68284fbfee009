// PRN code generation and small host helpers shared by the engine.
//
// Own implementation of the ICD generators the reference builds from LFSR
// objects (src/prn_codes/lfsr.hpp:93-114):
//   GPS L1 C/A  Gold code G1 xor G2 delayed by the per-PRN G2 delay
//               (GoldCodes.hpp:25-41, GpsL1Ca.hpp:9-21; IS-GPS-200 table 3-Ia)
//   GPS L5I/Q   XA (short-cycled at 8190 chips) xor XB advanced per PRN
//               (L5.hpp:25-43, GpsL5I.hpp:9-21, GpsL5Q.hpp:9-21; IS-GPS-705 table 3-1)
//   GLONASS     511-chip m-sequence x^9 + x^5 + 1, output of stage 7 (GlonassOf.hpp:25-36)
//   Galileo E1B/E1C  memory codes (Galileo OS SIS ICD tables, the reference's
//               GalileoMemoryCodes.cpp) embedded from data/, BOC(1,1) expanded
// The delay/advance tables and memory codes are ICD data and therefore
// identical to the reference's.  Chips are +-1 with bit b -> 1 - 2b, as the reference emits.
#include "internal.hpp"

#include <array>
#include <cmath>
#include <cstring>

extern const unsigned char ugsdr_galileo_e1_table[51200];

namespace ugsdr_gpu {
	namespace {
		// Fibonacci LFSR over `stages` cells (cell 1 newest .. cell `stages` oldest):
		// returns the output cell `out_cell` for `len` clocks.  Taps are 1-based cells.
		std::vector<uint8_t> lfsr_sequence(int stages, std::initializer_list<int> taps, int out_cell, int len,
			uint32_t init = 0xFFFFFFFFu, int reset_period = 0) {
			std::vector<uint8_t> cell(stages + 1);
			for (int i = 1; i <= stages; ++i)
				cell[i] = (init >> (i - 1)) & 1u;
			const std::vector<uint8_t> start = cell;
			std::vector<uint8_t> seq(len);
			for (int t = 0; t < len; ++t) {
				seq[t] = cell[out_cell];
				if (reset_period && (t + 1) % reset_period == 0) {
					cell = start;
					continue;
				}
				uint8_t fb = 0;
				for (int tap : taps)
					fb ^= cell[tap];
				for (int i = stages; i > 1; --i)
					cell[i] = cell[i - 1];
				cell[1] = fb;
			}
			return seq;
		}

		// IS-GPS-200 G2 delays (chips) for PRN 1..37
		constexpr std::array<int, 37> kCaG2Delay = {
			5, 6, 7, 8, 17, 18, 139, 140, 141, 251, 252, 254, 255, 256, 257, 258, 469, 470, 471,
			472, 473, 474, 509, 512, 513, 514, 515, 516, 859, 860, 861, 862, 863, 950, 947, 948, 950};

		// IS-GPS-705 XB code advance (chips), PRN 1..32
		constexpr std::array<int, 32> kL5IAdvance = {
			266, 365, 804, 1138, 1509, 1559, 1756, 2084, 2170, 2303, 2527, 2687, 2930, 3471, 3940, 4132,
			4332, 4924, 5343, 5443, 5641, 5816, 5898, 5918, 5955, 6243, 6345, 6477, 6518, 6875, 7168, 7187};
		constexpr std::array<int, 32> kL5QAdvance = {
			1701, 323, 5292, 2020, 5429, 7136, 1041, 5947, 4315, 148, 535, 1939, 5206, 5910, 3595, 5135,
			6082, 6990, 3546, 1523, 4548, 4484, 1893, 3961, 7106, 5299, 4660, 276, 4389, 3783, 1591, 1601};

		void write_chips(const std::vector<uint8_t>& bits, float* out) {
			for (size_t i = 0; i < bits.size(); ++i)
				out[i] = 1.0f - 2.0f * static_cast<float>(bits[i]);
		}

		void gps_ca(int sv, float* out) {
			static const std::vector<uint8_t> g1 = lfsr_sequence(10, {3, 10}, 10, 1023);
			static const std::vector<uint8_t> g2 = lfsr_sequence(10, {2, 3, 6, 8, 9, 10}, 10, 1023);
			const int delay = kCaG2Delay[sv];
			std::vector<uint8_t> c(1023);
			for (int i = 0; i < 1023; ++i)
				c[i] = g1[i] ^ g2[(i - delay + 1023) % 1023];
			write_chips(c, out);
		}

		void gps_l5(int sv, bool quadrature, float* out) {
			// XA: x^13 + x^12 + x^10 + x^9 + 1, reset to all ones every 8190 chips
			static const std::vector<uint8_t> xa = lfsr_sequence(13, {9, 10, 12, 13}, 13, 10230, 0x1FFF, 8190);
			// XB: x^13 + x^12 + x^8 + x^7 + x^6 + x^4 + x^3 + x + 1 (period 8191)
			static const std::vector<uint8_t> xb = lfsr_sequence(13, {1, 3, 4, 6, 7, 8, 12, 13}, 13, 8191, 0x1FFF);
			const int adv = quadrature ? kL5QAdvance[sv] : kL5IAdvance[sv];
			std::vector<uint8_t> c(10230);
			for (int i = 0; i < 10230; ++i)
				c[i] = xa[i] ^ xb[(i + adv) % 8191];
			write_chips(c, out);
		}

		// Galileo E1B / E1C: the ICD's memory codes (table data, embedded from
		// data/galileo_e1_memory_codes.bin: 4,092 chips per code, bit 1 = -1)
		// as sine-BOC(1,1) half-chips [c, -c] per chip, the form
		// MemoryCodes::DecodeBoc returns (src/prn_codes/MemoryCodes.hpp:33-40).
		void galileo_e1(int sv, bool pilot, float* out) {
			const unsigned char* code = ugsdr_galileo_e1_table + (pilot ? 50 : 0) * 512 + static_cast<size_t>(sv) * 512;
			for (int i = 0; i < 4092; ++i) {
				const float c = ((code[i >> 3] >> (7 - (i & 7))) & 1) ? -1.0f : 1.0f;
				out[2 * i] = c;
				out[2 * i + 1] = -c;
			}
		}

		void glonass_of(float* out) {
			static const std::vector<uint8_t> m = lfsr_sequence(9, {5, 9}, 7, 511);
			write_chips(m, out);
		}
	}

	int prn_code(int signal, int sv, float* out, size_t cap, size_t* len) {
		size_t n = 0;
		switch (signal) {
		case UGSDR_GPS_L1CA:
			require(sv >= 0 && sv < 37, "GPS L1 C/A: satellite index outside 0..36");
			n = 1023;
			break;
		case UGSDR_GPS_L5I:
		case UGSDR_GPS_L5Q:
			require(sv >= 0 && sv < 32, "GPS L5: satellite index outside 0..31");
			n = 10230;
			break;
		case UGSDR_GLONASS_L1OF:
		case UGSDR_GLONASS_L2OF:
			n = 511;
			break;
		case UGSDR_GALILEO_E1B:
		case UGSDR_GALILEO_E1C:
			require(sv >= 0 && sv < 50, "Galileo E1: satellite index outside 0..49");
			n = 2 * 4092;
			break;
		default:
			throw Error(UGSDR_E_UNSUPPORTED, "signal not generated by this library");
		}
		if (len)
			*len = n;
		require(out != nullptr && cap >= n, "output buffer too small for the code");
		switch (signal) {
		case UGSDR_GPS_L1CA: gps_ca(sv, out); break;
		case UGSDR_GPS_L5I: gps_l5(sv, false, out); break;
		case UGSDR_GPS_L5Q: gps_l5(sv, true, out); break;
		case UGSDR_GALILEO_E1B: galileo_e1(sv, false, out); break;
		case UGSDR_GALILEO_E1C: galileo_e1(sv, true, out); break;
		default: glonass_of(out); break;
		}
		return UGSDR_OK;
	}

	uint32_t nco_adder(double fs, double f) {
		// NumericallyControlledOscillator<32> (src/mixer/nco.hpp:17-20)
		if (f < 0)
			f = fs + f;
		return static_cast<uint32_t>(static_cast<uint64_t>(4294967296.0 * f / fs));
	}

	uint32_t nco_phase(double phase) {
		// Mixer::FixPhase (src/mixer/mixer.hpp:21-25) then the NCO holder
		const double two_pi = 2 * 3.14159265358979323846;
		phase = std::fmod(phase, two_pi);
		if (phase < 0)
			phase += two_pi;
		return static_cast<uint32_t>(static_cast<uint64_t>(4294967296.0 * phase / two_pi));
	}

	std::vector<double> doppler_grid(double range, double step) {
		require(step > 0 && range >= 0, "doppler step must be positive and range non-negative");
		std::vector<double> grid;
		// the reference loop, accumulation included (fse.hpp:250-252)
		for (double d = -range; d <= range; d += step) {
			grid.push_back(d);
			require(grid.size() <= 1000000, "doppler grid too large");
		}
		return grid;
	}
}

extern "C" {
int ugsdr_prn_code(int signal, int sv, float* out, size_t cap, size_t* len) {
	return ugsdr_gpu::guarded(nullptr, [&] { ugsdr_gpu::prn_code(signal, sv, out, cap, len); });
}

int ugsdr_repeat_upsample(const float* chips, size_t len, size_t repeats, float* dst, size_t samples) {
	return ugsdr_gpu::guarded(nullptr, [&] {
		ugsdr_gpu::require(chips && dst && len > 0 && repeats > 0, "null buffer or empty code");
		const size_t total = len * repeats;
		for (size_t i = 0; i < samples; ++i)
			dst[i] = chips[((i * total / samples) % total) % len];
	});
}

int ugsdr_doppler_bins(double range, double step, uint32_t* n) {
	return ugsdr_gpu::guarded(nullptr, [&] {
		ugsdr_gpu::require(n != nullptr, "null output");
		*n = static_cast<uint32_t>(ugsdr_gpu::doppler_grid(range, step).size());
	});
}

int ugsdr_abi_version(void) { return UGSDR_CUDA_ABI_VERSION; }
}

namespace ugsdr_gpu {
	// SignalParametersBase::OpenFile, FileType::BbpDdc (signal_parameters.hpp:78-85):
	// 4 bits per complex sample in 64-bit words plus a header word, padded to
	// an even number of words
	size_t bbp_epoch_bytes(double fs) {
		if (!(fs > 0) || std::fmod(fs, 1e3) != 0.0)
			return 0;
		const double words = fs / 1e3 * 4 / 64 + 1;
		size_t b = static_cast<size_t>(words / 2) * 2;
		if (std::fmod(words, 2.0) != 0.0)
			b += 2;
		return b * 8;
	}

	size_t capture_bytes(int sample_type, double fs, size_t n) {
		switch (sample_type) {
		case UGSDR_SAMPLES_CF32: return 8 * n;
		case UGSDR_SAMPLES_CI8: return 2 * n;
		case UGSDR_SAMPLES_CI16: return 4 * n;
		case UGSDR_SAMPLES_BBP_DDC: {
			const size_t eb = bbp_epoch_bytes(fs);
			const size_t spm = eb ? static_cast<size_t>(fs / 1e3) : 0;
			return spm && n % spm == 0 ? n / spm * eb : 0;
		}
		default: return n;  // RI8 and NT1065: one byte per sample
		}
	}
}

extern "C" int ugsdr_sample_bytes(int sample_type, double sampling_rate, size_t n_samples, size_t* bytes) {
	if (!bytes || sample_type < 0 || sample_type > UGSDR_SAMPLES_NT1065_4)
		return UGSDR_E_INVALID;
	*bytes = ugsdr_gpu::capture_bytes(sample_type, sampling_rate, n_samples);
	return *bytes || n_samples == 0 ? UGSDR_OK : UGSDR_E_INVALID;
}

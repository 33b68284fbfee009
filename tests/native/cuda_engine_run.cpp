// Runs CudaFastSearchEngine (include/ugsdr_cuda_engine.hpp) on a raw capture
// and prints one line per kept satellite:
//   system id signal doppler code_offset level sigma intermediate_frequency
// Arguments: file sample_type fs central_frequency range step [ms_offset],
// or --rate fs target to print AdjustSamplingRate(fs, target) (no GPU work).
// Process() runs twice; the second call (code spectra cached on the device)
// must print the same satellites, or the program fails.
#include "ugsdr_cuda_engine.hpp"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iterator>
#include <string>
#include <vector>

int main(int argc, char** argv) {
	if (argc == 4 && std::string(argv[1]) == "--rate") {
		std::printf("%.17g\n", ugsdr::cuda::CudaFastSearchEngine::AdjustSamplingRate(std::atof(argv[2]), std::atof(argv[3])));
		return 0;
	}
	if (argc < 7) {
		std::fprintf(stderr, "usage: %s file sample_type fs central_frequency range step [ms_offset]\n", argv[0]);
		return 2;
	}
	std::ifstream f(argv[1], std::ios::binary);
	const std::vector<char> bytes((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
	ugsdr::cuda::Subband s;
	s.signal = UGSDR_GPS_L1CA;
	s.samples = bytes.data();
	s.sample_type = std::atoi(argv[2]);
	s.sampling_rate = std::atof(argv[3]);
	s.central_frequency = std::atof(argv[4]);
	const std::size_t per = s.sample_type == UGSDR_SAMPLES_CF32 ? 8 : s.sample_type == UGSDR_SAMPLES_CI16 ? 4
		: s.sample_type == UGSDR_SAMPLES_CI8 ? 2 : 1;
	s.n_samples = bytes.size() / per;
	const std::size_t ms_offset = argc > 7 ? static_cast<std::size_t>(std::atoi(argv[7])) : 0;
	try {
		ugsdr::cuda::CudaFastSearchEngine engine({s}, std::atof(argv[5]), std::atof(argv[6]));
		const auto first = engine.Process(false, ms_offset);
		const auto second = engine.Process(false, ms_offset);
		if (first.size() != second.size())
			return 3;
		for (std::size_t i = 0; i < first.size(); ++i) {
			const auto& a = first[i];
			const auto& b = second[i];
			if (a.sv_number.id != b.sv_number.id || a.level != b.level || a.doppler != b.doppler || a.code_offset != b.code_offset)
				return 4;
			std::printf("%u %d %u %.6f %.6f %.9g %.9g %.6f\n", static_cast<unsigned>(a.sv_number.system), a.sv_number.id,
				a.sv_number.signal, a.doppler, a.code_offset, a.level, a.sigma, a.intermediate_frequency);
		}
	}
	catch (const std::exception& e) {
		std::fprintf(stderr, "%s\n", e.what());
		return 1;
	}
	return 0;
}

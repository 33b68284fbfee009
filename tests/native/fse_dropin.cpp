// Drop-in check: the reference's FastSearchEngineBase and policy interfaces
// instantiated on the Cuda* policies (include/ugsdr_cuda_policies.hpp) and
// linked against libugsdr_cuda.so.  Compiled and linked by
// tests/test_integration.py; executed only where a GPU is present.
#include "ugsdr_cuda_policies.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>

using Fse = ugsdr::FastSearchEngineBase<ugsdr::ParametricCudaFseConfig<8192000>, ugsdr::DefaultChannelConfig, float>;
auto instantiate_process = &Fse::Process;
// the batched engine on the reference's DigitalFrontend, same call shape
using BatchedFse = ugsdr::CudaFastSearchEngineFor<ugsdr::DefaultChannelConfig, float>;
auto instantiate_batched = &BatchedFse::Process;

int main() {
	// correlator KAT (basic_tests.cpp:72-86) and mixer KAT (321-357) through the policies
	const auto code = ugsdr::Codegen<ugsdr::GpsL1Ca>::Get<float>(0);
	const std::vector<std::complex<float>> signal(code.begin(), code.end());
	const auto dst = ugsdr::CudaCorrelator::Correlate(std::span(signal), std::span(code));
	auto mixer = ugsdr::CudaMixer(1e6, 1e6 / 2, 0);
	std::vector<std::complex<float>> ones(1000, 1);
	mixer.Translate(ones);
	int bad = dst.real() != 1023.0f || dst.imag() != 0.0f;
	for (std::size_t i = 0; i < ones.size(); ++i)
		bad |= ones[i].real() != 1.0f - 2.0f * (i & 1);
	// matched filter KAT (basic_tests.cpp:368-383)
	const auto glo = ugsdr::Codegen<ugsdr::GlonassOf>::Get<float>(0);
	const std::vector<std::complex<float>> gsig(glo.begin(), glo.end());
	const auto mf = ugsdr::CudaMatchedFilter::Filter(gsig, glo);
	bad |= std::abs(mf[0].real() - 511.0f) > 5e-3f;
	// interference stage: the GPU engine against the reference's own on a CW
	// jammer over small noise (jse.hpp:89-102)
	std::vector<std::complex<float>> jam(4000);
	unsigned s = 12345u;
	auto noise = [&s] {
		s = s * 1664525u + 1013904223u;
		return (static_cast<float>(s >> 8) / 16777216.0f - 0.5f) * 0.8f;
	};
	for (std::size_t i = 0; i < jam.size(); ++i) {
		const double ph = 2 * 3.14159265358979323846 * 16.0 / 128.0 * static_cast<double>(i);
		jam[i] = {noise() + 10.0f * static_cast<float>(std::cos(ph)), noise() + 10.0f * static_cast<float>(std::sin(ph))};
	}
	auto cpu = jam, gpu = jam;
	ugsdr::JammingSuppressionEngine<std::complex<float>> ref_engine(4e6);
	ref_engine.Process(cpu);
	ugsdr::CudaJammingSuppressionEngine<std::complex<float>> cuda_engine(4e6);
	cuda_engine.Process(gpu);
	const auto& rd = ref_engine.GetDetectionResults();
	const auto& gd = cuda_engine.GetDetectionResults();
	bad |= rd.size() != gd.size() || rd.empty();
	for (std::size_t i = 0; i < rd.size() && i < gd.size(); ++i)
		bad |= rd[i].interference_type != gd[i].interference_type || rd[i].frequency_bin != gd[i].frequency_bin;
	float worst = 0.0f;
	for (std::size_t i = 0; i < cpu.size(); ++i)
		worst = std::max(worst, std::abs(cpu[i] - gpu[i]));
	bad |= worst > 1e-3f;
	const auto cols = ugsdr::ShortTimeFourierTransform<ugsdr::CudaStft>::Transform(jam);
	const auto back = ugsdr::ShortTimeFourierTransform<ugsdr::CudaStft>::Transform(cols);
	bad |= cols.size() != (jam.size() - 96) / 32 || back.size() != 128 + (cols.size() - 1) * 32;
	std::printf("%s correlate=(%g,%g) mf0=%g jamming=%zu worst=%g\n", bad ? "FAIL" : "ok", dst.real(), dst.imag(),
		mf[0].real(), gd.size(), worst);
	return bad || instantiate_process == nullptr || instantiate_batched == nullptr;
}

// Drop-in check: the reference's FastSearchEngineBase and policy interfaces
// instantiated on the Cuda* policies (include/ugsdr_cuda_policies.hpp) and
// linked against libugsdr_cuda.so.  Compiled and linked by
// tests/test_integration.py; executed only where a GPU is present.
#include "ugsdr_cuda_policies.hpp"

#include <cstdio>

using Fse = ugsdr::FastSearchEngineBase<ugsdr::ParametricCudaFseConfig<8192000>, ugsdr::DefaultChannelConfig, float>;
auto instantiate_process = &Fse::Process;

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
	std::printf("%s correlate=(%g,%g) mf0=%g\n", bad ? "FAIL" : "ok", dst.real(), dst.imag(), mf[0].real());
	return bad || instantiate_process == nullptr;
}

// Host-side check of the device FFT building blocks (fft_core.cuh): runs the
// same Stockham butterflies the kernels run, sequentially, and compares with
// a double-precision direct DFT.  Built with nvcc as host code; no GPU used.
// Usage: fft_core_check N [N ...]  -> prints "N max_rel_err_fwd max_rel_err_inv radices"
#include "../../ugsdr_gb300/csrc/fft_core.cuh"
#include "../../ugsdr_gb300/csrc/fft_plan.hpp"

#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

using namespace ugsdr_gpu;

static double run(int n, bool inv, const std::vector<int>& radices) {
	std::vector<float2> tw(n);
	for (int m = 0; m < n; ++m) {
		const double a = 2.0 * 3.14159265358979323846 * m / n;
		tw[m] = c2(static_cast<float>(std::cos(a)), static_cast<float>(-std::sin(a)));
	}
	std::mt19937 rng(n);
	std::normal_distribution<float> g;
	std::vector<float2> a(n), b(n);
	for (auto& v : a)
		v = c2(g(rng), g(rng));
	const std::vector<float2> x = a;
	int ns = 1;
	for (int r : radices) {
		for (int j = 0; j < n / r; ++j) {
			const bool ok = inv ? butterfly_dispatch<true>(r, a.data(), b.data(), n, ns, tw.data(), j, j % ns)
			                    : butterfly_dispatch<false>(r, a.data(), b.data(), n, ns, tw.data(), j, j % ns);
			if (!ok) {
				std::printf("radix %d unsupported\n", r);
				std::exit(2);
			}
		}
		std::swap(a, b);
		ns *= r;
	}
	double max_err = 0, norm = 0;
	const double sgn = inv ? 1.0 : -1.0;
	for (int k = 0; k < n; ++k) {
		std::complex<double> acc = 0;
		for (int j = 0; j < n; ++j) {
			const double ang = sgn * 2.0 * 3.14159265358979323846 * static_cast<double>((static_cast<long long>(j) * k) % n) / n;
			acc += std::complex<double>(x[j].x, x[j].y) * std::complex<double>(std::cos(ang), std::sin(ang));
		}
		const double e = std::abs(acc - std::complex<double>(a[k].x, a[k].y));
		max_err = std::max(max_err, e);
		norm = std::max(norm, std::abs(acc));
	}
	return max_err / norm;
}

int main(int argc, char** argv) {
	int worst = 0;
	for (int i = 1; i < argc; ++i) {
		const int n = std::atoi(argv[i]);
		std::vector<int> radices;
		if (!plan_radices(n, radices)) {
			std::printf("%d unplannable\n", n);
			return 3;
		}
		const double ef = run(n, false, radices), ei = run(n, true, radices);
		std::printf("%d %.3e %.3e", n, ef, ei);
		for (int r : radices)
			std::printf(" %d", r);
		std::printf("\n");
		if (ef > 1e-5 || ei > 1e-5)
			worst = 1;
	}
	return worst;
}

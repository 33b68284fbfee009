// ORACLE / TEST INFRASTRUCTURE ONLY — never linked into the product library.
//
// Double-precision mixed-radix DFT used by the CPU oracle and by the FFTW-API
// shim that lets the reference's FFTW path (src/math/dft.hpp:114-135) compile
// here without libfftw3.  Written from the textbook Cooley-Tukey recursion:
// N = p * m, p sub-DFTs of length m over decimated inputs, then a combine with
// twiddles w_N^{q k} and a p-point DFT per output column.  Any prime factor is
// handled by a direct p-point DFT, so every N (including 2046 = 2*3*11*31 and
// 204600 = 2^3*3*5^2*11*31) is exact up to double rounding; the cost is
// O(N * sum of prime factors).
//
// Convention (FFTW's): out[k] = sum_j in[j] * exp(sign * 2*pi*i * j*k / N),
// unnormalised; sign = -1 forward, +1 backward.
#pragma once

#include <cmath>
#include <complex>
#include <cstddef>
#include <vector>

namespace oracle {
	using cd = std::complex<double>;

	class Fft64 {
	public:
		Fft64(std::size_t n, int sign) : n_(n), sign_(sign) {
			std::size_t rest = n;
			for (std::size_t p = 2; p * p <= rest; ++p)
				while (rest % p == 0) {
					primes_.push_back(p);
					rest /= p;
				}
			if (rest > 1)
				primes_.push_back(rest);
			// prefer large radices first: fewer recursion levels, same result
			tw_.resize(n);
			const double two_pi = 2.0 * 3.14159265358979323846;
			for (std::size_t i = 0; i < n; ++i) {
				// reduce the angle exactly in integers before the double multiply
				const double a = two_pi * static_cast<double>(i) / static_cast<double>(n);
				tw_[i] = cd(std::cos(a), sign * std::sin(a));
			}
			scratch_.resize(primes_.empty() ? 1 : primes_.back() > 64 ? primes_.back() : 64);
		}

		void Execute(const cd* in, cd* out) {
			if (n_ == 0)
				return;
			if (n_ == 1) {
				out[0] = in[0];
				return;
			}
			Rec(out, in, n_, 1, 0, 1);
		}

		std::size_t Size() const { return n_; }

	private:
		std::size_t n_;
		int sign_;
		std::vector<std::size_t> primes_;
		std::vector<cd> tw_;
		std::vector<cd> scratch_;

		// out[0..n) = DFT_n of in[j*s], j < n; level indexes primes_; tw_step = N / n
		void Rec(cd* out, const cd* in, std::size_t n, std::size_t s, std::size_t level, std::size_t tw_step) {
			if (n == 1) {
				out[0] = in[0];
				return;
			}
			const std::size_t p = primes_[level];
			const std::size_t m = n / p;
			for (std::size_t q = 0; q < p; ++q)
				Rec(out + q * m, in + q * s, m, s * p, level + 1, tw_step * p);

			std::vector<cd> t(p), y(p);
			const std::size_t wp_step = n_ / p;  // w_p^{1} = tw_[N/p]
			for (std::size_t k = 0; k < m; ++k) {
				for (std::size_t q = 0; q < p; ++q) {
					const std::size_t e = (q * k * tw_step) % n_;
					t[q] = out[q * m + k] * tw_[e];
				}
				for (std::size_t r = 0; r < p; ++r) {
					cd acc = 0.0;
					for (std::size_t q = 0; q < p; ++q)
						acc += t[q] * tw_[((q * r) % p) * wp_step];
					y[r] = acc;
				}
				for (std::size_t r = 0; r < p; ++r)
					out[k + m * r] = y[r];
			}
		}
	};
}

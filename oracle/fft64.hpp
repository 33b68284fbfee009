// ORACLE / TEST INFRASTRUCTURE ONLY — never linked into the product library.
//
// Mixed-radix DFT used by the CPU oracle (double precision) and by the
// FFTW-API shim that lets the reference's FFTW path (src/math/dft.hpp:114-135)
// compile here without libfftw3.  Iterative Stockham autosort (Cooley-Tukey
// decimation in frequency of the index map, no bit reversal): N = p_0 p_1 ...,
// one pass per prime-power factor with radix-4/2/3/5 butterflies written out
// and a direct p-point DFT for any other prime p, so every N (including
// 2046 = 2*3*11*31 and 204600 = 2^3*3*5^2*11*31) is exact up to rounding;
// the cost is O(N * sum of factors).  Twiddles come from a per-size table
// computed in double.  FftT<float> is the float build of the same algorithm
// (the CPU baseline's FFTW-class float transform); the oracle checker uses
// FftT<double>.
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

	template <typename T>
	class FftT {
	public:
		using C = std::complex<T>;

		FftT(std::size_t n, int sign) : n_(n), sign_(sign) {
			std::size_t rest = n;
			while (rest % 4 == 0) {
				radix_.push_back(4);
				rest /= 4;
			}
			for (std::size_t p = 2; p * p <= rest; ++p)
				while (rest % p == 0) {
					radix_.push_back(p);
					rest /= p;
				}
			if (rest > 1)
				radix_.push_back(rest);
			// per-pass twiddles W_N^{r k N / (ns p)}, laid out [r - 1][k] (k < ns,
			// 1 <= r < p) so the inner loop over k reads them contiguously
			const double two_pi = 2.0 * 3.14159265358979323846;
			std::size_t ns = 1;
			for (const std::size_t p : radix_) {
				offset_.push_back(tw_.size());
				for (std::size_t r = 1; r < p; ++r)
					for (std::size_t k = 0; k < ns; ++k) {
						const std::size_t e = (r * k * (n / (ns * p))) % n;
						const double a = two_pi * static_cast<double>(e) / static_cast<double>(n);
						tw_.push_back(C(static_cast<T>(std::cos(a)), static_cast<T>(sign * std::sin(a))));
					}
				// p-point DFT table for the generic butterfly
				wp_offset_.push_back(wp_.size());
				if (p != 2 && p != 3 && p != 4 && p != 5)
					for (std::size_t m = 0; m < p; ++m) {
						const double a = two_pi * static_cast<double>(m) / static_cast<double>(p);
						wp_.push_back(C(static_cast<T>(std::cos(a)), static_cast<T>(sign * std::sin(a))));
					}
				ns *= p;
			}
		}

		// out may alias in
		void Execute(const C* in, C* out) const {
			if (n_ == 0)
				return;
			if (n_ == 1) {
				out[0] = in[0];
				return;
			}
			std::vector<C> a(in, in + n_), b(n_);
			C* src = a.data();
			C* dst = b.data();
			std::size_t ns = 1;
			for (std::size_t s = 0; s < radix_.size(); ++s) {
				Pass(src, dst, radix_[s], ns, tw_.data() + offset_[s], wp_.data() + wp_offset_[s]);
				std::swap(src, dst);
				ns *= radix_[s];
			}
			std::copy(src, src + n_, out);
		}

		std::size_t Size() const { return n_; }

	private:
		std::size_t n_;
		int sign_;
		std::vector<std::size_t> radix_, offset_, wp_offset_;
		std::vector<C> tw_, wp_;

		// one radix-p pass: v_r = in[j + r n/p] W^{r k}, k = j mod ns; DFT_p;
		// out[(j - k) p + k + r ns] = v_r.  Loop order: groups b = j / ns
		// outside, k inside (contiguous loads, stores and twiddles).
		void Pass(const C* in, C* out, std::size_t p, std::size_t ns, const C* tw, const C* wp) const {
			const std::size_t nb = n_ / p;
			C v[64];
			std::vector<C> big(p > 64 ? p : 0), acc(p > 64 ? p : 0);
			C* vv = p > 64 ? big.data() : v;
			C y[64];
			C* yy = p > 64 ? acc.data() : y;
			for (std::size_t j0 = 0; j0 < nb; j0 += ns) {
				const C* src = in + j0;
				C* o = out + j0 * p;
				for (std::size_t k = 0; k < ns; ++k) {
					vv[0] = src[k];
					for (std::size_t r = 1; r < p; ++r)
						vv[r] = ns > 1 ? Mul(src[k + r * nb], tw[(r - 1) * ns + k]) : src[k + r * nb];
					Butterfly(vv, yy, p, wp);
					for (std::size_t r = 0; r < p; ++r)
						o[k + r * ns] = yy[r];
				}
			}
		}

		// plain complex product (no C99 Annex G infinity recovery)
		static C Mul(const C& a, const C& b) {
			return C(a.real() * b.real() - a.imag() * b.imag(), a.real() * b.imag() + a.imag() * b.real());
		}

		void Butterfly(const C* v, C* y, std::size_t p, const C* wp) const {
			const T s = static_cast<T>(sign_);
			switch (p) {
			case 2:
				y[0] = v[0] + v[1];
				y[1] = v[0] - v[1];
				return;
			case 4: {
				const C a0 = v[0] + v[2], a1 = v[0] - v[2];
				const C b0 = v[1] + v[3], d = v[1] - v[3];
				const C b1(-s * d.imag(), s * d.real());  // d * (sign i)
				y[0] = a0 + b0;
				y[2] = a0 - b0;
				y[1] = a1 + b1;
				y[3] = a1 - b1;
				return;
			}
			case 3: {
				const T c1 = static_cast<T>(-0.5), s1 = static_cast<T>(0.86602540378443864676) * s;
				const C t = v[1] + v[2], d = v[1] - v[2];
				y[0] = v[0] + t;
				const C m = v[0] + c1 * t;
				const C r(-s1 * d.imag(), s1 * d.real());
				y[1] = m + r;
				y[2] = m - r;
				return;
			}
			case 5: {
				const T c1 = static_cast<T>(0.30901699437494742410), c2 = static_cast<T>(-0.80901699437494742410);
				const T s1 = static_cast<T>(0.95105651629515357212) * s, s2 = static_cast<T>(0.58778525229247312917) * s;
				const C t1 = v[1] + v[4], d1 = v[1] - v[4], t2 = v[2] + v[3], d2 = v[2] - v[3];
				y[0] = v[0] + t1 + t2;
				const C m1 = v[0] + c1 * t1 + c2 * t2, m2 = v[0] + c2 * t1 + c1 * t2;
				const C n1 = s1 * d1 + s2 * d2, n2 = s2 * d1 - s1 * d2;
				const C r1(-n1.imag(), n1.real()), r2(-n2.imag(), n2.real());
				y[1] = m1 + r1;
				y[4] = m1 - r1;
				y[2] = m2 + r2;
				y[3] = m2 - r2;
				return;
			}
			default:
				for (std::size_t r = 0; r < p; ++r) {
					C a = v[0];
					std::size_t e = 0;
					for (std::size_t q = 1; q < p; ++q) {
						e += r;
						if (e >= p)
							e -= p;
						a += Mul(v[q], wp[e]);
					}
					y[r] = a;
				}
			}
		}
	};

	using Fft64 = FftT<double>;
	using Fft32 = FftT<float>;
}

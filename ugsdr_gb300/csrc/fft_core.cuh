// Mixed-radix FFT building blocks for the acquisition kernels.
//
// The reference computes every matched filter with FFTW (src/math/dft.hpp:
// 114-135) one transform per call; here the same transforms run inside fused
// kernels, so the transform is split into reusable pieces:
//   * Dft<R, INV>::run(v)  - an R-point DFT held in registers, fully unrolled,
//                            with compile-time twiddles (R any product of
//                            primes; trivial rotations use no multiplies);
//   * stockham_butterfly    - one butterfly of a radix-R Stockham pass
//                            (natural-order in and out, no bit reversal), the
//                            pass twiddles read from a per-size table
//                            W_N^m = exp(-2 pi i m / N) computed on the host in
//                            double precision.
// Everything is __host__ __device__, so the same source can run on the CPU.
#pragma once

#include <cstdint>
#include <type_traits>
#include <utility>

#include <vector_types.h>

#define UG_HD __host__ __device__ __forceinline__

namespace ugsdr_gpu {

	UG_HD float2 c2(float x, float y) {
		float2 r;
		r.x = x;
		r.y = y;
		return r;
	}
	// Complex sums and the real-scalar multiply-add of the DFT kernels as
	// packed FP32 pair instructions on the device (sm_100 and later: one
	// instruction for both halves, each half rounded as the scalar form)
#if defined(__CUDA_ARCH__) && (__CUDA_ARCH__ >= 1000)
#define UG_PACKED_F32 1
#endif
	UG_HD float2 cadd(float2 a, float2 b) {
#ifdef UG_PACKED_F32
		return __fadd2_rn(a, b);
#else
		return c2(a.x + b.x, a.y + b.y);
#endif
	}
	UG_HD float2 csub(float2 a, float2 b) {
#ifdef UG_PACKED_F32
		return __fadd2_rn(a, c2(-b.x, -b.y));
#else
		return c2(a.x - b.x, a.y - b.y);
#endif
	}
	// acc + s a per half, the product fused into the sum (the contraction the
	// compiler forms for the scalar expression on the device)
	UG_HD float2 cfma_s(float s, float2 a, float2 acc) {
#ifdef UG_PACKED_F32
		return __ffma2_rn(c2(s, s), a, acc);
#else
		return c2(acc.x + s * a.x, acc.y + s * a.y);
#endif
	}
	UG_HD float2 cmul(float2 a, float2 b) { return c2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
	// a * conj(b)
	UG_HD float2 cmulc(float2 a, float2 b) { return c2(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }
	UG_HD float2 cscale(float2 a, float s) { return c2(a.x * s, a.y * s); }

	// ---------------------------------------------------------------------
	// Compile-time trigonometry on rational angles 2*pi*num/den, evaluated
	// in double by octant reduction + Taylor series (|x| <= pi/4, 14 terms:
	// error far below float rounding).
	namespace ct {
		constexpr double kPi = 3.14159265358979323846;
		constexpr double sin_taylor(double x) {
			double term = x, sum = x;
			for (int i = 1; i < 14; ++i) {
				term *= -x * x / ((2.0 * i) * (2.0 * i + 1.0));
				sum += term;
			}
			return sum;
		}
		constexpr double cos_taylor(double x) {
			double term = 1.0, sum = 1.0;
			for (int i = 1; i < 14; ++i) {
				term *= -x * x / ((2.0 * i - 1.0) * (2.0 * i));
				sum += term;
			}
			return sum;
		}
		// cos and sin of 2*pi*num/den for integers (any sign)
		constexpr long mod_pos(long a, long m) { return ((a % m) + m) % m; }
		constexpr double cos2pi(long num, long den) {
			// reduce to eighths: 8*num/den = q + f, f in [0,1)
			const long n = mod_pos(num, den);
			const long n8 = 8 * n;
			const long q = n8 / den;                   // octant 0..7
			const double f = static_cast<double>(n8 - q * den) / static_cast<double>(den);  // [0,1)
			const double a = f * kPi / 4.0;            // angle within octant
			const double b = (1.0 - f) * kPi / 4.0;    // complement
			switch (q) {
			case 0: return cos_taylor(a);
			case 1: return sin_taylor(b);
			case 2: return -sin_taylor(a);
			case 3: return -cos_taylor(b);
			case 4: return -cos_taylor(a);
			case 5: return -sin_taylor(b);
			case 6: return sin_taylor(a);
			default: return cos_taylor(b);
			}
		}
		constexpr double sin2pi(long num, long den) { return cos2pi(num * 4 - den, 4 * den); }
	}

	// multiply by W = exp(s * 2 pi i num/den), s = -1 forward, +1 inverse,
	// with the trivial and 45-degree rotations special-cased.
	template <long NUM, long DEN, bool INV>
	UG_HD float2 twiddle_mul(float2 v) {
		constexpr long n = ct::mod_pos(NUM, DEN);
		if constexpr (n == 0) {
			return v;
		}
		else if constexpr ((4 * n) % DEN == 0) {
			constexpr long quarter = (4 * n) / DEN;  // 1,2,3 quarter turns of exp(-2 pi i x)
			// forward: exp(-i pi/2 * quarter); inverse: exp(+i pi/2 * quarter)
			constexpr long qq = INV ? (4 - quarter) % 4 : quarter;
			if constexpr (qq == 1) return c2(v.y, -v.x);   // * (-i)
			else if constexpr (qq == 2) return c2(-v.x, -v.y);
			else return c2(-v.y, v.x);                     // * (+i)
		}
		else if constexpr ((8 * n) % DEN == 0) {
			constexpr float h = 0.70710678118654752440f;
			constexpr double c = ct::cos2pi(NUM, DEN);
			constexpr double s = INV ? ct::sin2pi(NUM, DEN) : -ct::sin2pi(NUM, DEN);
			constexpr float cr = c > 0 ? h : -h;
			constexpr float ci = s > 0 ? h : -h;
			return c2(cr * v.x - ci * v.y, cr * v.y + ci * v.x);
		}
		else {
			constexpr float cr = static_cast<float>(ct::cos2pi(NUM, DEN));
			constexpr float ci = static_cast<float>(INV ? ct::sin2pi(NUM, DEN) : -ct::sin2pi(NUM, DEN));
			return c2(cr * v.x - ci * v.y, cr * v.y + ci * v.x);
		}
	}

	// ---------------------------------------------------------------------
	// compile-time loops
	template <int I, int N, typename F>
	UG_HD void static_for(F&& f) {
		if constexpr (I < N) {
			f(std::integral_constant<int, I>{});
			static_for<I + 1, N>(f);
		}
	}

	constexpr int smallest_factor(int n) {
		if (n % 4 == 0 && n != 4 && n != 8 && n != 16) return 4;
		for (int p = 2; p * p <= n; ++p)
			if (n % p == 0)
				return p;
		return n;
	}
	constexpr bool is_prime(int n) {
		if (n < 2) return false;
		for (int p = 2; p * p <= n; ++p)
			if (n % p == 0)
				return false;
		return true;
	}

	// ---------------------------------------------------------------------
	// R-point DFT in registers: out[k] = sum_j in[j] exp(-/+ 2 pi i jk/R),
	// natural order in and out, in place on v[0..R).
	template <int R, bool INV>
	struct Dft {
		UG_HD static void run(float2* v);
	};

	template <bool INV>
	struct Dft<1, INV> {
		UG_HD static void run(float2*) {}
	};

	template <bool INV>
	struct Dft<2, INV> {
		UG_HD static void run(float2* v) {
			const float2 a = v[0], b = v[1];
			v[0] = cadd(a, b);
			v[1] = csub(a, b);
		}
	};

	template <bool INV>
	struct Dft<4, INV> {
		UG_HD static void run(float2* v) {
			const float2 a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
			const float2 b0 = cadd(v[1], v[3]), b1 = twiddle_mul<1, 4, INV>(csub(v[1], v[3]));
			v[0] = cadd(a0, b0);
			v[2] = csub(a0, b0);
			v[1] = cadd(a1, b1);
			v[3] = csub(a1, b1);
		}
	};

	// odd prime P: pairwise symmetric direct DFT,
	// out[k] = v0 + sum_{j=1}^{(P-1)/2} (v_j + v_{P-j}) cos(2 pi jk/P) -/+ i (v_j - v_{P-j}) sin(2 pi jk/P)
	template <int P, bool INV>
	struct DftPrime {
		UG_HD static void run(float2* v) {
			constexpr int H = (P - 1) / 2;
			float2 sp[H + 1], sm[H + 1];
			static_for<1, H + 1>([&](auto jc) {
				constexpr int j = decltype(jc)::value;
				sp[j] = cadd(v[j], v[P - j]);
				sm[j] = csub(v[j], v[P - j]);
			});
			float2 out[P];
			float2 dc = v[0];
			static_for<1, H + 1>([&](auto jc) {
				constexpr int j = decltype(jc)::value;
				dc = cadd(dc, sp[j]);
			});
			out[0] = dc;
			static_for<1, H + 1>([&](auto kc) {
				constexpr int k = decltype(kc)::value;
				float2 re = v[0];       // real-cos part
				float2 im = c2(0.f, 0.f); // sin part (to be multiplied by -/+ i)
				static_for<1, H + 1>([&](auto jc) {
					constexpr int j = decltype(jc)::value;
					constexpr float c = static_cast<float>(ct::cos2pi(static_cast<long>(j) * k, P));
					constexpr float s = static_cast<float>(ct::sin2pi(static_cast<long>(j) * k, P));
					re = cfma_s(c, sp[j], re);
					im = cfma_s(s, sm[j], im);
				});
				// forward: exp(-i t) -> term = re - i*im ; inverse: re + i*im
				if constexpr (!INV) {
					out[k] = c2(re.x + im.y, re.y - im.x);
					out[P - k] = c2(re.x - im.y, re.y + im.x);
				}
				else {
					out[k] = c2(re.x - im.y, re.y + im.x);
					out[P - k] = c2(re.x + im.y, re.y - im.x);
				}
			});
			static_for<0, P>([&](auto kc) {
				constexpr int k = decltype(kc)::value;
				v[k] = out[k];
			});
		}
	};

	// composite R = A * B (A = chosen factor): decimation in time
	template <int R, bool INV>
	struct DftComposite {
		UG_HD static void run(float2* v) {
			constexpr int A = smallest_factor(R);
			constexpr int B = R / A;
			float2 t[A][B];
			static_for<0, A>([&](auto ac) {
				constexpr int a = decltype(ac)::value;
				static_for<0, B>([&](auto bc) {
					constexpr int b = decltype(bc)::value;
					t[a][b] = v[a + A * b];
				});
				Dft<B, INV>::run(t[a]);
			});
			static_for<0, B>([&](auto kc) {
				constexpr int k = decltype(kc)::value;
				float2 col[A];
				static_for<0, A>([&](auto ac) {
					constexpr int a = decltype(ac)::value;
					col[a] = twiddle_mul<static_cast<long>(a) * k, R, INV>(t[a][k]);
				});
				Dft<A, INV>::run(col);
				static_for<0, A>([&](auto rc) {
					constexpr int r = decltype(rc)::value;
					v[k + B * r] = col[r];
				});
			});
		}
	};

	template <int R, bool INV>
	UG_HD void Dft<R, INV>::run(float2* v) {
		if constexpr (is_prime(R))
			DftPrime<R, INV>::run(v);
		else
			DftComposite<R, INV>::run(v);
	}

	// ---------------------------------------------------------------------
	// R-point DFT whose inputs v[NZ..R) are zero and are not read: Dft<R>'s
	// operations with the terms of those inputs left out.  Dropping x + 0,
	// x - 0 and the c * 0 terms of the FMA chains changes no value but the
	// sign of an exact zero, so the outputs equal Dft<R>'s on the
	// zero-filled input in magnitude, bit for bit.
	template <int R, bool INV, int NZ>
	struct DftPruned {
		UG_HD static void run(float2* v);
	};

	template <int P, bool INV, int NZ>
	struct DftPrimePruned {
		UG_HD static void run(float2* v) {
			constexpr int H = (P - 1) / 2;
			// j <= H < P - j: input P - j is zero whenever j is; sp / sm of a
			// zero input j are zero and their terms are left out (j < NZ live)
			constexpr int JL = NZ - 1 < H ? NZ - 1 : H;  // live pairs j = 1..JL
			float2 sp[H + 1], sm[H + 1];
			static_for<1, JL + 1>([&](auto jc) {
				constexpr int j = decltype(jc)::value;
				if constexpr (P - j < NZ) {
					sp[j] = cadd(v[j], v[P - j]);
					sm[j] = csub(v[j], v[P - j]);
				}
				else {
					sp[j] = v[j];
					sm[j] = v[j];
				}
			});
			float2 out[P];
			float2 dc = v[0];
			static_for<1, JL + 1>([&](auto jc) {
				constexpr int j = decltype(jc)::value;
				dc = cadd(dc, sp[j]);
			});
			out[0] = dc;
			static_for<1, H + 1>([&](auto kc) {
				constexpr int k = decltype(kc)::value;
				float2 re = v[0];
				float2 im = c2(0.f, 0.f);
				static_for<1, JL + 1>([&](auto jc) {
					constexpr int j = decltype(jc)::value;
					constexpr float c = static_cast<float>(ct::cos2pi(static_cast<long>(j) * k, P));
					constexpr float s = static_cast<float>(ct::sin2pi(static_cast<long>(j) * k, P));
					re = cfma_s(c, sp[j], re);
					im = cfma_s(s, sm[j], im);
				});
				if constexpr (!INV) {
					out[k] = c2(re.x + im.y, re.y - im.x);
					out[P - k] = c2(re.x - im.y, re.y + im.x);
				}
				else {
					out[k] = c2(re.x - im.y, re.y + im.x);
					out[P - k] = c2(re.x + im.y, re.y - im.x);
				}
			});
			static_for<0, P>([&](auto kc) {
				constexpr int k = decltype(kc)::value;
				v[k] = out[k];
			});
		}
	};

	template <int R, bool INV, int NZ>
	struct DftCompositePruned {
		UG_HD static void run(float2* v) {
			constexpr int A = smallest_factor(R);
			constexpr int B = R / A;
			constexpr int AL = NZ < A ? NZ : A;  // rows a < AL hold a live input
			float2 t[A][B];
			static_for<0, AL>([&](auto ac) {
				constexpr int a = decltype(ac)::value;
				constexpr int live = (NZ - a + A - 1) / A;  // b with a + A b < NZ
				static_for<0, live>([&](auto bc) {
					constexpr int b = decltype(bc)::value;
					t[a][b] = v[a + A * b];
				});
				DftPruned<B, INV, live>::run(t[a]);
			});
			static_for<0, B>([&](auto kc) {
				constexpr int k = decltype(kc)::value;
				float2 col[A];
				static_for<0, AL>([&](auto ac) {
					constexpr int a = decltype(ac)::value;
					col[a] = twiddle_mul<static_cast<long>(a) * k, R, INV>(t[a][k]);
				});
				DftPruned<A, INV, AL>::run(col);
				static_for<0, A>([&](auto rc) {
					constexpr int r = decltype(rc)::value;
					v[k + B * r] = col[r];
				});
			});
		}
	};

	template <int R, bool INV, int NZ>
	UG_HD void DftPruned<R, INV, NZ>::run(float2* v) {
		static_assert(NZ >= 1, "a pruned DFT keeps input 0");
		if constexpr (NZ >= R) {
			Dft<R, INV>::run(v);
		}
		else if constexpr (NZ == 1) {
			// a lone input: every output is v[0]
			static_for<1, R>([&](auto kc) { v[decltype(kc)::value] = v[0]; });
		}
		else if constexpr (is_prime(R)) {
			DftPrimePruned<R, INV, NZ>::run(v);
		}
		else if constexpr (R == 4) {
			// Dft<4, INV> with v[3] (NZ == 3) or v[2], v[3] (NZ == 2) zero
			float2 a0 = v[0], a1 = v[0];
			if constexpr (NZ == 3) {
				a0 = cadd(v[0], v[2]);
				a1 = csub(v[0], v[2]);
			}
			const float2 b0 = v[1], b1 = twiddle_mul<1, 4, INV>(v[1]);
			v[0] = cadd(a0, b0);
			v[2] = csub(a0, b0);
			v[1] = cadd(a1, b1);
			v[3] = csub(a1, b1);
		}
		else {
			DftCompositePruned<R, INV, NZ>::run(v);
		}
	}

	// ---------------------------------------------------------------------
	// One butterfly (index j < N/R) of a radix-R Stockham pass:
	//   v[r] = in[j + r N/R] * W_{Ns R}^{r (j mod Ns)},  DFT_R(v),
	//   out[(j / Ns) Ns R + (j mod Ns) + r Ns] = v[r].
	// tw[m] = exp(-2 pi i m / N) (conjugated for the inverse).
	// k = j mod ns is passed in (callers divide with a float reciprocal).
	template <int R, bool INV>
	UG_HD void stockham_load(const float2* in, int n, int ns, const float2* tw, int j, int k, float2* v) {
		const int stride = n / R;
#pragma unroll
		for (int r = 0; r < R; ++r)
			v[r] = in[j + r * stride];
		if (ns == 1)
			return;  // first pass: every twiddle is 1
		const int tw_step = (n / (ns * R)) * k;  // twiddle exponent per r, in units of 1/N
#pragma unroll
		for (int r = 1; r < R; ++r) {
			const float2 w = tw[r * tw_step];
			v[r] = INV ? cmulc(v[r], w) : cmul(v[r], w);
		}
	}

	template <int R>
	UG_HD void stockham_store(float2* out, int ns, int j, int k, const float2* v) {
		const int base = (j - k) * R + k;
#pragma unroll
		for (int r = 0; r < R; ++r)
			out[base + r * ns] = v[r];
	}

	template <int R, bool INV>
	UG_HD void stockham_butterfly(const float2* in, float2* out, int n, int ns, const float2* tw, int j, int k) {
		float2 v[R];
		stockham_load<R, INV>(in, n, ns, tw, j, k, v);
		Dft<R, INV>::run(v);
		stockham_store<R>(out, ns, j, k, v);
	}

	// floor(a / b) for 0 <= a < 2^20, b >= 1, from inv_b = 1.0f / b:
	// (a + 0.5) / b is at least 0.5 / b away from an integer and the float
	// product errs by less than 2^20 / b * 2^-23 = 2^-3 / b, so truncation is exact.
	UG_HD int fdiv(int a, float inv_b) { return static_cast<int>((static_cast<float>(a) + 0.5f) * inv_b); }

	// Runtime dispatch of one butterfly; returns false for an unsupported radix.
	template <bool INV>
	UG_HD bool butterfly_dispatch(int radix, const float2* in, float2* out, int n, int ns, const float2* tw, int j, int k) {
		switch (radix) {
		case 2: stockham_butterfly<2, INV>(in, out, n, ns, tw, j, k); return true;
		case 3: stockham_butterfly<3, INV>(in, out, n, ns, tw, j, k); return true;
		case 4: stockham_butterfly<4, INV>(in, out, n, ns, tw, j, k); return true;
		case 5: stockham_butterfly<5, INV>(in, out, n, ns, tw, j, k); return true;
		case 6: stockham_butterfly<6, INV>(in, out, n, ns, tw, j, k); return true;
		case 7: stockham_butterfly<7, INV>(in, out, n, ns, tw, j, k); return true;
		case 8: stockham_butterfly<8, INV>(in, out, n, ns, tw, j, k); return true;
		case 9: stockham_butterfly<9, INV>(in, out, n, ns, tw, j, k); return true;
		case 10: stockham_butterfly<10, INV>(in, out, n, ns, tw, j, k); return true;
		case 11: stockham_butterfly<11, INV>(in, out, n, ns, tw, j, k); return true;
		case 12: stockham_butterfly<12, INV>(in, out, n, ns, tw, j, k); return true;
		case 13: stockham_butterfly<13, INV>(in, out, n, ns, tw, j, k); return true;
		case 16: stockham_butterfly<16, INV>(in, out, n, ns, tw, j, k); return true;
		case 17: stockham_butterfly<17, INV>(in, out, n, ns, tw, j, k); return true;
		case 19: stockham_butterfly<19, INV>(in, out, n, ns, tw, j, k); return true;
		case 20: stockham_butterfly<20, INV>(in, out, n, ns, tw, j, k); return true;
		case 23: stockham_butterfly<23, INV>(in, out, n, ns, tw, j, k); return true;
		case 25: stockham_butterfly<25, INV>(in, out, n, ns, tw, j, k); return true;
		case 27: stockham_butterfly<27, INV>(in, out, n, ns, tw, j, k); return true;
		case 29: stockham_butterfly<29, INV>(in, out, n, ns, tw, j, k); return true;
		case 31: stockham_butterfly<31, INV>(in, out, n, ns, tw, j, k); return true;
		case 32: stockham_butterfly<32, INV>(in, out, n, ns, tw, j, k); return true;
		default: return false;
		}
	}
}

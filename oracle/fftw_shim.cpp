// ORACLE / TEST INFRASTRUCTURE ONLY: implementation of the FFTW-API subset in
// oracle/shims/fftw3.h over oracle/fft64.hpp.  Linked only into
// oracle/_ref/libugsdr_ref.so (the reference's primitives compiled here).
#include "shims/fftw3.h"
#include "fft64.hpp"

#include <vector>

struct oracle_fftw_plan_s {
	int n;
	int sign;
	bool r2c;
};

namespace {
	template <typename R>
	void ExecC2c(const oracle_fftw_plan_s* p, const R* in, R* out) {
		std::vector<oracle::cd> x(p->n), y(p->n);
		for (int i = 0; i < p->n; ++i)
			x[i] = oracle::cd(in[2 * i], in[2 * i + 1]);
		oracle::Fft64(p->n, p->sign).Execute(x.data(), y.data());
		for (int i = 0; i < p->n; ++i) {
			out[2 * i] = static_cast<R>(y[i].real());
			out[2 * i + 1] = static_cast<R>(y[i].imag());
		}
	}

	template <typename R>
	void ExecR2c(const oracle_fftw_plan_s* p, const R* in, R* out) {
		std::vector<oracle::cd> x(p->n), y(p->n);
		for (int i = 0; i < p->n; ++i)
			x[i] = oracle::cd(in[i], 0.0);
		oracle::Fft64(p->n, -1).Execute(x.data(), y.data());
		for (int i = 0; i <= p->n / 2; ++i) {
			out[2 * i] = static_cast<R>(y[i].real());
			out[2 * i + 1] = static_cast<R>(y[i].imag());
		}
	}
}

extern "C" {
fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex*, fftwf_complex*, int sign, unsigned) {
	return new oracle_fftw_plan_s{n, sign, false};
}
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float*, fftwf_complex*, unsigned) {
	return new oracle_fftw_plan_s{n, -1, true};
}
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out) {
	ExecC2c<float>(p, &in[0][0], &out[0][0]);
}
void fftwf_execute_dft_r2c(const fftwf_plan p, float* in, fftwf_complex* out) {
	ExecR2c<float>(p, in, &out[0][0]);
}
void fftwf_destroy_plan(fftwf_plan p) { delete p; }
void fftwf_make_planner_thread_safe(void) {}

fftw_plan fftw_plan_dft_1d(int n, fftw_complex*, fftw_complex*, int sign, unsigned) {
	return new oracle_fftw_plan_s{n, sign, false};
}
fftw_plan fftw_plan_dft_r2c_1d(int n, double*, fftw_complex*, unsigned) {
	return new oracle_fftw_plan_s{n, -1, true};
}
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out) {
	ExecC2c<double>(p, &in[0][0], &out[0][0]);
}
void fftw_execute_dft_r2c(const fftw_plan p, double* in, fftw_complex* out) {
	ExecR2c<double>(p, in, &out[0][0]);
}
void fftw_destroy_plan(fftw_plan p) { delete p; }
void fftw_make_planner_thread_safe(void) {}
}

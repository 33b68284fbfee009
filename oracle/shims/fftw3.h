/* Project-written FFTW-API subset.  ORACLE / TEST INFRASTRUCTURE ONLY.
 *
 * The reference's CPU matched filter calls FFTW 3 (src/math/dft.hpp:114-135;
 * CMakeLists.txt:53-55 asks for FFTW >= 3.3.5, not vendored and not installed
 * here).  This header declares the few entry points that file binds, with
 * FFTW's published semantics; oracle/fftw_shim.cpp implements them over the
 * double-precision DFT in oracle/fft64.hpp:
 *   - unnormalised transforms, FFTW_FORWARD = -1 (exp(-2 pi i jk/N)),
 *     FFTW_BACKWARD = +1;
 *   - r2c of length n writes only bins 0..n/2 (n/2+1 complex values);
 *   - plans carry size/sign only, so the new-array execute calls work.
 */
#ifndef UGSDR_ORACLE_FFTW3_SHIM_H
#define UGSDR_ORACLE_FFTW3_SHIM_H

#ifdef __cplusplus
extern "C" {
#endif

typedef float fftwf_complex[2];
typedef double fftw_complex[2];
typedef struct oracle_fftw_plan_s* fftwf_plan;
typedef struct oracle_fftw_plan_s* fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftwf_plan fftwf_plan_dft_1d(int n, fftwf_complex* in, fftwf_complex* out, int sign, unsigned flags);
fftwf_plan fftwf_plan_dft_r2c_1d(int n, float* in, fftwf_complex* out, unsigned flags);
void fftwf_execute_dft(const fftwf_plan p, fftwf_complex* in, fftwf_complex* out);
void fftwf_execute_dft_r2c(const fftwf_plan p, float* in, fftwf_complex* out);
void fftwf_destroy_plan(fftwf_plan p);
void fftwf_make_planner_thread_safe(void);

fftw_plan fftw_plan_dft_1d(int n, fftw_complex* in, fftw_complex* out, int sign, unsigned flags);
fftw_plan fftw_plan_dft_r2c_1d(int n, double* in, fftw_complex* out, unsigned flags);
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out);
void fftw_execute_dft_r2c(const fftw_plan p, double* in, fftw_complex* out);
void fftw_destroy_plan(fftw_plan p);
void fftw_make_planner_thread_safe(void);

#ifdef __cplusplus
}
#endif

#endif

/* fftw3.h -- the FFTW 3 interface the reference's FFT code calls, for compiling the
 * unmodified reference with its FFT drivers (turbulence driving, FFT self-gravity) on a
 * machine without FFTW. Test infrastructure only: the transforms are direct discrete
 * Fourier transforms (fftw3_dft.cpp), unnormalised, with FFTW's sign convention
 * (X_k = sum_j x_j exp(sign 2 pi i j k / n), FFTW_FORWARD = -1), row-major arrays with the
 * last index fastest. Only the calls the reference makes without MPI are implemented;
 * fftw_plan_many_dft (used by its MPI transposes) aborts. */
#ifndef ATHG_TEST_FFTW3_H_
#define ATHG_TEST_FFTW3_H_

#ifdef __cplusplus
extern "C" {
#endif

typedef double fftw_complex[2];
typedef struct athg_test_fftw_plan* fftw_plan;

#define FFTW_FORWARD (-1)
#define FFTW_BACKWARD (+1)
#define FFTW_MEASURE (0U)
#define FFTW_ESTIMATE (1U << 6)

fftw_plan fftw_plan_dft_1d(int n0, fftw_complex* in, fftw_complex* out, int sign,
                           unsigned flags);
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex* in, fftw_complex* out, int sign,
                           unsigned flags);
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex* in, fftw_complex* out,
                           int sign, unsigned flags);
fftw_plan fftw_plan_many_dft(int rank, const int* n, int howmany, fftw_complex* in,
                             const int* inembed, int istride, int idist, fftw_complex* out,
                             const int* onembed, int ostride, int odist, int sign,
                             unsigned flags);
void fftw_execute(const fftw_plan p);
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out);
void fftw_destroy_plan(fftw_plan p);
void fftw_cleanup(void);

#ifdef __cplusplus
}
#endif
#endif

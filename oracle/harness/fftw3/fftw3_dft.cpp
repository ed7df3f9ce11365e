// fftw3_dft.cpp -- direct discrete Fourier transforms behind the FFTW 3 calls of fftw3.h
// (test infrastructure: compiled into the reference by oracle/build_ref.py so that its
// unmodified FFT drivers run here). A d-dimensional transform is d passes of 1-D
// transforms along each axis; each 1-D transform is the defining sum with the twiddle
// factors exp(sign 2 pi i m / n) tabulated once per length (m = j k mod n, so every
// product uses the same rounded table entry), accumulated in index order.
#include "fftw3.h"

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

struct athg_test_fftw_plan {
  int rank;
  int n[3];
  int sign;
  fftw_complex *in, *out;
};

namespace {

void dft_axis(double* a, const int* n, int rank, int axis, int sign) {
  const int len = n[axis];
  long long inner = 1, outer = 1;
  for (int d = axis + 1; d < rank; ++d) inner *= n[d];
  for (int d = 0; d < axis; ++d) outer *= n[d];
  const double pi = 3.14159265358979323846;
  std::vector<double> cw(len), sw(len), xr(len), xi(len);
  for (int m = 0; m < len; ++m) {
    cw[m] = std::cos(2.0 * pi * m / len);
    sw[m] = sign * std::sin(2.0 * pi * m / len);
  }
  for (long long o = 0; o < outer; ++o)
    for (long long q = 0; q < inner; ++q) {
      const long long base = o * len * inner + q;
      for (int j = 0; j < len; ++j) {
        xr[j] = a[2 * (base + j * inner)];
        xi[j] = a[2 * (base + j * inner) + 1];
      }
      for (int k = 0; k < len; ++k) {
        double sr = 0.0, si = 0.0;
        for (int j = 0; j < len; ++j) {
          const int m = (int)(((long long)j * k) % len);
          sr += xr[j] * cw[m] - xi[j] * sw[m];
          si += xr[j] * sw[m] + xi[j] * cw[m];
        }
        a[2 * (base + k * inner)] = sr;
        a[2 * (base + k * inner) + 1] = si;
      }
    }
}

fftw_plan make(int rank, const int* n, fftw_complex* in, fftw_complex* out, int sign) {
  fftw_plan p = new athg_test_fftw_plan;
  p->rank = rank;
  for (int d = 0; d < 3; ++d) p->n[d] = d < rank ? n[d] : 1;
  p->sign = sign;
  p->in = in;
  p->out = out;
  return p;
}

}  // namespace

extern "C" {

fftw_plan fftw_plan_dft_1d(int n0, fftw_complex* in, fftw_complex* out, int sign, unsigned) {
  const int n[1] = {n0};
  return make(1, n, in, out, sign);
}
fftw_plan fftw_plan_dft_2d(int n0, int n1, fftw_complex* in, fftw_complex* out, int sign,
                           unsigned) {
  const int n[2] = {n0, n1};
  return make(2, n, in, out, sign);
}
fftw_plan fftw_plan_dft_3d(int n0, int n1, int n2, fftw_complex* in, fftw_complex* out,
                           int sign, unsigned) {
  const int n[3] = {n0, n1, n2};
  return make(3, n, in, out, sign);
}
fftw_plan fftw_plan_many_dft(int, const int*, int, fftw_complex*, const int*, int, int,
                             fftw_complex*, const int*, int, int, int, unsigned) {
  std::fprintf(stderr, "fftw3 test shim: fftw_plan_many_dft is not implemented\n");
  std::abort();
}
void fftw_execute_dft(const fftw_plan p, fftw_complex* in, fftw_complex* out) {
  long long total = 1;
  for (int d = 0; d < p->rank; ++d) total *= p->n[d];
  std::vector<double> a(2 * total);
  for (long long q = 0; q < total; ++q) {
    a[2 * q] = in[q][0];
    a[2 * q + 1] = in[q][1];
  }
  for (int axis = p->rank - 1; axis >= 0; --axis) dft_axis(a.data(), p->n, p->rank, axis, p->sign);
  for (long long q = 0; q < total; ++q) {
    out[q][0] = a[2 * q];
    out[q][1] = a[2 * q + 1];
  }
}
void fftw_execute(const fftw_plan p) { fftw_execute_dft(p, p->in, p->out); }
void fftw_destroy_plan(fftw_plan p) { delete p; }
void fftw_cleanup(void) {}

}  // extern "C"

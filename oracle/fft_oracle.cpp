// fft_oracle.cpp -- CPU restatement of the reference's FFT-based routines.
//
// TEST INFRASTRUCTURE ONLY (the oracle): the cuFFT implementation is checked against it.
// Parity unpinned against the reference binary: the reference builds these files only
// with FFTW, which is not present here; this restatement follows the reference's source
// line by line, with the same standard-library random engine and distributions, and a
// direct discrete Fourier transform in place of FFTW.
//
// Reference routines followed (paths relative to the reference src/), one FFT block
// covering the whole mesh (one MPI rank):
//   driver          fft/turbulence.cpp:42-135 (seed, global spectrum), Driving :157-178
//   Generate        fft/turbulence.cpp:184-211 (backward transform, RetrieveResult with
//                   the 1/gcnt normalisation of fft/fft_driver.cpp:160-162)
//   OUProcess       fft/turbulence.cpp:221-236
//   PowerSpectrum   fft/turbulence.cpp:244-327
//   Perturb         fft/turbulence.cpp:334-441
//   Project         fft/turbulence.cpp:448-530, GetKcomp :538-541
//   FFT gravity     gravity/fft_gravity.cpp:58-148 (LoadSource, forward transform,
//                   ApplyKernel mode 0, backward transform, RetrieveResult x 4 pi G / gcnt)
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <random>
#include <vector>

namespace {

typedef std::complex<double> cplx;
const double TWO_PI = 6.2831853071795862;

// In-place 3-D DFT of a[i + n1*(j + n2*k)] with exponent sign `sgn` (+1: FFTW_BACKWARD,
// -1: FFTW_FORWARD), unnormalised, as one direct 1-D transform per line and axis
void dft3(std::vector<cplx>* a, int n1, int n2, int n3, int sgn) {
  const int n[3] = {n1, n2, n3};
  const int64_t stride[3] = {1, n1, (int64_t)n1 * n2};
  for (int ax = 0; ax < 3; ++ax) {
    const int N = n[ax];
    std::vector<cplx> w(N), line(N), out(N);
    for (int m = 0; m < N; ++m) {
      const double ang = sgn * TWO_PI * m / N;
      w[m] = cplx(std::cos(ang), std::sin(ang));
    }
    const int o1 = ax == 0 ? 1 : 0, o2 = ax == 2 ? 1 : 2;  // the other two axes
    for (int b = 0; b < n[o2]; ++b)
      for (int c = 0; c < n[o1]; ++c) {
        const int64_t base = b * stride[o2] + c * stride[o1];
        for (int x = 0; x < N; ++x) line[x] = (*a)[base + x * stride[ax]];
        for (int kk = 0; kk < N; ++kk) {
          cplx s(0.0, 0.0);
          for (int x = 0; x < N; ++x) s += line[x] * w[(int64_t)kk * x % N];
          out[kk] = s;
        }
        for (int x = 0; x < N; ++x) (*a)[base + x * stride[ax]] = out[x];
      }
  }
}

int64_t kcomp(int idx, int disp, int Nx) {
  return ((idx + disp) - static_cast<int64_t>(2 * (idx + disp) / Nx) * Nx);
}

struct Turb {
  int n1, n2, n3;
  double len[3];
  int turb_flag, nlow, nhigh;
  double dtdrive, tcorr, f_shear, expo, dedt, tdrive, dvol, dkx[3];
  bool initialized = false;
  std::mt19937_64 rng;
  std::vector<cplx> fv[3], fv_new[3], fv_sh[3], fv_co[3];

  int64_t cnt() const { return (int64_t)n1 * n2 * n3; }

  void power_spectrum(std::vector<cplx>* amp) {
    std::normal_distribution<double> ndist(0.0, 1.0);
    std::uniform_real_distribution<double> udist(0.0, 1.0);
    for (int gk = 0; gk < n3; gk++)
      for (int gj = 0; gj < n2; gj++)
        for (int gi = 0; gi < n1; gi++) {
          const int64_t kidx = gi + (int64_t)n1 * (gj + (int64_t)n2 * gk);
          double A = ndist(rng);
          double ph = udist(rng) * TWO_PI;
          (*amp)[kidx] = A * cplx(std::cos(ph), std::sin(ph));
        }
    double dk = dkx[0];
    if (n2 > 1) dk = dk < dkx[1] ? dk : dkx[1];
    if (n3 > 2) dk = dk < dkx[2] ? dk : dkx[2];
    for (int k = 0; k < n3; k++)
      for (int j = 0; j < n2; j++)
        for (int i = 0; i < n1; i++) {
          int64_t nx = kcomp(i, 0, n1), ny = kcomp(j, 0, n2), nz = kcomp(k, 0, n3);
          double kx = nx * dkx[0], ky = ny * dkx[1], kz = nz * dkx[2];
          double kmag = std::sqrt(kx * kx + ky * ky + kz * kz);
          int64_t gidx = i + (int64_t)n1 * (j + (int64_t)n2 * k);
          double pcoeff;
          if (gidx == 0) {
            pcoeff = 0.0;
          } else {
            if ((kmag / dk > nlow) && (kmag / dk < nhigh))
              pcoeff = 1.0 / std::pow(kmag, (expo + 2.0) / 2.0);
            else
              pcoeff = 0.0;
          }
          (*amp)[gidx] *= pcoeff;
        }
  }

  void project(std::vector<cplx>* f) {
    for (int k = 0; k < n3; k++)
      for (int j = 0; j < n2; j++)
        for (int i = 0; i < n1; i++) {
          int64_t nx = kcomp(i, 0, n1), ny = kcomp(j, 0, n2), nz = kcomp(k, 0, n3);
          double kx = nx * dkx[0], ky = ny * dkx[1], kz = nz * dkx[2];
          double kmag = std::sqrt(kx * kx + ky * ky + kz * kz);
          int64_t kidx = i + (int64_t)n1 * (j + (int64_t)n2 * k);
          if (kidx == 0) {
            for (int nv = 0; nv < 3; ++nv) fv_co[nv][kidx] = fv_sh[nv][kidx] = cplx(0, 0);
          } else {
            kx /= kmag;
            ky /= kmag;
            kz /= kmag;
            cplx kdotf = kx * f[0][kidx] + ky * f[1][kidx] + kz * f[2][kidx];
            fv_co[0][kidx] = kdotf * kx;
            fv_co[1][kidx] = kdotf * ky;
            fv_co[2][kidx] = kdotf * kz;
            for (int nv = 0; nv < 3; ++nv) fv_sh[nv][kidx] = f[nv][kidx] - fv_co[nv][kidx];
          }
        }
    for (int nv = 0; nv < 3; nv++)
      for (int64_t q = 0; q < cnt(); q++)
        f[nv][q] = (1 - f_shear) * fv_co[nv][q] + f_shear * fv_sh[nv][q];
  }

  // Generate + Perturb on u[5][n3][n2][n1] (the mesh's interior cells)
  void generate_perturb(double* u, double dt, double ou_dt) {
    if (!initialized) {
      for (int nv = 0; nv < 3; nv++) power_spectrum(&fv[nv]);
      if (f_shear >= 0) project(fv);
      if (tcorr > 0.) initialized = true;
    } else {
      double factor = std::exp(-ou_dt / tcorr);
      double sqrt_factor = std::sqrt(1 - factor * factor);
      for (int nv = 0; nv < 3; nv++) power_spectrum(&fv_new[nv]);
      if (f_shear >= 0) project(fv_new);
      for (int nv = 0; nv < 3; nv++)
        for (int64_t q = 0; q < cnt(); q++) fv[nv][q] = factor * fv[nv][q] + sqrt_factor * fv_new[nv][q];
    }
    const double norm = 1. / cnt();
    std::vector<double> dv[3];
    for (int nv = 0; nv < 3; nv++) {
      std::vector<cplx> a = fv[nv];
      dft3(&a, n1, n2, n3, +1);
      dv[nv].resize(cnt());
      for (int64_t q = 0; q < cnt(); q++) dv[nv][q] = std::real(a[q]) * norm;
    }
    const int64_t N = cnt();
    double m[4] = {0, 0, 0, 0};
    for (int64_t q = 0; q < N; ++q) {
      double den = u[q];
      m[0] += den;
      m[1] += den * dv[0][q];
      m[2] += den * dv[1][q];
      m[3] += den * dv[2][q];
    }
    for (int64_t q = 0; q < N; ++q) {
      dv[0][q] -= m[1] / m[0];
      dv[1][q] -= m[2] / m[0];
      dv[2][q] -= m[3] / m[0];
    }
    m[0] = m[1] = 0.0;
    for (int64_t q = 0; q < N; ++q) {
      double v1 = dv[0][q], v2 = dv[1][q], v3 = dv[2][q];
      double den = u[q], M1 = u[N + q], M2 = u[2 * N + q], M3 = u[3 * N + q];
      m[0] += den * (v1 * v1 + v2 * v2 + v3 * v3);
      m[1] += M1 * v1 + M2 * v2 + M3 * v3;
    }
    double de = turb_flag > 1 ? dedt * dt : dedt;
    double aa = 0.5 * m[0];
    aa = std::max(aa, static_cast<double>(1.0e-20));
    double b = m[1];
    double c = -de / dvol;
    double s;
    if (b >= 0.0)
      s = (-2.0 * c) / (b + std::sqrt(b * b - 4.0 * aa * c));
    else
      s = (-b + std::sqrt(b * b - 4.0 * aa * c)) / (2.0 * aa);
    for (int64_t q = 0; q < N; ++q) {
      double v1 = dv[0][q], v2 = dv[1][q], v3 = dv[2][q];
      double den = u[q], M1 = u[N + q], M2 = u[2 * N + q], M3 = u[3 * N + q];
      u[4 * N + q] += s * (M1 * v1 + M2 * v2 + M3 * v3) + 0.5 * s * s * den * (v1 * v1 + v2 * v2 + v3 * v3);
      u[N + q] += s * den * v1;
      u[2 * N + q] += s * den * v2;
      u[3 * N + q] += s * den * v3;
    }
  }
};

}  // namespace

extern "C" {

// cfg: turb_flag, nlow, nhigh; dcfg: dtdrive, tcorr, f_shear, expo, dedt
void* orc_turb_create(int n1, int n2, int n3, const double* len, const int* cfg,
                      const double* dcfg, int64_t rseed, double time) {
  Turb* t = new Turb();
  t->n1 = n1; t->n2 = n2; t->n3 = n3;
  for (int d = 0; d < 3; ++d) t->len[d] = len[d];
  t->turb_flag = cfg[0]; t->nlow = cfg[1]; t->nhigh = cfg[2];
  t->dtdrive = dcfg[0]; t->tcorr = dcfg[1]; t->f_shear = dcfg[2]; t->expo = dcfg[3];
  t->dedt = dcfg[4];
  t->tdrive = time;
  const double dx1 = len[0] / static_cast<double>(n1), dx2 = len[1] / static_cast<double>(n2),
               dx3 = len[2] / static_cast<double>(n3);
  t->dvol = dx1 * dx2 * dx3;
  for (int d = 0; d < 3; ++d) t->dkx[d] = TWO_PI / len[d];
  t->rng.seed(rseed);
  for (int nv = 0; nv < 3; ++nv) {
    t->fv[nv].assign(t->cnt(), cplx(0, 0));
    t->fv_new[nv].assign(t->cnt(), cplx(0, 0));
    t->fv_sh[nv].assign(t->cnt(), cplx(0, 0));
    t->fv_co[nv].assign(t->cnt(), cplx(0, 0));
  }
  return t;
}

void orc_turb_destroy(void* h) { delete static_cast<Turb*>(h); }

// TurbulenceDriver::Driving at (time, dt) on the mesh's interior conserved variables
void orc_turb_drive(void* h, double* u, double time, double dt) {
  Turb* t = static_cast<Turb*>(h);
  switch (t->turb_flag) {
    case 1:
      t->generate_perturb(u, 0.0, 0.0);
      break;
    case 2:
      if (time >= t->tdrive) {
        t->tdrive = time + t->dtdrive;
        t->generate_perturb(u, t->dtdrive, t->dtdrive);
      }
      break;
    default:
      t->generate_perturb(u, dt, dt);
  }
}

// FFTGravityDriver::Solve on the whole mesh: rho[n3][n2][n1] -> phi[n3][n2][n1]
void orc_fft_gravity(int n1, int n2, int n3, const double* len, double four_pi_G,
                     const double* rho, double* phi) {
  const int64_t N = (int64_t)n1 * n2 * n3;
  std::vector<cplx> a(N);
  for (int64_t q = 0; q < N; ++q) a[q] = cplx(rho[q], 0.0);
  dft3(&a, n1, n2, n3, -1);
  const int kNx[3] = {n1, n2, n3};
  double dkx[3];
  for (int d = 0; d < 3; ++d) dkx[d] = TWO_PI / len[d];
  double dx1sq = (TWO_PI / (kNx[0] * dkx[0])) * (TWO_PI / (kNx[0] * dkx[0]));
  double dx2sq = (TWO_PI / (kNx[1] * dkx[1])) * (TWO_PI / (kNx[1] * dkx[1]));
  double dx3sq = (TWO_PI / (kNx[2] * dkx[2])) * (TWO_PI / (kNx[2] * dkx[2]));
  for (int k = 0; k < n3; k++)
    for (int j = 0; j < n2; j++)
      for (int i = 0; i < n1; i++) {
        int64_t gidx = i + (int64_t)n1 * (j + (int64_t)n2 * k);
        double pcoeff;
        if (gidx == 0) {
          pcoeff = 0.0;
        } else {
          double kx = i, ky = j, kz = k;
          if (kx > 0.5 * kNx[0]) kx -= kNx[0];
          if (ky > 0.5 * kNx[1]) ky -= kNx[1];
          if (kz > 0.5 * kNx[2]) kz -= kNx[2];
          kx *= TWO_PI / static_cast<double>(kNx[0]);
          ky *= TWO_PI / static_cast<double>(kNx[1]);
          kz *= TWO_PI / static_cast<double>(kNx[2]);
          pcoeff = ((2.0 * std::cos(kx) - 2.0) / dx1sq);
          pcoeff += ((2.0 * std::cos(ky) - 2.0) / dx2sq);
          pcoeff += ((2.0 * std::cos(kz) - 2.0) / dx3sq);
          pcoeff = 1.0 / pcoeff;
        }
        a[gidx] = pcoeff * a[gidx];
      }
  dft3(&a, n1, n2, n3, +1);
  const double norm = four_pi_G / N;
  for (int64_t q = 0; q < N; ++q) phi[q] = std::real(a[q]) * norm;
}

}  // extern "C"

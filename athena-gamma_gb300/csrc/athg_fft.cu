// athg_fft.cu -- turbulence driving and FFT self-gravity on cuFFT (declarations and the
// reference functions each part follows: athg_fft.h). Built without FMA contraction, so
// the per-cell arithmetic rounds like the reference's scalar FP64 code; the transforms
// themselves (cuFFT against FFTW) and the order of the global sums differ at round-off.
#include <cufft.h>

#include <algorithm>
#include <cmath>
#include <complex>
#include <random>
#include <vector>

#include "athg_fft.h"
#include "athg_numeric.h"

namespace athg {
namespace {

constexpr double kTwoPi = 6.2831853071795862;  // TWO_PI of athena.hpp
constexpr int kThreads = 256;

const char* cufft_msg(cufftResult r) {
  switch (r) {
    case CUFFT_SUCCESS: return "success";
    case CUFFT_ALLOC_FAILED: return "allocation failed";
    case CUFFT_INVALID_VALUE: return "invalid value";
    case CUFFT_EXEC_FAILED: return "execution failed";
    case CUFFT_SETUP_FAILED: return "setup failed";
    case CUFFT_INVALID_SIZE: return "invalid size";
    default: return "error";
  }
}

bool cu_ok(cudaError_t e, const char* what, std::string* err) {
  if (e == cudaSuccess) return true;
  *err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

bool fft_ok(cufftResult r, const char* what, std::string* err) {
  if (r == CUFFT_SUCCESS) return true;
  *err = std::string(what) + ": cuFFT " + cufft_msg(r);
  return false;
}

// position of interior cell (k, j, i) of block b in the mesh-wide FFT array (i fastest)
__device__ inline int64_t mesh_index(const int* boff, int b, int k, int j, int i, int n1, int n2) {
  const int64_t I = boff[3 * b] + i, J = boff[3 * b + 1] + j, K = boff[3 * b + 2] + k;
  return (K * n2 + J) * n1 + I;
}

// Sum of `nv` values over the threads of a block into part[blockid * nv + v], in a fixed
// order (deterministic)
template <int NV>
__device__ inline void block_sum(double (&v)[NV], double* part) {
  __shared__ double sh[NV][kThreads];
  const int t = threadIdx.x;
  for (int q = 0; q < NV; ++q) sh[q][t] = v[q];
  __syncthreads();
  for (int s = kThreads / 2; s > 0; s >>= 1) {
    if (t < s)
      for (int q = 0; q < NV; ++q) sh[q][t] += sh[q][t + s];
    __syncthreads();
  }
  if (t == 0) {
    const int64_t bid = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
    for (int q = 0; q < NV; ++q) part[bid * NV + q] = sh[q][0];
  }
}

// ---- FFT self-gravity ----------------------------------------------------------------

// FFTBlock::LoadSource of u(IDN) (athena_fft.cpp:169-203): real input
__global__ void k_fg_gather(Geom g, const double* __restrict__ u, const int* __restrict__ boff,
                            double* __restrict__ r, int n1, int n2) {
  const int b = blockIdx.z, k = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nx1 * g.nx2) return;
  const int j = t / g.nx1, i = t - j * g.nx1;
  r[mesh_index(boff, b, k, j, i, n1, n2)] =
      u[(int64_t)b * NHYD * g.ncell + cidx(g, k + g.ks, j + g.js, i + g.is)];
}

// FFTGravity::ApplyKernel, mode 0 (fft_gravity.cpp:105-148) on the half spectrum of a real
// transform: t1/t2/t3 hold (2 cos(k) - 2) / dx^2 per wavenumber of each axis
__global__ void k_fg_kernel(cufftDoubleComplex* __restrict__ c, const double* __restrict__ t1,
                            const double* __restrict__ t2, const double* __restrict__ t3,
                            int h1, int n2, int n3) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t tot = (int64_t)h1 * n2 * n3;
  if (q >= tot) return;
  const int i = (int)(q % h1);
  const int j = (int)((q / h1) % n2);
  const int k = (int)(q / ((int64_t)h1 * n2));
  double pcoeff = 0.0;
  if (i != 0 || j != 0 || k != 0) {
    pcoeff = t1[i];
    pcoeff += t2[j];
    pcoeff += t3[k];
    pcoeff = 1.0 / pcoeff;
  }
  cufftDoubleComplex v = c[q];
  v.x = pcoeff * v.x;
  v.y = pcoeff * v.y;
  c[q] = v;
}

// FFTBlock::RetrieveResult (athena_fft.cpp:133-162) times the normalisation, plus the one
// ghost layer the gravity boundary exchange fills from the periodic neighbours (and, for
// the mixed path's source term, the same potential as FP32 pairs in phi2)
__global__ void k_fg_scatter(Geom g, double* __restrict__ phi, float2* __restrict__ phi2,
                             const int* __restrict__ boff, const double* __restrict__ r, int n1,
                             int n2, int n3, double norm) {
  const int b = blockIdx.z, k = blockIdx.y;  // k over nx3 + 2
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int w1 = g.nx1 + 2, w2 = g.nx2 + 2;
  if (t >= w1 * w2) return;
  const int j = t / w1, i = t - j * w1;
  int I = boff[3 * b] + i - 1, J = boff[3 * b + 1] + j - 1, K = boff[3 * b + 2] + k - 1;
  I = (I + n1) % n1;
  J = (J + n2) % n2;
  K = (K + n3) % n3;
  const int64_t q = (int64_t)b * g.ncell + cidx(g, k + g.ks - 1, j + g.js - 1, i + g.is - 1);
  const double v = r[((int64_t)K * n2 + J) * n1 + I] * norm;
  phi[q] = v;
  if (phi2) {
    const ff f = split_ff(v);
    phi2[q] = make_float2(f.hi, f.lo);
  }
}

// ---- turbulence ----------------------------------------------------------------------

// the non-zero modes of the three spectra into the zeroed mesh-wide arrays
__global__ void k_turb_scatter(cufftDoubleComplex* __restrict__ grid, int64_t ncell,
                               const int64_t* __restrict__ idx, const double2* __restrict__ amp,
                               int64_t m) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= 3 * m) return;
  const int nv = (int)(q / m);
  const int64_t p = q - nv * m;
  const double2 a = amp[q];
  grid[nv * ncell + idx[p]] = make_cuDoubleComplex(a.x, a.y);
}

// TurbulenceDriver::Perturb (turbulence.cpp:306-441), sums over the interior of every
// block. PASS 1: density and density-weighted perturbation; PASS 2: with the mean
// removed, rho |dv|^2 and M.dv. dv = Re(transform) * norm (RetrieveResult).
template <int PASS>
__global__ void k_turb_sum(Geom g, const double* __restrict__ u, const int* __restrict__ boff,
                           const cufftDoubleComplex* __restrict__ grid, int64_t ncell, int n1,
                           int n2, double norm, const double* __restrict__ q,
                           double* __restrict__ part) {
  const int b = blockIdx.z, k = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  constexpr int NV = PASS == 1 ? 4 : 2;
  double v[NV];
  for (int s = 0; s < NV; ++s) v[s] = 0.0;
  if (t < g.nx1 * g.nx2) {
    const int j = t / g.nx1, i = t - j * g.nx1;
    const int64_t gi = mesh_index(boff, b, k, j, i, n1, n2);
    const int64_t c = (int64_t)b * NHYD * g.ncell + cidx(g, k + g.ks, j + g.js, i + g.is);
    double d1 = grid[gi].x * norm, d2 = grid[ncell + gi].x * norm,
           d3 = grid[2 * ncell + gi].x * norm;
    const double den = u[c];
    if (PASS == 1) {
      v[0] = den;
      v[1] = den * d1;
      v[2] = den * d2;
      v[NV > 3 ? 3 : 0] = den * d3;
    } else {
      d1 -= q[0];
      d2 -= q[1];
      d3 -= q[2];
      const double M1 = u[c + g.ncell], M2 = u[c + 2 * g.ncell], M3 = u[c + 3 * g.ncell];
      v[0] = den * (d1 * d1 + d2 * d2 + d3 * d3);
      v[1] = M1 * d1 + M2 * d2 + M3 * d3;
    }
  }
  block_sum<NV>(v, part);
}

// The partial sums in a fixed order; PASS 1 stores the mean perturbation m[1..3] / m[0],
// PASS 2 the scale s solving (1/2) m0 s^2 + m1 s = de / dvol (turbulence.cpp:395-413).
template <int PASS>
__global__ void k_turb_final(const double* __restrict__ part, int64_t nparts,
                             double* __restrict__ q, double de, double dvol) {
  constexpr int NV = PASS == 1 ? 4 : 2;
  __shared__ double sh[NV][1024];
  const int t = threadIdx.x;
  double v[NV];
  for (int s = 0; s < NV; ++s) v[s] = 0.0;
  for (int64_t p = t; p < nparts; p += blockDim.x)
    for (int s = 0; s < NV; ++s) v[s] += part[p * NV + s];
  for (int s = 0; s < NV; ++s) sh[s][t] = v[s];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w)
      for (int s = 0; s < NV; ++s) sh[s][t] += sh[s][t + w];
    __syncthreads();
  }
  if (t != 0) return;
  if (PASS == 1) {
    q[0] = sh[1][0] / sh[0][0];
    q[1] = sh[2][0] / sh[0][0];
    q[2] = sh[NV > 3 ? 3 : 0][0] / sh[0][0];
  } else {
    double aa = 0.5 * sh[0][0];
    aa = fmax(aa, 1.0e-20);
    const double bb = sh[1][0];
    const double cc = -de / dvol;
    double s;
    if (bb >= 0.0)
      s = (-2.0 * cc) / (bb + sqrt(bb * bb - 4.0 * aa * cc));
    else
      s = (-bb + sqrt(bb * bb - 4.0 * aa * cc)) / (2.0 * aa);
    q[3] = s;
  }
}

// the momentum and energy perturbation of every interior cell (turbulence.cpp:418-440)
__global__ void k_turb_apply(Geom g, double* __restrict__ u, const int* __restrict__ boff,
                             const cufftDoubleComplex* __restrict__ grid, int64_t ncell, int n1,
                             int n2, double norm, const double* __restrict__ q) {
  const int b = blockIdx.z, k = blockIdx.y;
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nx1 * g.nx2) return;
  const int j = t / g.nx1, i = t - j * g.nx1;
  const int64_t gi = mesh_index(boff, b, k, j, i, n1, n2);
  const int64_t c = (int64_t)b * NHYD * g.ncell + cidx(g, k + g.ks, j + g.js, i + g.is);
  const double v1 = grid[gi].x * norm - q[0];
  const double v2 = grid[ncell + gi].x * norm - q[1];
  const double v3 = grid[2 * ncell + gi].x * norm - q[2];
  const double s = q[3];
  const double den = u[c];
  const double M1 = u[c + g.ncell], M2 = u[c + 2 * g.ncell], M3 = u[c + 3 * g.ncell];
  u[c + IEN * g.ncell] += s * (M1 * v1 + M2 * v2 + M3 * v3) +
                          0.5 * s * s * den * (v1 * v1 + v2 * v2 + v3 * v3);
  u[c + g.ncell] += s * den * v1;
  u[c + 2 * g.ncell] += s * den * v2;
  u[c + 3 * g.ncell] += s * den * v3;
}

// TurbulenceDriver::GetKcomp (turbulence.cpp:538-541)
int64_t kcomp(int idx, int nx) {
  return (int64_t)idx - (int64_t)(2 * (int64_t)idx / nx) * nx;
}

}  // namespace

// ---- FFT self-gravity ----------------------------------------------------------------

struct FftGravity {
  FftMesh m{};
  int64_t ncell = 0, nhalf = 0;
  double norm = 0.0;
  cufftHandle fwd = 0, inv = 0;
  bool have_fwd = false, have_inv = false;
  double* r = nullptr;
  cufftDoubleComplex* c = nullptr;
  double *t1 = nullptr, *t2 = nullptr, *t3 = nullptr;
};

void fftgrav_destroy(FftGravity* f) {
  if (!f) return;
  if (f->have_fwd) cufftDestroy(f->fwd);
  if (f->have_inv) cufftDestroy(f->inv);
  cudaFree(f->r);
  cudaFree(f->c);
  cudaFree(f->t1);
  cudaFree(f->t2);
  cudaFree(f->t3);
  delete f;
}

int fftgrav_create(const FftMesh& m, double four_pi_G, FftGravity** out, std::string* err) {
  FftGravity* f = new FftGravity();
  f->m = m;
  const int n1 = m.n[0], n2 = m.n[1], n3 = m.n[2], h1 = n1 / 2 + 1;
  f->ncell = (int64_t)n1 * n2 * n3;
  f->nhalf = (int64_t)h1 * n2 * n3;
  const int64_t gcnt = f->ncell;
  f->norm = four_pi_G / gcnt;  // SetNormFactor(four_pi_G_ / gcnt_)
  // per-axis terms of the discrete Laplacian's eigenvalue, with the reference's
  // expressions: dkx = 2 pi / L, dx^2 = (2 pi / (N dkx))^2, k -> k - N above N/2
  std::vector<double> t[3];
  for (int a = 0; a < 3; ++a) {
    const int N = m.n[a];
    const double dkx = kTwoPi / m.len[a];
    const double dxsq = (kTwoPi / (N * dkx)) * (kTwoPi / (N * dkx));
    const int cnt = a == 0 ? h1 : N;
    t[a].resize(cnt);
    for (int i = 0; i < cnt; ++i) {
      double kx = i;
      if (kx > 0.5 * N) kx -= N;
      kx *= kTwoPi / static_cast<double>(N);
      t[a][i] = (2.0 * std::cos(kx) - 2.0) / dxsq;
    }
  }
  bool ok = cu_ok(cudaMalloc(&f->r, sizeof(double) * f->ncell), "fft gravity", err) &&
            cu_ok(cudaMalloc(&f->c, sizeof(cufftDoubleComplex) * f->nhalf), "fft gravity", err) &&
            cu_ok(cudaMalloc(&f->t1, sizeof(double) * h1), "fft gravity", err) &&
            cu_ok(cudaMalloc(&f->t2, sizeof(double) * n2), "fft gravity", err) &&
            cu_ok(cudaMalloc(&f->t3, sizeof(double) * n3), "fft gravity", err);
  ok = ok && cu_ok(cudaMemcpy(f->t1, t[0].data(), sizeof(double) * h1, cudaMemcpyHostToDevice),
                   "fft gravity", err) &&
       cu_ok(cudaMemcpy(f->t2, t[1].data(), sizeof(double) * n2, cudaMemcpyHostToDevice),
             "fft gravity", err) &&
       cu_ok(cudaMemcpy(f->t3, t[2].data(), sizeof(double) * n3, cudaMemcpyHostToDevice),
             "fft gravity", err);
  if (ok) {
    ok = fft_ok(cufftPlan3d(&f->fwd, n3, n2, n1, CUFFT_D2Z), "forward plan", err);
    f->have_fwd = ok;
  }
  if (ok) {
    ok = fft_ok(cufftPlan3d(&f->inv, n3, n2, n1, CUFFT_Z2D), "backward plan", err);
    f->have_inv = ok;
  }
  if (!ok) {
    fftgrav_destroy(f);
    return -1;
  }
  *out = f;
  return 0;
}

int fftgrav_solve(FftGravity* f, const Geom& g, int nb, const double* u, const int* boff,
                  double* phi, float2* phi2, cudaStream_t st, std::string* err) {
  const int n1 = f->m.n[0], n2 = f->m.n[1], n3 = f->m.n[2];
  dim3 gg((unsigned)((g.nx1 * g.nx2 + kThreads - 1) / kThreads), (unsigned)g.nx3, (unsigned)nb);
  k_fg_gather<<<gg, kThreads, 0, st>>>(g, u, boff, f->r, n1, n2);
  if (!cu_ok(cudaGetLastError(), "fft gravity gather", err)) return -1;
  if (!fft_ok(cufftSetStream(f->fwd, st), "stream", err) ||
      !fft_ok(cufftExecD2Z(f->fwd, f->r, f->c), "forward transform", err))
    return -1;
  k_fg_kernel<<<(unsigned)((f->nhalf + kThreads - 1) / kThreads), kThreads, 0, st>>>(
      f->c, f->t1, f->t2, f->t3, n1 / 2 + 1, n2, n3);
  if (!cu_ok(cudaGetLastError(), "fft gravity kernel", err)) return -1;
  if (!fft_ok(cufftSetStream(f->inv, st), "stream", err) ||
      !fft_ok(cufftExecZ2D(f->inv, f->c, f->r), "backward transform", err))
    return -1;
  dim3 gs((unsigned)(((g.nx1 + 2) * (g.nx2 + 2) + kThreads - 1) / kThreads),
          (unsigned)(g.nx3 + 2), (unsigned)nb);
  k_fg_scatter<<<gs, kThreads, 0, st>>>(g, phi, phi2, boff, f->r, n1, n2, n3, f->norm);
  if (!cu_ok(cudaGetLastError(), "fft gravity scatter", err)) return -1;
  return 0;
}

// ---- turbulence driving --------------------------------------------------------------

struct Turb {
  athg_turb_config cfg{};
  FftMesh m{};
  int64_t ncell = 0;
  double dvol = 0.0, norm = 0.0, tdrive = 0.0;
  bool initialized = false, global_ps = false;
  std::mt19937_64 rng;
  // the modes the power law keeps (ascending mesh-wide index) and their coefficients
  std::vector<int64_t> idx;
  std::vector<double> pcoeff;
  std::vector<double> kvec;                   // 3 per mode: kx, ky, kz
  std::vector<std::complex<double>> fv[3];    // the driver's spectrum on those modes
  std::vector<double2> amp;                   // upload buffer, 3 x modes
  cufftHandle plan = 0;
  bool have_plan = false;
  cufftDoubleComplex* grid = nullptr;  // 3 mesh-wide complex arrays
  int64_t* didx = nullptr;
  double2* damp = nullptr;
  double* part = nullptr;
  int64_t npart = 0;
  double* q = nullptr;  // mean perturbation (3), scale s
};

void turb_destroy(Turb* t) {
  if (!t) return;
  if (t->have_plan) cufftDestroy(t->plan);
  cudaFree(t->grid);
  cudaFree(t->didx);
  cudaFree(t->damp);
  cudaFree(t->part);
  cudaFree(t->q);
  delete t;
}

int turb_flag(const Turb* t) { return t->cfg.turb_flag; }

int turb_create(const FftMesh& m, const athg_turb_config& cfg, double time, Turb** out,
                std::string* err) {
  if (cfg.turb_flag < 1 || cfg.turb_flag > 3) {
    *err = "turb_flag must be 1, 2 or 3";
    return 1;
  }
  if (cfg.f_shear > 1) {
    *err = "The ratio between shear and compressible components should be less than one";
    return 1;
  }
  if ((cfg.turb_flag == 2 && !(cfg.dtdrive > 0.0)) || (cfg.turb_flag > 1 && !(cfg.tcorr >= 0.0))) {
    *err = "driven turbulence needs dtdrive (turb_flag 2) and tcorr";
    return 1;
  }
  Turb* t = new Turb();
  t->cfg = cfg;
  t->m = m;
  const int n1 = m.n[0], n2 = m.n[1], n3 = m.n[2];
  t->ncell = (int64_t)n1 * n2 * n3;
  t->tdrive = time;
  // FFTBlock dx (mesh size / cells) and the normalisation 1 / gcnt of InitializeFFTBlock(true)
  const double dx1 = m.len[0] / static_cast<double>(n1), dx2 = m.len[1] / static_cast<double>(n2),
               dx3 = m.len[2] / static_cast<double>(n3);
  t->dvol = dx1 * dx2 * dx3;
  t->norm = 1. / t->ncell;
  // random sequence (turbulence.cpp:115-133): a given seed draws the whole mesh's spectrum
  int64_t seed = cfg.rseed;
  if (seed < 0) {
    std::random_device device;
    seed = static_cast<int64_t>(device());
  } else {
    t->global_ps = true;
  }
  t->rng.seed(seed);
  // power-law coefficients (PowerSpectrum, turbulence.cpp:290-324)
  const double dk[3] = {kTwoPi / m.len[0], kTwoPi / m.len[1], kTwoPi / m.len[2]};
  double dkx = dk[0];
  if (n2 > 1) dkx = dkx < dk[1] ? dkx : dk[1];
  if (n3 > 2) dkx = dkx < dk[2] ? dkx : dk[2];
  for (int k = 0; k < n3; ++k)
    for (int j = 0; j < n2; ++j)
      for (int i = 0; i < n1; ++i) {
        const int64_t nx = kcomp(i, n1), ny = kcomp(j, n2), nz = kcomp(k, n3);
        const double kx = nx * dk[0], ky = ny * dk[1], kz = nz * dk[2];
        const double kmag = std::sqrt(kx * kx + ky * ky + kz * kz);
        const int64_t gidx = i + (int64_t)n1 * (j + (int64_t)n2 * k);
        double pc = 0.0;
        if (gidx != 0 && (kmag / dkx > cfg.nlow) && (kmag / dkx < cfg.nhigh))
          pc = 1.0 / std::pow(kmag, (cfg.expo + 2.0) / 2.0);
        if (pc != 0.0) {
          t->idx.push_back(gidx);
          t->pcoeff.push_back(pc);
          t->kvec.push_back(kx);
          t->kvec.push_back(ky);
          t->kvec.push_back(kz);
        }
      }
  const int64_t nm = (int64_t)t->idx.size();
  for (int nv = 0; nv < 3; ++nv) t->fv[nv].assign(nm, std::complex<double>(0.0, 0.0));
  t->amp.resize(3 * std::max<int64_t>(nm, 1));
  bool ok = cu_ok(cudaMalloc(&t->grid, sizeof(cufftDoubleComplex) * 3 * t->ncell), "turbulence", err) &&
            cu_ok(cudaMalloc(&t->didx, sizeof(int64_t) * std::max<int64_t>(nm, 1)), "turbulence", err) &&
            cu_ok(cudaMalloc(&t->damp, sizeof(double2) * 3 * std::max<int64_t>(nm, 1)), "turbulence", err) &&
            cu_ok(cudaMalloc(&t->q, sizeof(double) * 4), "turbulence", err);
  if (ok && nm > 0)
    ok = cu_ok(cudaMemcpy(t->didx, t->idx.data(), sizeof(int64_t) * nm, cudaMemcpyHostToDevice),
               "turbulence", err);
  if (ok) {
    int n[3] = {n3, n2, n1};
    ok = fft_ok(cufftPlanMany(&t->plan, 3, n, nullptr, 1, (int)t->ncell, nullptr, 1,
                              (int)t->ncell, CUFFT_Z2Z, 3),
                "backward plan", err);
    t->have_plan = ok;
  }
  if (!ok) {
    turb_destroy(t);
    return -1;
  }
  *out = t;
  return 0;
}

namespace {

// PowerSpectrum (turbulence.cpp:244-327) on the kept modes: a Gaussian amplitude and a
// uniform phase drawn for every mode of the mesh in index order (fresh distributions per
// call, as the reference constructs them), times the power-law coefficient
void power_spectrum(Turb* t, std::vector<std::complex<double>>* amp) {
  std::normal_distribution<double> ndist(0.0, 1.0);
  std::uniform_real_distribution<double> udist(0.0, 1.0);
  const int64_t nm = (int64_t)t->idx.size();
  int64_t p = 0;
  for (int64_t g = 0; g < t->ncell; ++g) {
    const double A = ndist(t->rng);
    const double ph = udist(t->rng) * kTwoPi;
    if (p < nm && t->idx[p] == g) {
      std::complex<double> a = A * std::complex<double>(std::cos(ph), std::sin(ph));
      a *= t->pcoeff[p];
      (*amp)[p] = a;
      ++p;
    }
  }
}

// Project(fv, f_shear) (turbulence.cpp:448-530): compressive part along k-hat, shear part
// the rest, recombined with the ratio f_shear
void project(Turb* t, std::vector<std::complex<double>>* fv, double f_shear) {
  const int64_t nm = (int64_t)t->idx.size();
  for (int64_t p = 0; p < nm; ++p) {
    double kx = t->kvec[3 * p], ky = t->kvec[3 * p + 1], kz = t->kvec[3 * p + 2];
    const double kmag = std::sqrt(kx * kx + ky * ky + kz * kz);
    kx /= kmag;
    ky /= kmag;
    kz /= kmag;
    const std::complex<double> kdotf = kx * fv[0][p] + ky * fv[1][p] + kz * fv[2][p];
    const std::complex<double> co[3] = {kdotf * kx, kdotf * ky, kdotf * kz};
    for (int nv = 0; nv < 3; ++nv) {
      const std::complex<double> sh = fv[nv][p] - co[nv];
      fv[nv][p] = (1 - f_shear) * co[nv] + f_shear * sh;
    }
  }
}

}  // namespace

int turb_drive(Turb* t, const Geom& g, int nb, double* u, const int* boff, double time,
               double dt, cudaStream_t st, std::string* err) {
  const athg_turb_config& c = t->cfg;
  double pdt;  // the dt Perturb scales dedt with (0: decaying, all at once)
  if (c.turb_flag == 1) {
    pdt = 0.0;
  } else if (c.turb_flag == 2) {
    if (!(time >= t->tdrive)) return 0;
    t->tdrive = time + c.dtdrive;
    pdt = c.dtdrive;
  } else {
    pdt = dt;
  }
  // Generate (turbulence.cpp:176-211): the spectrum, projected, smoothed in time by the
  // Ornstein-Uhlenbeck process once initialised
  const int64_t nm = (int64_t)t->idx.size();
  if (!t->initialized) {
    for (int nv = 0; nv < 3; ++nv) power_spectrum(t, &t->fv[nv]);
    if (c.f_shear >= 0) project(t, t->fv, c.f_shear);
    if (c.tcorr > 0.) t->initialized = true;
  } else {
    const double OUdt = c.turb_flag == 2 ? c.dtdrive : dt;
    const double factor = std::exp(-OUdt / c.tcorr);
    const double sqrt_factor = std::sqrt(1 - factor * factor);
    std::vector<std::complex<double>> fnew[3];
    for (int nv = 0; nv < 3; ++nv) {
      fnew[nv].assign(nm, std::complex<double>(0.0, 0.0));
      power_spectrum(t, &fnew[nv]);
    }
    if (c.f_shear >= 0) project(t, fnew, c.f_shear);
    for (int nv = 0; nv < 3; ++nv)
      for (int64_t p = 0; p < nm; ++p) t->fv[nv][p] = factor * t->fv[nv][p] + sqrt_factor * fnew[nv][p];
  }
  for (int nv = 0; nv < 3; ++nv)
    for (int64_t p = 0; p < nm; ++p)
      t->amp[nv * nm + p] = make_double2(t->fv[nv][p].real(), t->fv[nv][p].imag());
  // the three transforms (FFTW_BACKWARD, unnormalised) of the mesh-wide spectra
  if (!cu_ok(cudaMemsetAsync(t->grid, 0, sizeof(cufftDoubleComplex) * 3 * t->ncell, st),
             "turbulence", err))
    return -1;
  if (nm > 0) {
    if (!cu_ok(cudaMemcpyAsync(t->damp, t->amp.data(), sizeof(double2) * 3 * nm,
                               cudaMemcpyHostToDevice, st), "turbulence", err))
      return -1;
    k_turb_scatter<<<(unsigned)((3 * nm + kThreads - 1) / kThreads), kThreads, 0, st>>>(
        t->grid, t->ncell, t->didx, t->damp, nm);
    if (!cu_ok(cudaGetLastError(), "turbulence scatter", err)) return -1;
  }
  if (!fft_ok(cufftSetStream(t->plan, st), "stream", err) ||
      !fft_ok(cufftExecZ2Z(t->plan, t->grid, t->grid, CUFFT_INVERSE), "backward transform", err))
    return -1;
  // Perturb: mean removal, energy normalisation, momentum and energy kick
  dim3 gg((unsigned)((g.nx1 * g.nx2 + kThreads - 1) / kThreads), (unsigned)g.nx3, (unsigned)nb);
  const int64_t np = (int64_t)gg.x * gg.y * gg.z;
  if (np > t->npart) {
    cudaFree(t->part);
    t->part = nullptr;
    if (!cu_ok(cudaMalloc(&t->part, sizeof(double) * 4 * np), "turbulence", err)) return -1;
    t->npart = np;
  }
  const int n1 = t->m.n[0], n2 = t->m.n[1];
  k_turb_sum<1><<<gg, kThreads, 0, st>>>(g, u, boff, t->grid, t->ncell, n1, n2, t->norm, nullptr,
                                         t->part);
  k_turb_final<1><<<1, 1024, 0, st>>>(t->part, np, t->q, 0.0, t->dvol);
  k_turb_sum<2><<<gg, kThreads, 0, st>>>(g, u, boff, t->grid, t->ncell, n1, n2, t->norm, t->q,
                                         t->part);
  const double de = c.turb_flag > 1 ? c.dedt * pdt : c.dedt;
  k_turb_final<2><<<1, 1024, 0, st>>>(t->part, np, t->q, de, t->dvol);
  k_turb_apply<<<gg, kThreads, 0, st>>>(g, u, boff, t->grid, t->ncell, n1, n2, t->norm, t->q);
  if (!cu_ok(cudaGetLastError(), "turbulence perturb", err)) return -1;
  return 0;
}

}  // namespace athg

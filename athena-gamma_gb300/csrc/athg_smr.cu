// athg_smr.cu -- device side of static mesh refinement: one generic kernel per work list
// (athg_smr.h, planned by athg_smr_plan.cpp). Built without FMA contraction, like the
// FP64 stage, so that every list reproduces the reference's FP64 arithmetic.
#include <cuda_runtime.h>

#include "athg_internal.h"

namespace athg {

namespace {

constexpr int kThreads = 256;

unsigned grid_of(int64_t n) { return (unsigned)((n + kThreads - 1) / kThreads); }

__global__ void k_smr_xfer(SmrDims d, SmrPool P, const SmrXfer* __restrict__ x, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) smr_exec_xfer(d, P, x[t]);
}
__global__ void k_smr_flux(SmrDims d, SmrPool P, const SmrFlux* __restrict__ f, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) smr_exec_flux(d, P, f[t]);
}
__global__ void k_smr_emf_eval(SmrDims d, SmrPool P, const SmrEmf* __restrict__ e,
                               const SmrEmfAdd* __restrict__ a, int64_t n,
                               double* __restrict__ tmp) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) tmp[t] = smr_exec_emf(d, P, e[t], a);
}
__global__ void k_smr_emf_store(SmrDims d, SmrPool P, const SmrEmf* __restrict__ e, int64_t n,
                                const double* __restrict__ tmp) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int64_t q = ((int64_t)e[t].blk * 3 + e[t].comp) * d.ne + e[t].idx;
  if (P.edge32) P.edge32[q] = (float)tmp[t];
  else P.edge[q] = tmp[t];
}
__global__ void k_smr_c2p(SmrDims d, SmrPool P, const SmrPos* __restrict__ p, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) smr_exec_c2p(d, P, p[t]);
}
__global__ void k_smr_pcc(SmrDims d, SmrPool P, const SmrPos* __restrict__ p, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) smr_exec_pcc(d, P, p[t]);
}
__global__ void k_smr_psf(SmrDims d, SmrPool P, int f, const SmrPos* __restrict__ p, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) smr_exec_psf(d, P, f, p[t]);
}
__global__ void k_smr_pint(SmrDims d, SmrPool P, const SmrPos* __restrict__ p, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) smr_exec_pint(d, P, p[t]);
}
__global__ void k_smr_pfine(SmrDims d, SmrPool P, const SmrPos* __restrict__ p, int64_t n) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) smr_exec_pfine(d, P, p[t]);
}

template <typename T>
cudaError_t upload(T** dst, const std::vector<T>& src, int64_t* n, cudaStream_t st) {
  *n = (int64_t)src.size();
  if (src.empty()) { *dst = nullptr; return cudaSuccess; }
  cudaError_t e = cudaMalloc(dst, sizeof(T) * src.size());
  if (e != cudaSuccess) return e;
  return cudaMemcpyAsync(*dst, src.data(), sizeof(T) * src.size(), cudaMemcpyHostToDevice, st);
}

cudaError_t zeros(double** p, int64_t n, cudaStream_t st) {
  cudaError_t e = cudaMalloc(p, sizeof(double) * n);
  if (e != cudaSuccess) return e;
  return cudaMemsetAsync(*p, 0, sizeof(double) * n, st);
}

// Refinement criterion of the reference's blast (pgen/blast.cpp:413-442): the largest
// |grad p| / p over the interior and one ring of ghost cells of each block, reduced to one
// value per block (non-negative doubles order like their bit patterns)
__global__ void k_amr_pgrad(SmrDims d, const double* __restrict__ w,
                            unsigned long long* __restrict__ maxbits) {
  const int b = blockIdx.y;
  const int n1 = d.nx1 + 2, n2 = d.nx2 + 2, n3 = d.nx3 + 2;
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  double eps = 0.0;
  if (t < (int64_t)n1 * n2 * n3) {
    const int i = d.is - 1 + (int)(t % n1), j = d.js - 1 + (int)((t / n1) % n2),
              k = d.ks - 1 + (int)(t / ((int64_t)n1 * n2));
    const double* p = w + ((int64_t)b * 5 + 4) * d.ncell;
    const int64_t c = d.c(k, j, i), sj = d.nc1, sk = (int64_t)d.nc1 * d.nc2;
    const double gx = 0.5 * (p[c + 1] - p[c - 1]), gy = 0.5 * (p[c + sj] - p[c - sj]),
                 gz = 0.5 * (p[c + sk] - p[c - sk]);
    eps = sqrt(gx * gx + gy * gy + gz * gz) / p[c];
    if (!(eps > 0.0)) eps = 0.0;  // std::max(maxeps, eps) never picks NaN or negatives
  }
  unsigned long long v = (unsigned long long)__double_as_longlong(eps);
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long x = __shfl_xor_sync(0xffffffffu, v, o);
    v = x > v ? x : v;
  }
  if ((threadIdx.x & 31) == 0 && v) atomicMax(maxbits + b, v);
}

}  // namespace

int amr_criterion(const SmrDims& d, int nb, const double* w, unsigned long long* maxbits,
                  cudaStream_t st) {
  cudaMemsetAsync(maxbits, 0, sizeof(unsigned long long) * nb, st);
  const int64_t n = (int64_t)(d.nx1 + 2) * (d.nx2 + 2) * (d.nx3 + 2);
  dim3 grid((unsigned)((n + kThreads - 1) / kThreads), (unsigned)nb);
  k_amr_pgrad<<<grid, kThreads, 0, st>>>(d, w, maxbits);
  return 1;
}

void smr_destroy(SmrDevice* s) {
  if (!s) return;
  void* ps[] = {s->xfer, s->pre, s->flux, s->emf, s->emf_add, s->emf_tmp, s->c2p, s->pcc,
                s->pint, s->pfine, s->psf[0], s->psf[1], s->psf[2], s->cu, s->cw, s->cb1,
                s->cb2, s->cb3, s->cbcc, s->dx, s->xvf, s->xvc};
  for (void* p : ps)
    if (p) cudaFree(p);
  delete s;
}

int smr_create(SmrDevice** out, const SmrDims& d, const int nrb[3],
               const std::vector<SmrLoc>& loc, const std::vector<double>& dx,
               const std::vector<double>& xvf, const std::vector<double>& xvc, bool mhd,
               cudaStream_t st, std::string* err) {
  *out = nullptr;
  SmrPlan plan;
  if (!smr_plan(d, nrb, loc, dx.data(), mhd, &plan, err)) return -1;
  SmrDevice* s = new SmrDevice();
  s->d = d;
  s->nb = (int)loc.size();
  s->nlevels = plan.nlevels;
  s->ncmax = std::max(d.nc1, std::max(d.nc2, d.nc3));
  s->nccmax = std::max(d.ncc1, std::max(d.ncc2, d.ncc3));
  s->mhd = mhd ? 1 : 0;
  const int64_t nb = s->nb;
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t r) { if (e == cudaSuccess) e = r; };
  ok(upload(&s->xfer, plan.xfer, &s->nxfer, st));
  ok(upload(&s->pre, plan.pre, &s->npre, st));
  ok(upload(&s->flux, plan.flux, &s->nflux, st));
  ok(upload(&s->emf, plan.emf, &s->nemf, st));
  int64_t nadd = 0;
  ok(upload(&s->emf_add, plan.emf_add, &nadd, st));
  if (s->nemf) ok(cudaMalloc(&s->emf_tmp, sizeof(double) * s->nemf));
  ok(upload(&s->c2p, plan.c2p, &s->nc2p, st));
  ok(upload(&s->pcc, plan.pcc, &s->npcc, st));
  ok(upload(&s->pint, plan.pint, &s->npint, st));
  ok(upload(&s->pfine, plan.pfine, &s->npfine, st));
  for (int f = 0; f < 3; ++f) ok(upload(&s->psf[f], plan.psf[f], &s->npsf[f], st));
  ok(zeros(&s->cu, 5 * d.ccell * nb, st));
  ok(zeros(&s->cw, 5 * d.ccell * nb, st));
  if (mhd) {
    ok(zeros(&s->cb1, d.cf1 * nb, st));
    ok(zeros(&s->cb2, d.cf2 * nb, st));
    ok(zeros(&s->cb3, d.cf3 * nb, st));
    ok(zeros(&s->cbcc, 3 * d.ccell * nb, st));
  }
  int64_t n0;
  ok(upload(&s->dx, dx, &n0, st));
  ok(upload(&s->xvf, xvf, &n0, st));
  ok(upload(&s->xvc, xvc, &n0, st));
  ok(cudaStreamSynchronize(st));  // the host plan goes out of scope
  if (e != cudaSuccess) {
    *err = std::string("SMR plan upload: ") + cudaGetErrorString(e);
    smr_destroy(s);
    return -2;
  }
  *out = s;
  return 0;
}

SmrPool smr_pool(const SmrDevice* s) {
  SmrPool P{};
  P.cu = s->cu; P.cw = s->cw; P.cb1 = s->cb1; P.cb2 = s->cb2; P.cb3 = s->cb3; P.cbcc = s->cbcc;
  P.dx = s->dx; P.xvf = s->xvf; P.xvc = s->xvc;
  P.ncmax = s->ncmax; P.nccmax = s->nccmax;
  P.mhd = s->mhd;
  return P;
}

int smr_fill(const SmrDevice* s, const SmrPool& P, cudaStream_t st) {
  const SmrDims& d = s->d;
  int n = 0;
  if (s->nxfer) { k_smr_xfer<<<grid_of(s->nxfer), kThreads, 0, st>>>(d, P, s->xfer, s->nxfer); ++n; }
  if (s->npre) { k_smr_xfer<<<grid_of(s->npre), kThreads, 0, st>>>(d, P, s->pre, s->npre); ++n; }
  if (s->nc2p) { k_smr_c2p<<<grid_of(s->nc2p), kThreads, 0, st>>>(d, P, s->c2p, s->nc2p); ++n; }
  if (s->npcc) { k_smr_pcc<<<grid_of(s->npcc), kThreads, 0, st>>>(d, P, s->pcc, s->npcc); ++n; }
  if (s->mhd) {
    for (int f = 0; f < 3; ++f)
      if (s->npsf[f]) {
        k_smr_psf<<<grid_of(s->npsf[f]), kThreads, 0, st>>>(d, P, f, s->psf[f], s->npsf[f]);
        ++n;
      }
    if (s->npint) { k_smr_pint<<<grid_of(s->npint), kThreads, 0, st>>>(d, P, s->pint, s->npint); ++n; }
  }
  if (s->npfine) {
    k_smr_pfine<<<grid_of(s->npfine), kThreads, 0, st>>>(d, P, s->pfine, s->npfine);
    ++n;
  }
  return n;
}

int smr_correct_flux(const SmrDevice* s, const SmrPool& P, cudaStream_t st) {
  if (!s->nflux) return 0;
  k_smr_flux<<<grid_of(s->nflux), kThreads, 0, st>>>(s->d, P, s->flux, s->nflux);
  return 1;
}

int smr_correct_emf(const SmrDevice* s, const SmrPool& P, cudaStream_t st) {
  if (!s->nemf) return 0;
  k_smr_emf_eval<<<grid_of(s->nemf), kThreads, 0, st>>>(s->d, P, s->emf, s->emf_add, s->nemf,
                                                        s->emf_tmp);
  k_smr_emf_store<<<grid_of(s->nemf), kThreads, 0, st>>>(s->d, P, s->emf, s->nemf, s->emf_tmp);
  return 2;
}

}  // namespace athg

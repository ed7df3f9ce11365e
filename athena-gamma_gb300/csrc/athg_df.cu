// athg_df.cu -- flux sweeps and corner EMFs of the double-float path (precision ATHG_DFLOAT).
//
// The state, the primitives, the fluxes and the edge EMFs are FP64 arrays, as in the FP64
// path, and the flux divergence, CT, primitive recovery, ghost exchange and time step are
// the FP64 path's kernels. Only the two costliest parts -- reconstruction + Riemann solve
// (hydro/calculate_fluxes.cpp:36-378) and the corner EMFs (field/calculate_corner_e.cpp:
// 129-229) -- run here in double-float arithmetic (athg_dfloat.cuh) on the FP32 pipe, with
// the same expressions as the FP64 kernels: the FP64 inputs are split exactly into pairs
// on the integer pipe, the results widened back to FP64. The values agree with the FP64
// path's to about 2^-44 relative, so the truncation error of a run is the FP64 path's,
// including for waves whose amplitude is near the FP32 resolution of their background
// (where the FP32 flux path's rounding of O(1) fluxes is not small next to the signal).
//
// One thread per face (x1, x2, x3 sweeps over the face boxes of calculate_fluxes.cpp:63-74,
// 164-172, 274-279) and one per corner, like k_flux and k_corner_emf.
#include <cuda_runtime.h>

#include "athg_stage.cuh"
#include "athg_dfloat.cuh"  // after the templates: double-float overloads found by ADL
#include "athg_df.h"

namespace athg {

namespace {

constexpr int kThreads = 128;

__device__ __forceinline__ dfl ldf(const double* p, int64_t q) { return df_of(__ldg(p + q)); }

__device__ __forceinline__ dfl lpair(const float2* p, int64_t q) {
  const float2 v = __ldg(p + q);
  return dfl(v.x, v.y);
}

// W and bcc of every cell split once into pairs [nb][8][cells] (the flux sweeps read each
// cell up to 12 times)
__global__ void __launch_bounds__(256) k_split_w(Geom g, StagePtrs<double> p, int nv,
                                                  float2* __restrict__ wp) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nc = g.ncell;
  if (t >= nc) return;
  const int b = blockIdx.y;
  const double* w = p.w + (int64_t)b * NHYD * nc;
  float2* o = wp + (int64_t)b * nv * nc;
#pragma unroll
  for (int n = 0; n < NHYD; ++n) {
    const dfl v = df_of(__ldg(w + n * nc + t));
    o[n * nc + t] = make_float2(v.hi, v.lo);
  }
  if (nv > NHYD) {
    const double* bc = p.bcc + (int64_t)b * 3 * nc;
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      const dfl v = df_of(__ldg(bc + n * nc + t));
      o[(NHYD + n) * nc + t] = make_float2(v.hi, v.lo);
    }
  }
}

template <int DIR, int ORDER, int SOLVER, bool MHD>
__global__ void __launch_bounds__(kThreads)
k_flux_df(Geom g, StagePtrs<double> p, Box bx, Phys ph, const float2* __restrict__ wpairs) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  constexpr int NW = MHD ? 7 : 5;
  constexpr int NF = MHD ? 8 : 5;
  constexpr int NV = MHD ? 8 : 5;
  const int64_t nc = g.ncell;
  const float2* __restrict__ wq = wpairs + (int64_t)b * NV * nc;
  const int64_t st = DIR == 0 ? 1 : (DIR == 1 ? (int64_t)g.nc1 : (int64_t)g.nc1 * g.nc2);
  const int64_t c = cidx(g, k, j, i);  // cell on the right of the face
  const int f = DIR == 0 ? i : (DIR == 1 ? j : k);
  auto wv = [&](int n, int64_t q) -> dfl {  // wave variable n of cell q (plm.cpp:44-55 order)
    if (n < NHYD) return lpair(wq, n * nc + q);
    constexpr int by = DIR == 0 ? 1 : (DIR == 1 ? 2 : 0);
    constexpr int bz = DIR == 0 ? 2 : (DIR == 1 ? 0 : 1);
    return lpair(wq, (NHYD + (n == IBY ? by : bz)) * nc + q);
  };
  dfl wl[7], wr[7];
  if (ORDER == 1) {
#pragma unroll
    for (int n = 0; n < NW; ++n) {
      wl[n] = wv(n, c - st);
      wr[n] = wv(n, c);
    }
  } else {
    const double* cf = p.coef + ((int64_t)b * 3 + DIR) * 2 * g.ncmax;
    const dfl cpL = ldf(cf, f - 1), cmR = ldf(cf, g.ncmax + f);
#pragma unroll
    for (int n = 0; n < NW; ++n) {
      const dfl a0 = wv(n, c - 2 * st), a1 = wv(n, c - st), a2 = wv(n, c), a3 = wv(n, c + st);
      // van Leer slopes, uniform branch of plm.cpp (the arithmetic of k_flux)
      dfl dwl = (a1 - a0), dwr = (a2 - a1);
      dfl dw2 = dwl * dwr;
      dfl dwm = dfl(2.0) * dw2 / (dwl + dwr);
      if (dw2 <= dfl(0.0)) dwm = dfl(0.0);
      wl[n] = a1 + cpL * dwm;
      dwl = (a2 - a1); dwr = (a3 - a2);
      dw2 = dwl * dwr;
      dwm = dfl(2.0) * dw2 / (dwl + dwr);
      if (dw2 <= dfl(0.0)) dwm = dfl(0.0);
      wr[n] = a2 - cmR * dwm;
    }
  }
  constexpr int ivx = IVX + DIR, ivy = IVX + (DIR + 1) % 3, ivz = IVX + (DIR + 2) % 3;
  dfl wli[7], wri[7], fx[7];
  wli[IDN] = wl[IDN]; wli[IVX] = wl[ivx]; wli[IVY] = wl[ivy]; wli[IVZ] = wl[ivz];
  wli[IPR] = wl[IPR];
  wri[IDN] = wr[IDN]; wri[IVX] = wr[ivx]; wri[IVY] = wr[ivy]; wri[IVZ] = wr[ivz];
  wri[IPR] = wr[IPR];
  const int64_t nf = fsize<DIR>(g);
  const int64_t fi = fidx<DIR>(g, k, j, i);
  double* __restrict__ out = p.flx[DIR] + (int64_t)b * NF * nf;
  const dfl gam = df_of(ph.gamma);
  if constexpr (MHD) {
    wli[IBY] = wl[IBY]; wli[IBZ] = wl[IBZ];
    wri[IBY] = wr[IBY]; wri[IBZ] = wr[IBZ];
    const dfl bxi = ldf(p.bf[DIR], (int64_t)b * nf + fi);
    if (SOLVER == HLLD) rs_hlld<dfl>(wli, wri, bxi, gam, fx);
    else rs_hlle_mhd<dfl>(wli, wri, bxi, gam, fx);
    // the face EMFs and the CT weight are read only by the corner-EMF kernel of this
    // path: kept as double-float pairs in their 8-byte slots (no split when read)
    float2* pr = reinterpret_cast<float2*>(out);
    const dfl e0 = -fx[IBY], e1 = fx[IBZ];
    pr[5 * nf + fi] = make_float2(e0.hi, e0.lo);
    pr[6 * nf + fi] = make_float2(e1.hi, e1.lo);
    const dfl dx = df_of(p.geo[b].dx[DIR]), dt = df_of(__ldg(p.dt));
    const dfl wct = ct_weight<dfl>(fx[IDN], wli[IDN], wri[IDN], dx, dt);
    pr[7 * nf + fi] = make_float2(wct.hi, wct.lo);
  } else {
    if (SOLVER == HLLC) rs_hllc<dfl>(wli, wri, gam, fx);
    else rs_hlle_hydro<dfl>(wli, wri, gam, fx);
  }
  out[IDN * nf + fi] = dbl(fx[IDN]);
  out[ivx * nf + fi] = dbl(fx[IVX]);
  out[ivy * nf + fi] = dbl(fx[IVY]);
  out[ivz * nf + fi] = dbl(fx[IVZ]);
  out[IEN * nf + fi] = dbl(fx[IEN]);
}

// cell-centred E = -v x B (field/calculate_corner_e.cpp:135-200) in double-float, one
// thread per cell of [is-1, ie+1]^3, stored as pairs [nb][3][cells]
__global__ void __launch_bounds__(kThreads) k_cce_df(Geom g, StagePtrs<double> p, Box bx,
                                                      float2* __restrict__ cce) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  const int64_t nc = g.ncell, q = cidx(g, k, j, i);
  const double* w = p.w + (int64_t)b * NHYD * nc;
  const double* bc = p.bcc + (int64_t)b * 3 * nc;
  const dfl vx = ldf(w, IVX * nc + q), vy = ldf(w, IVY * nc + q), vz = ldf(w, IVZ * nc + q);
  const dfl bx1 = ldf(bc, q), by1 = ldf(bc, nc + q), bz1 = ldf(bc, 2 * nc + q);
  const dfl e[3] = {vz * by1 - vy * bz1, vx * bz1 - vz * bx1, vy * bx1 - vx * by1};
  float2* o = cce + (int64_t)b * 3 * nc;
#pragma unroll
  for (int n = 0; n < 3; ++n) o[n * nc + q] = make_float2(e[n].hi, e[n].lo);
}

// Gardiner-Stone corner EMFs (the expressions of k_corner_emf) in double-float, from the
// pair-valued face EMFs and cell-centred EMFs
__global__ void __launch_bounds__(kThreads) k_corner_df(Geom g, StagePtrs<double> p, Box bx,
                                                         const float2* __restrict__ cc) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  const int64_t nc = g.ncell;
  const float2* ccb = cc + (int64_t)b * 3 * nc;
  auto cce = [&](int n, int kk, int jj, int ii) -> dfl {
    return lpair(ccb, n * nc + cidx(g, kk, jj, ii));
  };
  const int64_t n1 = g.nf1, n2 = g.nf2, n3 = g.nf3;
  const float2* F1 = reinterpret_cast<const float2*>(p.flx[0] + (int64_t)b * 8 * n1);
  const float2* F2 = reinterpret_cast<const float2*>(p.flx[1] + (int64_t)b * 8 * n2);
  const float2* F3 = reinterpret_cast<const float2*>(p.flx[2] + (int64_t)b * 8 * n3);
  auto e3x1 = [&](int kk, int jj, int ii) { return lpair(F1, 5 * n1 + f1idx(g, kk, jj, ii)); };
  auto e2x1 = [&](int kk, int jj, int ii) { return lpair(F1, 6 * n1 + f1idx(g, kk, jj, ii)); };
  auto wx1 = [&](int kk, int jj, int ii) { return lpair(F1, 7 * n1 + f1idx(g, kk, jj, ii)); };
  auto e1x2 = [&](int kk, int jj, int ii) { return lpair(F2, 5 * n2 + f2idx(g, kk, jj, ii)); };
  auto e3x2 = [&](int kk, int jj, int ii) { return lpair(F2, 6 * n2 + f2idx(g, kk, jj, ii)); };
  auto wx2 = [&](int kk, int jj, int ii) { return lpair(F2, 7 * n2 + f2idx(g, kk, jj, ii)); };
  auto e2x3 = [&](int kk, int jj, int ii) { return lpair(F3, 5 * n3 + f3idx(g, kk, jj, ii)); };
  auto e1x3 = [&](int kk, int jj, int ii) { return lpair(F3, 6 * n3 + f3idx(g, kk, jj, ii)); };
  auto wx3 = [&](int kk, int jj, int ii) { return lpair(F3, 7 * n3 + f3idx(g, kk, jj, ii)); };
  const dfl one = dfl(1.0), q = dfl(0.25);
  double* E = p.edge + (int64_t)b * 3 * g.ne;
  const int64_t ei = eidx(g, k, j, i);
  {
    dfl de1_l3 = (one - wx2(k - 1, j, i)) * (e1x3(k, j, i) - cce(0, k - 1, j, i)) +
                 (wx2(k - 1, j, i)) * (e1x3(k, j - 1, i) - cce(0, k - 1, j - 1, i));
    dfl de1_r3 = (one - wx2(k, j, i)) * (e1x3(k, j, i) - cce(0, k, j, i)) +
                 (wx2(k, j, i)) * (e1x3(k, j - 1, i) - cce(0, k, j - 1, i));
    dfl de1_l2 = (one - wx3(k, j - 1, i)) * (e1x2(k, j, i) - cce(0, k, j - 1, i)) +
                 (wx3(k, j - 1, i)) * (e1x2(k - 1, j, i) - cce(0, k - 1, j - 1, i));
    dfl de1_r2 = (one - wx3(k, j, i)) * (e1x2(k, j, i) - cce(0, k, j, i)) +
                 (wx3(k, j, i)) * (e1x2(k - 1, j, i) - cce(0, k - 1, j, i));
    E[ei] = dbl(q * (de1_l3 + de1_r3 + de1_l2 + de1_r2 + e1x2(k - 1, j, i) + e1x2(k, j, i) +
                     e1x3(k, j - 1, i) + e1x3(k, j, i)));
  }
  {
    dfl de2_l3 = (one - wx1(k - 1, j, i)) * (e2x3(k, j, i) - cce(1, k - 1, j, i)) +
                 (wx1(k - 1, j, i)) * (e2x3(k, j, i - 1) - cce(1, k - 1, j, i - 1));
    dfl de2_r3 = (one - wx1(k, j, i)) * (e2x3(k, j, i) - cce(1, k, j, i)) +
                 (wx1(k, j, i)) * (e2x3(k, j, i - 1) - cce(1, k, j, i - 1));
    dfl de2_l1 = (one - wx3(k, j, i - 1)) * (e2x1(k, j, i) - cce(1, k, j, i - 1)) +
                 (wx3(k, j, i - 1)) * (e2x1(k - 1, j, i) - cce(1, k - 1, j, i - 1));
    dfl de2_r1 = (one - wx3(k, j, i)) * (e2x1(k, j, i) - cce(1, k, j, i)) +
                 (wx3(k, j, i)) * (e2x1(k - 1, j, i) - cce(1, k - 1, j, i));
    E[g.ne + ei] = dbl(q * (de2_l3 + de2_r3 + de2_l1 + de2_r1 + e2x3(k, j, i - 1) +
                            e2x3(k, j, i) + e2x1(k - 1, j, i) + e2x1(k, j, i)));
  }
  {
    dfl de3_l2 = (one - wx1(k, j - 1, i)) * (e3x2(k, j, i) - cce(2, k, j - 1, i)) +
                 (wx1(k, j - 1, i)) * (e3x2(k, j, i - 1) - cce(2, k, j - 1, i - 1));
    dfl de3_r2 = (one - wx1(k, j, i)) * (e3x2(k, j, i) - cce(2, k, j, i)) +
                 (wx1(k, j, i)) * (e3x2(k, j, i - 1) - cce(2, k, j, i - 1));
    dfl de3_l1 = (one - wx2(k, j, i - 1)) * (e3x1(k, j, i) - cce(2, k, j, i - 1)) +
                 (wx2(k, j, i - 1)) * (e3x1(k, j - 1, i) - cce(2, k, j - 1, i - 1));
    dfl de3_r1 = (one - wx2(k, j, i)) * (e3x1(k, j, i) - cce(2, k, j, i)) +
                 (wx2(k, j, i)) * (e3x1(k, j - 1, i) - cce(2, k, j - 1, i));
    E[2 * g.ne + ei] = dbl(q * (de3_l1 + de3_r1 + de3_l2 + de3_r2 + e3x2(k, j, i - 1) +
                                e3x2(k, j, i) + e3x1(k, j - 1, i) + e3x1(k, j, i)));
  }
}

Box box_of(int il, int iu, int jl, int ju, int kl, int ku) {
  Box b;
  b.il = il; b.jl = jl; b.kl = kl;
  b.ni = iu - il + 1; b.nj = ju - jl + 1; b.nk = ku - kl + 1;
  return b;
}
dim3 grid_of(const Box& b, int nb) {
  return dim3((unsigned)((b.ni * b.nj + kThreads - 1) / kThreads), (unsigned)b.nk, (unsigned)nb);
}

template <int DIR, int ORDER>
void sweep(const Geom& g, const StagePtrs<double>& p, bool mhd, int solver, const Phys& ph,
           const float2* wp, cudaStream_t st) {
  int il = g.is, iu = g.ie, jl = g.js, ju = g.je, kl = g.ks, ku = g.ke;
  if (DIR == 0) {
    iu = g.ie + 1;
    if (mhd) { jl = g.js - 1; ju = g.je + 1; kl = g.ks - 1; ku = g.ke + 1; }
  } else if (DIR == 1) {
    ju = g.je + 1; il = g.is - 1; iu = g.ie + 1;
    if (mhd) { kl = g.ks - 1; ku = g.ke + 1; }
  } else {
    ku = g.ke + 1;
    if (mhd) { il = g.is - 1; iu = g.ie + 1; jl = g.js - 1; ju = g.je + 1; }
  }
  const Box b = box_of(il, iu, jl, ju, kl, ku);
  const dim3 gr = grid_of(b, g.nb);
  if (mhd) {
    if (solver == HLLD) k_flux_df<DIR, ORDER, HLLD, true><<<gr, kThreads, 0, st>>>(g, p, b, ph, wp);
    else k_flux_df<DIR, ORDER, HLLE, true><<<gr, kThreads, 0, st>>>(g, p, b, ph, wp);
  } else {
    if (solver == HLLC) k_flux_df<DIR, ORDER, HLLC, false><<<gr, kThreads, 0, st>>>(g, p, b, ph, wp);
    else k_flux_df<DIR, ORDER, HLLE, false><<<gr, kThreads, 0, st>>>(g, p, b, ph, wp);
  }
}

}  // namespace

bool df_supported(int mhd, int solver, int xorder) {
  const bool s = mhd ? (solver == HLLD || solver == HLLE) : (solver == HLLC || solver == HLLE);
  return s && (xorder == 1 || xorder == 2);
}

void df_fluxes(const Geom& g, const StagePtrs<double>& p, bool mhd, int solver, int order,
               const Phys& ph, float2* wp, cudaStream_t st) {
  const int nv = mhd ? 8 : 5;
  k_split_w<<<dim3((unsigned)((g.ncell + 255) / 256), (unsigned)g.nb), 256, 0, st>>>(g, p, nv, wp);
  if (order == 1) {
    sweep<0, 1>(g, p, mhd, solver, ph, wp, st);
    sweep<1, 1>(g, p, mhd, solver, ph, wp, st);
    sweep<2, 1>(g, p, mhd, solver, ph, wp, st);
  } else {
    sweep<0, 2>(g, p, mhd, solver, ph, wp, st);
    sweep<1, 2>(g, p, mhd, solver, ph, wp, st);
    sweep<2, 2>(g, p, mhd, solver, ph, wp, st);
  }
}

void df_corner_emf(const Geom& g, const StagePtrs<double>& p, float2* cce, cudaStream_t st) {
  const Box c = box_of(g.is - 1, g.ie + 1, g.js - 1, g.je + 1, g.ks - 1, g.ke + 1);
  k_cce_df<<<grid_of(c, g.nb), kThreads, 0, st>>>(g, p, c, cce);
  const Box b = box_of(g.is, g.ie + 1, g.js, g.je + 1, g.ks, g.ke + 1);
  k_corner_df<<<grid_of(b, g.nb), kThreads, 0, st>>>(g, p, b, cce);
}

}  // namespace athg

// athg_df.cu -- kernels of the double-float path (precision ATHG_DFLOAT).
//
// The state, the face field, the primitives and bcc are FP64 arrays, as in the FP64 path,
// and the ghost exchange is the FP64 path's. Reconstruction + Riemann solve
// (hydro/calculate_fluxes.cpp:36-378) and the corner EMFs (field/calculate_corner_e.cpp:
// 129-229) run here in double-float arithmetic (athg_dfloat.cuh) on the FP32 pipe, with the
// same expressions as the FP64 kernels: the FP64 inputs are split exactly into pairs on
// the integer pipe. On uniform periodic meshes without source terms the update, primitive
// recovery and time step run here in double-float too (k_update_df, k_c2p_df, k_dt_df), the
// fluxes and edge EMFs passing between the kernels as pairs; elsewhere those three are the
// FP64 path's kernels and the fluxes are widened back to FP64. The values agree with the FP64
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

// HLLD of this path on left/right lane pairs (hlld_lr in athg_device.cuh): pairs of
// double-float numbers whose hi and lo parts are float2 lanes, with the operations of
// athg_dfloat.cuh done on both lanes by Blackwell's packed FP32 instructions (the same
// operation sequence per lane; divisions and square roots per lane).
struct D2 {
  float2 hi, lo;
};
struct PkD {
  using S = dfl;
  using P = D2;
  static __device__ __forceinline__ S sc(double v) { return dfl(v); }
  static __device__ __forceinline__ P splat(S s) {
    return D2{make_float2(s.hi, s.hi), make_float2(s.lo, s.lo)};
  }
  static __device__ __forceinline__ P pair(S l, S r) {
    return D2{make_float2(l.hi, r.hi), make_float2(l.lo, r.lo)};
  }
  static __device__ __forceinline__ S L(P a) { return dfl(a.hi.x, a.lo.x); }
  static __device__ __forceinline__ S R(P a) { return dfl(a.hi.y, a.lo.y); }
  static __device__ __forceinline__ float2 ad(float2 a, float2 b) { return __fadd2_rn(a, b); }
  static __device__ __forceinline__ float2 sb(float2 a, float2 b) {  // a - b, one rounding
    return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a);
  }
  static __device__ __forceinline__ P fast(float2 s, float2 e) {  // df_fast on both lanes
    const float2 h = ad(s, e);
    return D2{h, sb(e, sb(h, s))};
  }
  static __device__ __forceinline__ P add(P a, P b) {  // dfl operator+ (TwoSum, renorm)
    const float2 s = ad(a.hi, b.hi);
    const float2 bp = sb(s, a.hi);
    float2 e = ad(sb(a.hi, sb(s, bp)), sb(b.hi, bp));
    e = ad(e, ad(a.lo, b.lo));
    return fast(s, e);
  }
  static __device__ __forceinline__ P neg(P a) {
    return D2{make_float2(-a.hi.x, -a.hi.y), make_float2(-a.lo.x, -a.lo.y)};
  }
  static __device__ __forceinline__ P sub(P a, P b) { return add(a, neg(b)); }
  static __device__ __forceinline__ P mul(P a, P b) {  // dfl operator* (TwoProduct)
    const float2 p = __fmul2_rn(a.hi, b.hi);
    float2 e = __ffma2_rn(a.hi, b.hi, make_float2(-p.x, -p.y));
    e = __ffma2_rn(a.hi, b.lo, e);
    e = __ffma2_rn(a.lo, b.hi, e);
    return fast(p, e);
  }
  static __device__ __forceinline__ P fma(P a, P b, P c) { return add(mul(a, b), c); }
  static __device__ __forceinline__ P div(P a, P b) { return pair(L(a) / L(b), R(a) / R(b)); }
  static __device__ __forceinline__ P sqrt2(P a) { return pair(sqrt(L(a)), sqrt(R(a))); }
  static __device__ __forceinline__ P sel(bool l, bool r, P a, P b) {
    return pair(l ? L(a) : L(b), r ? R(a) : R(b));
  }
  static __device__ __forceinline__ S abs(S a) { return fabs(a); }
};

template <>
__device__ __forceinline__ void rs_hlld<dfl>(const dfl* wli, const dfl* wri, dfl bxi, dfl gamma,
                                             dfl* flxi) {
  hlld_lr<PkD>(wli, wri, bxi, gamma, flxi);
}

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

// Four blocks of 128 per SM (at most 128 registers): measured 5.6% faster per cycle than the
// 148 registers HLLD takes unbounded (three blocks), and faster than five blocks (102).
template <int DIR, int ORDER, int SOLVER, bool MHD, bool PAIRS>
__global__ void __launch_bounds__(kThreads, 4)
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
  if constexpr (PAIRS) {  // read only by k_update_df: pairs in the 8-byte slots
    float2* pr = reinterpret_cast<float2*>(out);
    pr[IDN * nf + fi] = make_float2(fx[IDN].hi, fx[IDN].lo);
    pr[ivx * nf + fi] = make_float2(fx[IVX].hi, fx[IVX].lo);
    pr[ivy * nf + fi] = make_float2(fx[IVY].hi, fx[IVY].lo);
    pr[ivz * nf + fi] = make_float2(fx[IVZ].hi, fx[IVZ].lo);
    pr[IEN * nf + fi] = make_float2(fx[IEN].hi, fx[IEN].lo);
    return;
  }
  out[IDN * nf + fi] = dbl(fx[IDN]);
  out[ivx * nf + fi] = dbl(fx[IVX]);
  out[ivy * nf + fi] = dbl(fx[IVY]);
  out[ivz * nf + fi] = dbl(fx[IVZ]);
  out[IEN * nf + fi] = dbl(fx[IEN]);
}

// cell-centred E = -v x B (field/calculate_corner_e.cpp:135-200) in double-float, one
// thread per cell of [is-1, ie+1]^3, stored as pairs [nb][3][cells]
// (wpairs: the primitives and cell-centred field already as pairs [nb][8][cells], or null
// to split the FP64 arrays)
__global__ void __launch_bounds__(kThreads) k_cce_df(Geom g, StagePtrs<double> p, Box bx,
                                                      float2* __restrict__ cce,
                                                      const float2* __restrict__ wpairs) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  const int64_t nc = g.ncell, q = cidx(g, k, j, i);
  dfl vx, vy, vz, bx1, by1, bz1;
  if (wpairs) {
    const float2* wq = wpairs + (int64_t)b * 8 * nc;
    vx = lpair(wq, IVX * nc + q); vy = lpair(wq, IVY * nc + q); vz = lpair(wq, IVZ * nc + q);
    bx1 = lpair(wq, 5 * nc + q); by1 = lpair(wq, 6 * nc + q); bz1 = lpair(wq, 7 * nc + q);
  } else {
    const double* w = p.w + (int64_t)b * NHYD * nc;
    const double* bc = p.bcc + (int64_t)b * 3 * nc;
    vx = ldf(w, IVX * nc + q); vy = ldf(w, IVY * nc + q); vz = ldf(w, IVZ * nc + q);
    bx1 = ldf(bc, q); by1 = ldf(bc, nc + q); bz1 = ldf(bc, 2 * nc + q);
  }
  const dfl e[3] = {vz * by1 - vy * bz1, vx * bz1 - vz * bx1, vy * bx1 - vx * by1};
  float2* o = cce + (int64_t)b * 3 * nc;
#pragma unroll
  for (int n = 0; n < 3; ++n) o[n * nc + q] = make_float2(e[n].hi, e[n].lo);
}

// Gardiner-Stone corner EMFs (the expressions of k_corner_emf) in double-float, from the
// pair-valued face EMFs and cell-centred EMFs
// (PAIRS: the edge EMFs stored as pairs in their 8-byte slots, for k_update_df; the loads
// are addressed from this corner's base indices and the strides, as in k_corner_emf)
template <bool PAIRS>
__global__ void __launch_bounds__(kThreads) k_corner_df(Geom g, StagePtrs<double> p, Box bx,
                                                         const float2* __restrict__ cc) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  const int64_t nc = g.ncell;
  const int64_t c0 = cidx(g, k, j, i), q1 = f1idx(g, k, j, i), q2 = f2idx(g, k, j, i);
  const int64_t jc = g.nc1, kc = (int64_t)g.nc1 * g.nc2;
  const int64_t j1 = g.nc1 + 1, k1 = (int64_t)(g.nc1 + 1) * g.nc2;
  const int64_t j2 = g.nc1, k2 = (int64_t)g.nc1 * (g.nc2 + 1);
  const float2* ccb = cc + (int64_t)b * 3 * nc + c0;
  auto cce = [&](int n, int dk, int dj, int di) -> dfl {
    return lpair(ccb, n * nc + dk * kc + dj * jc + di);
  };
  const int64_t n1 = g.nf1, n2 = g.nf2, n3 = g.nf3;
  const float2* F1 = reinterpret_cast<const float2*>(p.flx[0] + (int64_t)b * 8 * n1) + q1;
  const float2* F2 = reinterpret_cast<const float2*>(p.flx[1] + (int64_t)b * 8 * n2) + q2;
  const float2* F3 = reinterpret_cast<const float2*>(p.flx[2] + (int64_t)b * 8 * n3) + c0;
  auto o1 = [&](int dk, int dj, int di) { return dk * k1 + dj * j1 + di; };
  auto o2 = [&](int dk, int dj, int di) { return dk * k2 + dj * j2 + di; };
  auto o3 = [&](int dk, int dj, int di) { return dk * kc + dj * jc + di; };
  auto e3x1 = [&](int dk, int dj, int di) { return lpair(F1, 5 * n1 + o1(dk, dj, di)); };
  auto e2x1 = [&](int dk, int dj, int di) { return lpair(F1, 6 * n1 + o1(dk, dj, di)); };
  auto wx1 = [&](int dk, int dj, int di) { return lpair(F1, 7 * n1 + o1(dk, dj, di)); };
  auto e1x2 = [&](int dk, int dj, int di) { return lpair(F2, 5 * n2 + o2(dk, dj, di)); };
  auto e3x2 = [&](int dk, int dj, int di) { return lpair(F2, 6 * n2 + o2(dk, dj, di)); };
  auto wx2 = [&](int dk, int dj, int di) { return lpair(F2, 7 * n2 + o2(dk, dj, di)); };
  auto e2x3 = [&](int dk, int dj, int di) { return lpair(F3, 5 * n3 + o3(dk, dj, di)); };
  auto e1x3 = [&](int dk, int dj, int di) { return lpair(F3, 6 * n3 + o3(dk, dj, di)); };
  auto wx3 = [&](int dk, int dj, int di) { return lpair(F3, 7 * n3 + o3(dk, dj, di)); };
  const dfl one = dfl(1.0), q = dfl(0.25);
  double* E = p.edge + (int64_t)b * 3 * g.ne;
  const int64_t ei = eidx(g, k, j, i);
  auto put = [&](int64_t at, dfl v) {
    if constexpr (PAIRS) reinterpret_cast<float2*>(E)[at] = make_float2(v.hi, v.lo);
    else E[at] = dbl(v);
  };
  {
    dfl de1_l3 = (one - wx2(-1, 0, 0)) * (e1x3(0, 0, 0) - cce(0, -1, 0, 0)) +
                 (wx2(-1, 0, 0)) * (e1x3(0, -1, 0) - cce(0, -1, -1, 0));
    dfl de1_r3 = (one - wx2(0, 0, 0)) * (e1x3(0, 0, 0) - cce(0, 0, 0, 0)) +
                 (wx2(0, 0, 0)) * (e1x3(0, -1, 0) - cce(0, 0, -1, 0));
    dfl de1_l2 = (one - wx3(0, -1, 0)) * (e1x2(0, 0, 0) - cce(0, 0, -1, 0)) +
                 (wx3(0, -1, 0)) * (e1x2(-1, 0, 0) - cce(0, -1, -1, 0));
    dfl de1_r2 = (one - wx3(0, 0, 0)) * (e1x2(0, 0, 0) - cce(0, 0, 0, 0)) +
                 (wx3(0, 0, 0)) * (e1x2(-1, 0, 0) - cce(0, -1, 0, 0));
    put(ei, q * (de1_l3 + de1_r3 + de1_l2 + de1_r2 + e1x2(-1, 0, 0) + e1x2(0, 0, 0) +
                 e1x3(0, -1, 0) + e1x3(0, 0, 0)));
  }
  {
    dfl de2_l3 = (one - wx1(-1, 0, 0)) * (e2x3(0, 0, 0) - cce(1, -1, 0, 0)) +
                 (wx1(-1, 0, 0)) * (e2x3(0, 0, -1) - cce(1, -1, 0, -1));
    dfl de2_r3 = (one - wx1(0, 0, 0)) * (e2x3(0, 0, 0) - cce(1, 0, 0, 0)) +
                 (wx1(0, 0, 0)) * (e2x3(0, 0, -1) - cce(1, 0, 0, -1));
    dfl de2_l1 = (one - wx3(0, 0, -1)) * (e2x1(0, 0, 0) - cce(1, 0, 0, -1)) +
                 (wx3(0, 0, -1)) * (e2x1(-1, 0, 0) - cce(1, -1, 0, -1));
    dfl de2_r1 = (one - wx3(0, 0, 0)) * (e2x1(0, 0, 0) - cce(1, 0, 0, 0)) +
                 (wx3(0, 0, 0)) * (e2x1(-1, 0, 0) - cce(1, -1, 0, 0));
    put(g.ne + ei, q * (de2_l3 + de2_r3 + de2_l1 + de2_r1 + e2x3(0, 0, -1) +
                        e2x3(0, 0, 0) + e2x1(-1, 0, 0) + e2x1(0, 0, 0)));
  }
  {
    dfl de3_l2 = (one - wx1(0, -1, 0)) * (e3x2(0, 0, 0) - cce(2, 0, -1, 0)) +
                 (wx1(0, -1, 0)) * (e3x2(0, 0, -1) - cce(2, 0, -1, -1));
    dfl de3_r2 = (one - wx1(0, 0, 0)) * (e3x2(0, 0, 0) - cce(2, 0, 0, 0)) +
                 (wx1(0, 0, 0)) * (e3x2(0, 0, -1) - cce(2, 0, 0, -1));
    dfl de3_l1 = (one - wx2(0, 0, -1)) * (e3x1(0, 0, 0) - cce(2, 0, 0, -1)) +
                 (wx2(0, 0, -1)) * (e3x1(0, -1, 0) - cce(2, 0, -1, -1));
    dfl de3_r1 = (one - wx2(0, 0, 0)) * (e3x1(0, 0, 0) - cce(2, 0, 0, 0)) +
                 (wx2(0, 0, 0)) * (e3x1(0, -1, 0) - cce(2, 0, -1, 0));
    put(2 * g.ne + ei, q * (de3_l1 + de3_r1 + de3_l2 + de3_r2 + e3x2(0, 0, -1) +
                            e3x2(0, 0, 0) + e3x1(0, -1, 0) + e3x1(0, 0, 0)));
  }
}


// ---- the rest of the stage without FP64 arithmetic (uniform periodic meshes) ------------
// The FP64 update, primitive recovery and time step (k_update, k_c2p, k_block_dt with T =
// double) run at the FP64 rate, 1/64 of FP32 here, and took most of this path's time. These
// kernels keep their inputs and outputs (FP64 state, face field, primitives, bcc) but do the
// arithmetic in double-float: the fluxes and edge EMFs arrive as pairs, each cell's
// increment sum_d (beta dt / dx_d) (F_d+ - F_d-) is a pair, and only base - hi - lo runs in
// FP64 (the register averaging of the integrators stays FP64, as in k_update). The state
// keeps FP64 precision; the increment carries about 2^-44 relative error.

__device__ __forceinline__ dfl ps(const float2* p, int64_t q) {  // pair load
  const float2 v = __ldg(p + q);
  return dfl(v.x, v.y);
}

// The register step of MeshBlock::WeightedAve (r = delta u, or r += delta u), written to
// the register and returned. COPY (a first stage with delta 1): 0 + 1 * u, a copy but for
// -0 becoming +0, done on the integer pipe with that same result; otherwise FP64.
template <bool COPY>
__device__ __forceinline__ double reg_update(const StageW& sw, double uo, double* reg) {
  if constexpr (COPY) {
    const double r = (bits_d(uo) << 1) == 0 ? 0.0 : uo;
    *reg = r;
    return r;
  } else {
    double r = sw.zero_reg ? 0.0 : *reg;
    if (sw.delta != 0.0) { r += sw.delta * uo; *reg = r; }
    return r;
  }
}

template <bool MHD, bool COPY>
__global__ void __launch_bounds__(kThreads) k_update_df(Geom g, StagePtrs<double> p, Box bx,
                                                         StageW sw) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  const MixedGeo mg = p.mg[b];
  const dfl wd = df_of(sw.beta * __ldg(p.dt));
  const dfl c1 = wd * dfl(mg.idxh[0], mg.idxl[0]), c2 = wd * dfl(mg.idxh[1], mg.idxl[1]),
            c3 = wd * dfl(mg.idxh[2], mg.idxl[2]);
  const int64_t nc = g.ncell;
  if (i <= g.ie && j <= g.je && k <= g.ke) {
    constexpr int NF = MHD ? 8 : 5;
    double* __restrict__ u = p.u + (int64_t)b * NHYD * nc;
    double* __restrict__ u1 = p.u1 + (int64_t)b * NHYD * nc;
    const int64_t c = cidx(g, k, j, i);
    const float2* __restrict__ F1 =
        reinterpret_cast<const float2*>(p.flx[0] + (int64_t)b * NF * g.nf1) + f1idx(g, k, j, i);
    const float2* __restrict__ F2 =
        reinterpret_cast<const float2*>(p.flx[1] + (int64_t)b * NF * g.nf2) + f2idx(g, k, j, i);
    const float2* __restrict__ F3 =
        reinterpret_cast<const float2*>(p.flx[2] + (int64_t)b * NF * g.nf3) + c;
    const int64_t s2 = g.nc1, s3 = (int64_t)g.nc1 * g.nc2;
    // every flux pair and state value loaded before the first store, so a thread keeps
    // all of its loads in flight at once
    float2 f[NHYD][6];
    double uo[NHYD];
#pragma unroll
    for (int n = 0; n < NHYD; ++n) {
      f[n][0] = __ldg(F1 + n * g.nf1 + 1);
      f[n][1] = __ldg(F1 + n * g.nf1);
      f[n][2] = __ldg(F2 + n * g.nf2 + s2);
      f[n][3] = __ldg(F2 + n * g.nf2);
      f[n][4] = __ldg(F3 + n * g.nf3 + s3);
      f[n][5] = __ldg(F3 + n * g.nf3);
      uo[n] = u[n * nc + c];
    }
    auto pr = [](float2 v) { return dfl(v.x, v.y); };
#pragma unroll
    for (int n = 0; n < NHYD; ++n) {
      const double r = reg_update<COPY>(sw, uo[n], u1 + n * nc + c);
      const double base = sw.swap ? r : sw.g1 * uo[n] + sw.g2 * r;
      const dfl inc = (c1 * (pr(f[n][0]) - pr(f[n][1])) + c2 * (pr(f[n][2]) - pr(f[n][3]))) +
                      c3 * (pr(f[n][4]) - pr(f[n][5]));
      u[n * nc + c] = (base - f2d_int(inc.hi)) - f2d_int(inc.lo);
    }
  }
  if constexpr (MHD) {
    // CT (field/ct.cpp:38-113): b1 -= (dt/dx2) d(e3)/dj - (dt/dx3) d(e2)/dk, and cyclic
    const float2* E1 = reinterpret_cast<const float2*>(p.edge + (int64_t)b * 3 * g.ne);
    const float2* E2 = E1 + g.ne;
    const float2* E3 = E2 + g.ne;
    const int64_t e = eidx(g, k, j, i);
    const int64_t ej = (int64_t)g.nc1 + 1, ek = ((int64_t)g.nc1 + 1) * (g.nc2 + 1);
    auto face = [&](double* bb, double* rr, int64_t q, dfl inc) {
      const double bo = bb[q];
      const double r = reg_update<COPY>(sw, bo, rr + q);
      const double v = sw.swap ? r : sw.g1 * bo + sw.g2 * r;
      bb[q] = (v + f2d_int(inc.hi)) + f2d_int(inc.lo);
    };
    if (j <= g.je && k <= g.ke)
      face(p.b1, p.r1, (int64_t)b * g.nf1 + f1idx(g, k, j, i),
           c3 * (ps(E2, e + ek) - ps(E2, e)) - c2 * (ps(E3, e + ej) - ps(E3, e)));
    if (i <= g.ie && k <= g.ke)
      face(p.b2, p.r2, (int64_t)b * g.nf2 + f2idx(g, k, j, i),
           c1 * (ps(E3, e + 1) - ps(E3, e)) - c3 * (ps(E1, e + ek) - ps(E1, e)));
    if (i <= g.ie && j <= g.je)
      face(p.b3, p.r3, (int64_t)b * g.nf3 + f3idx(g, k, j, i),
           c2 * (ps(E1, e + ej) - ps(E1, e)) - c1 * (ps(E2, e + 1) - ps(E2, e)));
  }
}

// ConservedToPrimitive and the cell-centred field (the formulas of k_c2p) over every cell
// of the block, in double-float: FP64 outputs (each hi + lo, one FP64 addition) and the
// pairs the flux sweeps read [nb][8][cells].
template <bool MHD>
__global__ void __launch_bounds__(256) k_c2p_df(Geom g, StagePtrs<double> p, Box bx, Phys ph,
                                                float2* __restrict__ wpairs) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  constexpr int NV = MHD ? 8 : 5;
  const int64_t nc = g.ncell, c = cidx(g, k, j, i);
  double* __restrict__ u = p.u + (int64_t)b * NHYD * nc;
  double* __restrict__ w = p.w + (int64_t)b * NHYD * nc;
  float2* __restrict__ wq = wpairs + (int64_t)b * NV * nc;
  // the conserved state first: its loads are issued before any store of this thread
  const double u0 = u[c], u1v = u[nc + c], u2v = u[2 * nc + c], u3v = u[3 * nc + c],
               u4v = u[4 * nc + c];
  dfl pb(0.0f, 0.0f);
  if constexpr (MHD) {
    const double* b1 = p.b1 + (int64_t)b * g.nf1;
    const double* b2 = p.b2 + (int64_t)b * g.nf2;
    const double* b3 = p.b3 + (int64_t)b * g.nf3;
    const int64_t q1 = f1idx(g, k, j, i), q2 = f2idx(g, k, j, i), q3 = f3idx(g, k, j, i);
    const dfl half(0.5f, 0.0f);
    const dfl bc[3] = {half * (df_of(b1[q1]) + df_of(b1[q1 + 1])),
                       half * (df_of(b2[q2]) + df_of(b2[q2 + g.nc1])),
                       half * (df_of(b3[q3]) + df_of(b3[q3 + (int64_t)g.nc1 * g.nc2]))};
    double* bcc = p.bcc + (int64_t)b * 3 * nc;
#pragma unroll
    for (int n = 0; n < 3; ++n) {
      bcc[n * nc + c] = dbl(bc[n]);
      wq[(NHYD + n) * nc + c] = make_float2(bc[n].hi, bc[n].lo);
    }
    pb = half * (bc[0] * bc[0] + bc[1] * bc[1] + bc[2] * bc[2]);
  }
  double ud = u0;
  const uint64_t ub = bits_d(ud);
  if (!((ub >> 63) == 0 && ub > bits_d(ph.dfloor) && ub <= 0x7ff0000000000000ull)) ud = ph.dfloor;
  u[c] = ud;
  const dfl dd = df_of(ud), m1 = df_of(u1v), m2 = df_of(u2v), m3 = df_of(u3v);
  const dfl di = dfl(1.0f, 0.0f) / dd;
  const dfl ek = dfl(0.5f, 0.0f) * di * (m1 * m1 + m2 * m2 + m3 * m3);
  const dfl gm1(ph.gm1f.hi, ph.gm1f.lo), pfl(ph.pfloorf.hi, ph.pfloorf.lo);
  dfl wp = gm1 * ((df_of(u4v) - ek) - pb);
  const bool floored = !(wp > pfl);
  if (floored) {
    u[4 * nc + c] = dbl((df_of(ph.pfloor / ph.gm1) + ek) + pb);
    wp = pfl;
  }
  const dfl v1 = m1 * di, v2 = m2 * di, v3 = m3 * di;
  w[c] = ud;
  w[nc + c] = dbl(v1);
  w[2 * nc + c] = dbl(v2);
  w[3 * nc + c] = dbl(v3);
  w[4 * nc + c] = floored ? ph.pfloor : dbl(wp);
  wq[c] = make_float2(dd.hi, dd.lo);
  wq[nc + c] = make_float2(v1.hi, v1.lo);
  wq[2 * nc + c] = make_float2(v2.hi, v2.lo);
  wq[3 * nc + c] = make_float2(v3.hi, v3.lo);
  wq[4 * nc + c] = make_float2(wp.hi, wp.lo);
}

// Hydro::NewBlockTimeStep (the formula of k_block_dt) in double-float from the pairs of
// k_c2p_df; the block minimum is taken on the FP64 values.
template <bool MHD>
__global__ void __launch_bounds__(256) k_dt_df(Geom g, StagePtrs<double> p, Box bx, Phys ph,
                                               const float2* __restrict__ wpairs,
                                               unsigned long long* dtmin) {
  int i, j, k, b;
  double mindt = 1.79769313486231570815e308;
  if (box_coords(bx, i, j, k, b)) {
    constexpr int NV = MHD ? 8 : 5;
    const int64_t nc = g.ncell, c = cidx(g, k, j, i);
    const float2* wq = wpairs + (int64_t)b * NV * nc;
    const dfl d = ps(wq, c), vx = ps(wq, nc + c), vy = ps(wq, 2 * nc + c),
              vz = ps(wq, 3 * nc + c), pr = ps(wq, 4 * nc + c);
    const BlockGeo geo = p.geo[b];
    const dfl dx1 = df_of(geo.dx[0]), dx2 = df_of(geo.dx[1]), dx3 = df_of(geo.dx[2]);
    const dfl gam = df_of(ph.gamma);
    dfl dt1, dt2, dt3;
    if constexpr (MHD) {
      const dfl bc1 = ps(wq, 5 * nc + c), bc2 = ps(wq, 6 * nc + c), bc3 = ps(wq, 7 * nc + c);
      const dfl bx1 = bc1 + fabs(df_of(p.bf[0][(int64_t)b * g.nf1 + f1idx(g, k, j, i)]) - bc1);
      dfl cf = fast_speed<dfl>(d, pr, bc2, bc3, bx1, gam);
      dt1 = dx1 / (fabs(vx) + cf);
      const dfl bx2 = bc2 + fabs(df_of(p.bf[1][(int64_t)b * g.nf2 + f2idx(g, k, j, i)]) - bc2);
      cf = fast_speed<dfl>(d, pr, bc3, bc1, bx2, gam);
      dt2 = dx2 / (fabs(vy) + cf);
      const dfl bx3 = bc3 + fabs(df_of(p.bf[2][(int64_t)b * g.nf3 + f3idx(g, k, j, i)]) - bc3);
      cf = fast_speed<dfl>(d, pr, bc1, bc2, bx3, gam);
      dt3 = dx3 / (fabs(vz) + cf);
    } else {
      const dfl cs = sqrt(gam * pr / d);
      dt1 = dx1 / (fabs(vx) + cs);
      dt2 = dx2 / (fabs(vy) + cs);
      dt3 = dx3 / (fabs(vz) + cs);
    }
    const dfl m = mn(mn(dt1, dt2), dt3);
    mindt = dbl(m);
  }
  for (int o = 16; o > 0; o >>= 1) mindt = fmin(mindt, __shfl_xor_sync(0xffffffffu, mindt, o));
  __shared__ double red[8];
  const int tid = threadIdx.x;
  if ((tid & 31) == 0) red[tid >> 5] = mindt;
  __syncthreads();
  if (tid < 32) {
    double v = (tid < (int)((blockDim.x + 31) / 32)) ? red[tid] : 1.79769313486231570815e308;
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (tid == 0) atomicMin(dtmin, (unsigned long long)__double_as_longlong(v));
  }
}

Box box_of(int il, int iu, int jl, int ju, int kl, int ku) {
  return box_make(il, iu, jl, ju, kl, ku);
}
dim3 grid_of(const Box& b, int nb) {
  return dim3((unsigned)((b.ni * b.nj + kThreads - 1) / kThreads), (unsigned)b.nk, (unsigned)nb);
}

template <int DIR, int ORDER, bool PAIRS>
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
    if (solver == HLLD)
      k_flux_df<DIR, ORDER, HLLD, true, PAIRS><<<gr, kThreads, 0, st>>>(g, p, b, ph, wp);
    else k_flux_df<DIR, ORDER, HLLE, true, PAIRS><<<gr, kThreads, 0, st>>>(g, p, b, ph, wp);
  } else {
    if (solver == HLLC)
      k_flux_df<DIR, ORDER, HLLC, false, PAIRS><<<gr, kThreads, 0, st>>>(g, p, b, ph, wp);
    else k_flux_df<DIR, ORDER, HLLE, false, PAIRS><<<gr, kThreads, 0, st>>>(g, p, b, ph, wp);
  }
}
template <bool PAIRS>
void sweeps(const Geom& g, const StagePtrs<double>& p, bool mhd, int solver, int order,
            const Phys& ph, const float2* wp, cudaStream_t st) {
  if (order == 1) {
    sweep<0, 1, PAIRS>(g, p, mhd, solver, ph, wp, st);
    sweep<1, 1, PAIRS>(g, p, mhd, solver, ph, wp, st);
    sweep<2, 1, PAIRS>(g, p, mhd, solver, ph, wp, st);
  } else {
    sweep<0, 2, PAIRS>(g, p, mhd, solver, ph, wp, st);
    sweep<1, 2, PAIRS>(g, p, mhd, solver, ph, wp, st);
    sweep<2, 2, PAIRS>(g, p, mhd, solver, ph, wp, st);
  }
}

}  // namespace

bool df_supported(int mhd, int solver, int xorder) {
  const bool s = mhd ? (solver == HLLD || solver == HLLE) : (solver == HLLC || solver == HLLE);
  return s && (xorder == 1 || xorder == 2);
}

void df_fluxes(const Geom& g, const StagePtrs<double>& p, bool mhd, int solver, int order,
               const Phys& ph, float2* wp, bool fast, cudaStream_t st) {
  if (fast) {  // k_c2p_df left the pairs; the fluxes go to k_update_df as pairs
    sweeps<true>(g, p, mhd, solver, order, ph, wp, st);
    return;
  }
  const int nv = mhd ? 8 : 5;
  k_split_w<<<dim3((unsigned)((g.ncell + 255) / 256), (unsigned)g.nb), 256, 0, st>>>(g, p, nv, wp);
  sweeps<false>(g, p, mhd, solver, order, ph, wp, st);
}

void df_corner_emf(const Geom& g, const StagePtrs<double>& p, float2* cce, const float2* wp,
                   bool fast, cudaStream_t st) {
  const Box c = box_of(g.is - 1, g.ie + 1, g.js - 1, g.je + 1, g.ks - 1, g.ke + 1);
  k_cce_df<<<grid_of(c, g.nb), kThreads, 0, st>>>(g, p, c, cce, fast ? wp : nullptr);
  const Box b = box_of(g.is, g.ie + 1, g.js, g.je + 1, g.ks, g.ke + 1);
  if (fast) k_corner_df<true><<<grid_of(b, g.nb), kThreads, 0, st>>>(g, p, b, cce);
  else k_corner_df<false><<<grid_of(b, g.nb), kThreads, 0, st>>>(g, p, b, cce);
}

void df_update(const Geom& g, const StagePtrs<double>& p, bool mhd, const StageW& sw,
               cudaStream_t st) {
  const Box b = mhd ? box_of(g.is, g.ie + 1, g.js, g.je + 1, g.ks, g.ke + 1)
                    : box_of(g.is, g.ie, g.js, g.je, g.ks, g.ke);
  const bool copy = sw.zero_reg && sw.delta == 1.0;  // a first stage's register copy
  if (mhd) {
    if (copy) k_update_df<true, true><<<grid_of(b, g.nb), kThreads, 0, st>>>(g, p, b, sw);
    else k_update_df<true, false><<<grid_of(b, g.nb), kThreads, 0, st>>>(g, p, b, sw);
  } else {
    if (copy) k_update_df<false, true><<<grid_of(b, g.nb), kThreads, 0, st>>>(g, p, b, sw);
    else k_update_df<false, false><<<grid_of(b, g.nb), kThreads, 0, st>>>(g, p, b, sw);
  }
}

void df_c2p(const Geom& g, const StagePtrs<double>& p, bool mhd, const Phys& ph, float2* wp,
            cudaStream_t st) {
  const Box b = box_of(0, g.nc1 - 1, 0, g.nc2 - 1, 0, g.nc3 - 1);
  const dim3 gr((unsigned)((b.ni * b.nj + 255) / 256), (unsigned)b.nk, (unsigned)g.nb);
  if (mhd) k_c2p_df<true><<<gr, 256, 0, st>>>(g, p, b, ph, wp);
  else k_c2p_df<false><<<gr, 256, 0, st>>>(g, p, b, ph, wp);
}

void df_block_dt(const Geom& g, const StagePtrs<double>& p, bool mhd, const Phys& ph,
                 const float2* wp, unsigned long long* dtmin, cudaStream_t st) {
  const Box b = box_of(g.is, g.ie, g.js, g.je, g.ks, g.ke);
  const dim3 gr((unsigned)((b.ni * b.nj + 255) / 256), (unsigned)b.nk, (unsigned)g.nb);
  if (mhd) k_dt_df<true><<<gr, 256, 0, st>>>(g, p, b, ph, wp, dtmin);
  else k_dt_df<false><<<gr, 256, 0, st>>>(g, p, b, ph, wp, dtmin);
}

}  // namespace athg

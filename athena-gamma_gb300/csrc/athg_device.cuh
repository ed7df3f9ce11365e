// athg_device.cuh -- device-side layout, EOS helpers and Riemann solvers.
//
// Block-pool layout (one pool for all MeshBlocks, every block the same interior size):
//   cell arrays   [block][var][k][j][i]   nc = nx + 2*ng per axis, i fastest
//                 (the AthenaArray (n,k,j,i) layout of one block, reference
//                  src/athena_arrays.hpp:140, so upload/download is one memcpy per block)
//   x1-face       [block][k][j][i]  (nc3, nc2, nc1+1)   src/athena.hpp:95-102
//   x2-face       [block][k][j][i]  (nc3, nc2+1, nc1)
//   x3-face       [block][k][j][i]  (nc3+1, nc2, nc1)
//   edges         [block][comp][k][j][i] (nc3+1, nc2+1, nc1+1)
// Conserved variables and face fields are always FP64. Primitives, reconstructed
// states, Riemann fluxes and face EMFs use the template type T: double for the plain
// FP64 path, float for the mixed path.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "athg_numeric.h"

namespace athg {

constexpr int NHYD = 5;
constexpr int IDN = 0, IVX = 1, IVY = 2, IVZ = 3, IPR = 4, IEN = 4, IBY = 5, IBZ = 6;
enum Solver { HLLE = 0, HLLC = 1, HLLD = 2, LHLLC = 3, LHLLD = 4 };

// Sizes shared by every block of the pool.
struct Geom {
  int nx1, nx2, nx3, ng;
  int nc1, nc2, nc3;
  int is, ie, js, je, ks, ke;
  int64_t ncell, nf1, nf2, nf3, ne;
  int nb;
  int ncmax;  // max(nc1, nc2, nc3), stride of the per-block coefficient arrays
  // divisions of the ghost-shell index (ghost_shell_pos): by nc1 + 1, nc2 + 1, the ghost
  // rows and columns per side pair (nc2 + 1 - nx2, nc1 + 1 - nx1) and nx2
  FastDiv dw1, dw2, dgj, dgi, dnx2;
};

__host__ __device__ inline int64_t cidx(const Geom& g, int k, int j, int i) {
  return ((int64_t)k * g.nc2 + j) * g.nc1 + i;
}
__host__ __device__ inline int64_t f1idx(const Geom& g, int k, int j, int i) {
  return ((int64_t)k * g.nc2 + j) * (g.nc1 + 1) + i;
}
__host__ __device__ inline int64_t f2idx(const Geom& g, int k, int j, int i) {
  return ((int64_t)k * (g.nc2 + 1) + j) * g.nc1 + i;
}
__host__ __device__ inline int64_t f3idx(const Geom& g, int k, int j, int i) {
  return cidx(g, k, j, i);
}
__host__ __device__ inline int64_t eidx(const Geom& g, int k, int j, int i) {
  return ((int64_t)k * (g.nc2 + 1) + j) * (g.nc1 + 1) + i;
}
template <int DIR>
__host__ __device__ inline int64_t fidx(const Geom& g, int k, int j, int i) {
  return DIR == 0 ? f1idx(g, k, j, i) : (DIR == 1 ? f2idx(g, k, j, i) : f3idx(g, k, j, i));
}
template <int DIR>
__host__ __device__ inline int64_t fsize(const Geom& g) {
  return DIR == 0 ? g.nf1 : (DIR == 1 ? g.nf2 : g.nf3);
}

// Per-block geometry (uniform Cartesian: one width per axis).
struct BlockGeo {
  double dx[3];
};

// Physics constants of a run.
struct Phys {
  double gamma, dfloor, pfloor;
  double gm1;  // gamma - 1
  ff gm1f, pfloorf;  // the same as double-float pairs (mixed primitive recovery)
  float gammas, dfloors, pfloors;  // rounded to FP32 on the host (no FP64 pipe in FP32 kernels)
};

// gamma and the floors in the flux precision
template <typename T> __device__ __forceinline__ T ph_gamma(const Phys& ph) {
  if constexpr (sizeof(T) == 4) return ph.gammas; else return ph.gamma;
}
template <typename T> __device__ __forceinline__ T ph_dfloor(const Phys& ph) {
  if constexpr (sizeof(T) == 4) return ph.dfloors; else return ph.dfloor;
}
template <typename T> __device__ __forceinline__ T ph_pfloor(const Phys& ph) {
  if constexpr (sizeof(T) == 4) return ph.pfloors; else return ph.pfloor;
}

// Stage weights of the low-storage integrator (reference
// src/task_list/time_integrator.cpp:100-600, applied as in :1563-1653).
struct StageW {
  double delta, g1, g2, beta;
  int swap;  // g1==0 && g2==1 && g3==0: the reference swaps registers
  int zero_reg;  // first stage: the register starts from zero
  int copy_reg;  // zero_reg && delta == 1: the register becomes a copy of the state
  int has_delta;  // delta != 0
  float betaf;  // beta in FP32 (mixed path)
};

// Per-block widths of the mixed-path update. Same-level blocks of a uniform mesh share one
// set of values, so a face flux or an edge EMF enters both neighbours with the same
// FP32 weight and the sums telescope (conservation and div B stay at round-off).
struct MixedGeo {
  float idx[3];    // 1 / dx_d
  float dx[3];     // dx_d
  double ia[3];    // dx_d / (dx1 dx2 dx3): face-flux change -> face-field change
  float idxh[3], idxl[3];  // 1 / dx_d as a double-float pair (double-float path)
};

// Comparisons. FP64 comparisons (and min/max) issue on the FP64 pipe, which runs at 1/64 of
// the FP32 rate on this GPU and bounds the FP64 flux sweeps, so for doubles they are made
// on the integer pipe: dkey maps a double to an int64 that orders like the value for every
// non-NaN double, with -0 equal to +0, so lt/le/gt/ge give the IEEE results. (With a NaN
// operand IEEE comparisons are all false; these order the NaN instead.)
__device__ __forceinline__ long long dkey(double x) {
  long long b = __double_as_longlong(x);
  b = ((unsigned long long)b << 1) == 0ull ? 0ll : b;
  return b < 0 ? (b ^ 0x7fffffffffffffffll) : b;
}
template <typename T> __device__ __forceinline__ bool lt(T a, T b) {
  if constexpr (sizeof(T) == 8) return dkey(a) < dkey(b); else return a < b;
}
template <typename T> __device__ __forceinline__ bool le(T a, T b) {
  if constexpr (sizeof(T) == 8) return dkey(a) <= dkey(b); else return a <= b;
}
template <typename T> __device__ __forceinline__ bool gt(T a, T b) { return lt(b, a); }
template <typename T> __device__ __forceinline__ bool ge(T a, T b) { return le(b, a); }
// |x| by clearing the sign bit (integer pipe for doubles)
template <typename T> __device__ __forceinline__ T fab(T x) {
  if constexpr (sizeof(T) == 8)
    return __longlong_as_double(__double_as_longlong(x) & 0x7fffffffffffffffll);
  else
    return fabsf(x);
}

// std::min / std::max semantics (first argument wins ties)
template <typename T> __device__ __forceinline__ T mn(T a, T b) { return lt(b, a) ? b : a; }
template <typename T> __device__ __forceinline__ T mx(T a, T b) { return lt(a, b) ? b : a; }
template <typename T> __device__ __forceinline__ T sq(T x) { return x * x; }

// eos/adiabatic_mhd.cpp:149-156 (fast magnetosonic speed)
template <typename T>
__device__ __forceinline__ T fast_speed(T d, T p, T by, T bz, T bx, T gamma) {
  T asq = gamma * p;
  T vaxsq = bx * bx;
  T ct2 = (by * by + bz * bz);
  T qsq = vaxsq + ct2 + asq;
  T tmp = vaxsq + ct2 - asq;
  return sqrt(T(0.5) * (qsq + sqrt(tmp * tmp + T(4.0) * asq * ct2)) / d);
}

// hydro/hydro.cpp:154-158 (upwind weight for the corner EMF)
template <typename T>
__device__ __forceinline__ T ct_weight(T dflx, T rhol, T rhor, T dx, T dt) {
  T v_over_c = (T(1024.0)) * dt * dflx / (dx * (rhol + rhor));
  T tmp_min = mn(T(0.5), v_over_c);
  return T(0.5) + mx(T(-0.5), tmp_min);
}

template <typename T> __device__ __forceinline__ T sgn(T x) { return lt(x, T(0.0)) ? T(-1.0) : T(1.0); }

// PPM of one cell on a uniform Cartesian axis: Colella-Woodward interface values with the
// Colella-Sekora extremum-preserving limiter (reference src/reconstruct/ppm.cpp:44-342,
// uniform weights 0.5 and +-1/6 of src/reconstruct/reconstruction.cpp:420-431). From the
// five cell values q[-2..2] it returns the states at the cell's lower (qm) and upper (qp)
// faces.
template <typename T>
__device__ __forceinline__ void ppm_cell(T q_im2, T q_im1, T q, T q_ip1, T q_ip2, T& qm, T& qp) {
  const T C2 = T(1.25);
  const T c1 = T(0.5), c2 = T(0.5), c3 = T(0.5), c4 = T(0.5);
  const T c5 = T(1.0 / 6.0), c6 = T(-1.0 / 6.0);
  T qa = (q - q_im1);
  T qb = (q_ip1 - q);
  T dd_im1 = c1 * qa + c2 * (q_im1 - q_im2);
  T dd = c1 * qb + c2 * qa;
  T dd_ip1 = c1 * (q_ip2 - q_ip1) + c2 * qb;
  T dph = (c3 * q_im1 + c4 * q) + (c5 * dd_im1 + c6 * dd);
  T dph_ip1 = (c3 * q + c4 * q_ip1) + (c5 * dd + c6 * dd_ip1);
  T d2qc_im1 = q_im2 + q - T(2.0) * q_im1;
  T d2qc = q_im1 + q_ip1 - T(2.0) * q;
  T d2qc_ip1 = q + q_ip2 - T(2.0) * q_ip1;
  {
    T qa_tmp = dph - q_im1, qb_tmp = q - dph;
    T a = T(3.0) * (q_im1 + q - T(2.0) * dph), b = d2qc_im1, c = d2qc;
    T qd = T(0.0);
    // sgn(a) * min(...) with sgn in {-1, 1}: a sign flip
    const bool na = lt(a, T(0.0)), nb = lt(b, T(0.0)), ncc = lt(c, T(0.0));
    if (na == nb && na == ncc) {
      const T m = mn(C2 * fab(b), mn(C2 * fab(c), fab(a)));
      qd = na ? -m : m;
    }
    T dph_tmp = T(0.5) * (q_im1 + q) - qd / T(6.0);
    if (lt(qa_tmp * qb_tmp, T(0.0))) dph = dph_tmp;
  }
  {
    T qa_tmp = dph_ip1 - q, qb_tmp = q_ip1 - dph_ip1;
    T a = T(3.0) * (q + q_ip1 - T(2.0) * dph_ip1), b = d2qc, c = d2qc_ip1;
    T qd = T(0.0);
    const bool na = lt(a, T(0.0)), nb = lt(b, T(0.0)), ncc = lt(c, T(0.0));
    if (na == nb && na == ncc) {
      const T m = mn(C2 * fab(b), mn(C2 * fab(c), fab(a)));
      qd = na ? -m : m;
    }
    T dphip1_tmp = T(0.5) * (q + q_ip1) - qd / T(6.0);
    if (lt(qa_tmp * qb_tmp, T(0.0))) dph_ip1 = dphip1_tmp;
  }
  T d2qf = T(6.0) * (dph + dph_ip1 - T(2.0) * q);
  T qminus = dph, qplus = dph_ip1;
  T dqf_minus = q - qminus, dqf_plus = qplus - q;
  T qa_tmp = dqf_minus * dqf_plus;
  T qb_tmp = (q_ip1 - q) * (q - q_im1);
  T a = d2qc_im1, b = d2qc, c = d2qc_ip1, d = d2qf, qe = T(0.0);
  {
    const bool na = lt(a, T(0.0)), nb = lt(b, T(0.0)), ncc = lt(c, T(0.0)), nd = lt(d, T(0.0));
    if (na == nb && na == ncc && na == nd) {
      const T m = mn(mn(C2 * fab(a), C2 * fab(b)), mn(C2 * fab(c), fab(d)));
      qe = nd ? -m : m;
    }
  }
  a = mx(fab(q_im1), fab(q_im2));
  b = mx(mx(fab(q), fab(q_ip1)), fab(q_ip2));
  T rho = T(0.0);
  if (gt(fab(d), T(1.0e-12) * mx(a, b))) rho = qe / d;
  T tmp_m = q - rho * dqf_minus, tmp_p = q + rho * dqf_plus;
  T tmp2_m = q - T(2.0) * dqf_plus, tmp2_p = q + T(2.0) * dqf_minus;
  if ((le(qa_tmp, T(0.0)) || le(qb_tmp, T(0.0)))) {
    if (le(rho, (T(1.0) - T(1.0e-12)))) {
      qminus = tmp_m;
      qplus = tmp_p;
    }
  } else {
    if (ge(fab(dqf_minus), T(2.0) * fab(dqf_plus))) qminus = tmp2_m;
    if (ge(fab(dqf_plus), T(2.0) * fab(dqf_minus))) qplus = tmp2_p;
  }
  qm = qminus;
  qp = qplus;
}

// ------------------------------------------------------------------------------------
// Riemann solvers. Input states are in the rotated order (d, vn, vt1, vt2, p[, by, bz]);
// the flux comes back in the same order.

// HLLC, Toro PVRS wave speeds (reference hydro/rsolvers/hydro/hllc.cpp:54-168)
template <typename T>
__device__ __forceinline__ void rs_hllc(const T* wli, const T* wri, T gamma, T* flxi) {
  const T gm1 = gamma - T(1.0), igm1 = T(1.0) / gm1;
  T cl = sqrt(gamma * wli[IPR] / wli[IDN]);
  T cr = sqrt(gamma * wri[IPR] / wri[IDN]);
  T el = wli[IPR] * igm1 + T(0.5) * wli[IDN] * (sq(wli[IVX]) + sq(wli[IVY]) + sq(wli[IVZ]));
  T er = wri[IPR] * igm1 + T(0.5) * wri[IDN] * (sq(wri[IVX]) + sq(wri[IVY]) + sq(wri[IVZ]));
  T rhoa = T(.5) * (wli[IDN] + wri[IDN]);
  T ca = T(.5) * (cl + cr);
  T pmid = T(.5) * (wli[IPR] + wri[IPR] + (wli[IVX] - wri[IVX]) * rhoa * ca);
  T ql = (pmid <= wli[IPR]) ? T(1.0)
         : sqrt(T(1.0) + (gamma + T(1)) / (T(2) * gamma) * (pmid / wli[IPR] - T(1.0)));
  T qr = (pmid <= wri[IPR]) ? T(1.0)
         : sqrt(T(1.0) + (gamma + T(1)) / (T(2) * gamma) * (pmid / wri[IPR] - T(1.0)));
  T al = wli[IVX] - cl * ql;
  T ar = wri[IVX] + cr * qr;
  T bp = ar > T(0.0) ? ar : T(1.0e-20);
  T bm = al < T(0.0) ? al : -T(1.0e-20);
  T vxl = wli[IVX] - al;
  T vxr = wri[IVX] - ar;
  T tl = wli[IPR] + vxl * wli[IDN] * wli[IVX];
  T tr = wri[IPR] + vxr * wri[IDN] * wri[IVX];
  T ml = wli[IDN] * vxl;
  T mr = -(wri[IDN] * vxr);
  T am = (tl - tr) / (ml + mr);
  T cp = (ml * tr + mr * tl) / (ml + mr);
  cp = cp > T(0.0) ? cp : T(0.0);
  vxl = wli[IVX] - bm;
  vxr = wri[IVX] - bp;
  T fl0 = wli[IDN] * vxl, fr0 = wri[IDN] * vxr;
  T fl1 = wli[IDN] * wli[IVX] * vxl + wli[IPR], fr1 = wri[IDN] * wri[IVX] * vxr + wri[IPR];
  T fl2 = wli[IDN] * wli[IVY] * vxl, fr2 = wri[IDN] * wri[IVY] * vxr;
  T fl3 = wli[IDN] * wli[IVZ] * vxl, fr3 = wri[IDN] * wri[IVZ] * vxr;
  T fl4 = el * vxl + wli[IPR] * wli[IVX], fr4 = er * vxr + wri[IPR] * wri[IVX];
  T sl, sr, sm;
  if (am >= T(0.0)) {
    sl = am / (am - bm); sr = T(0.0); sm = -bm / (am - bm);
  } else {
    sl = T(0.0); sr = -am / (bp - am); sm = bp / (bp - am);
  }
  flxi[IDN] = sl * fl0 + sr * fr0;
  flxi[IVX] = sl * fl1 + sr * fr1 + sm * cp;
  flxi[IVY] = sl * fl2 + sr * fr2;
  flxi[IVZ] = sl * fl3 + sr * fr3;
  flxi[IEN] = sl * fl4 + sr * fr4 + sm * cp * am;
}

// HLLE with Roe-averaged speeds, adiabatic hydro (hydro/rsolvers/hydro/hlle.cpp:64-151)
template <typename T>
__device__ __forceinline__ void rs_hlle_hydro(const T* wli, const T* wri, T gamma, T* flxi) {
  const T gm1 = gamma - T(1.0), igm1 = T(1.0) / gm1;
  T sqrtdl = sqrt(wli[IDN]), sqrtdr = sqrt(wri[IDN]);
  T isdlpdr = T(1.0) / (sqrtdl + sqrtdr);
  T rvx = (sqrtdl * wli[IVX] + sqrtdr * wri[IVX]) * isdlpdr;
  T rvy = (sqrtdl * wli[IVY] + sqrtdr * wri[IVY]) * isdlpdr;
  T rvz = (sqrtdl * wli[IVZ] + sqrtdr * wri[IVZ]) * isdlpdr;
  T el = wli[IPR] * igm1 + T(0.5) * wli[IDN] * (sq(wli[IVX]) + sq(wli[IVY]) + sq(wli[IVZ]));
  T er = wri[IPR] * igm1 + T(0.5) * wri[IDN] * (sq(wri[IVX]) + sq(wri[IVY]) + sq(wri[IVZ]));
  T hroe = ((el + wli[IPR]) / sqrtdl + (er + wri[IPR]) / sqrtdr) * isdlpdr;
  T cl = sqrt(gamma * wli[IPR] / wli[IDN]);
  T cr = sqrt(gamma * wri[IPR] / wri[IDN]);
  T q = hroe - T(0.5) * (sq(rvx) + sq(rvy) + sq(rvz));
  T a = (q < T(0.0)) ? T(0.0) : sqrt(gm1 * q);
  T al = mn(rvx - a, wli[IVX] - cl);
  T ar = mx(rvx + a, wri[IVX] + cr);
  T bp = ar > T(0.0) ? ar : T(0.0);
  T bm = al < T(0.0) ? al : T(0.0);
  T vxl = wli[IVX] - bm, vxr = wri[IVX] - bp;
  T fl[5], fr[5];
  fl[IDN] = wli[IDN] * vxl; fr[IDN] = wri[IDN] * vxr;
  fl[IVX] = wli[IDN] * wli[IVX] * vxl; fr[IVX] = wri[IDN] * wri[IVX] * vxr;
  fl[IVY] = wli[IDN] * wli[IVY] * vxl; fr[IVY] = wri[IDN] * wri[IVY] * vxr;
  fl[IVZ] = wli[IDN] * wli[IVZ] * vxl; fr[IVZ] = wri[IDN] * wri[IVZ] * vxr;
  fl[IVX] += wli[IPR]; fr[IVX] += wri[IPR];
  fl[IEN] = el * vxl + wli[IPR] * wli[IVX];
  fr[IEN] = er * vxr + wri[IPR] * wri[IVX];
  T tmp = T(0.0);
  if (bp != bm) tmp = T(0.5) * (bp + bm) / (bp - bm);
#pragma unroll
  for (int n = 0; n < 5; ++n) flxi[n] = T(0.5) * (fl[n] + fr[n]) + (fl[n] - fr[n]) * tmp;
}

// HLLE for adiabatic MHD (hydro/rsolvers/mhd/hlle_mhd.cpp:60-163)
template <typename T>
__device__ __forceinline__ void rs_hlle_mhd(const T* wli, const T* wri, T bxi, T gamma,
                                            T* flxi) {
  const T gm1 = gamma - T(1.0);
  T sqrtdl = sqrt(wli[IDN]), sqrtdr = sqrt(wri[IDN]);
  T isdlpdr = T(1.0) / (sqrtdl + sqrtdr);
  T rd = sqrtdl * sqrtdr;
  T rvx = (sqrtdl * wli[IVX] + sqrtdr * wri[IVX]) * isdlpdr;
  T rvy = (sqrtdl * wli[IVY] + sqrtdr * wri[IVY]) * isdlpdr;
  T rvz = (sqrtdl * wli[IVZ] + sqrtdr * wri[IVZ]) * isdlpdr;
  T rby = (sqrtdr * wli[IBY] + sqrtdl * wri[IBY]) * isdlpdr;
  T rbz = (sqrtdr * wli[IBZ] + sqrtdl * wri[IBZ]) * isdlpdr;
  T x = T(0.5) * (sq(wli[IBY] - wri[IBY]) + sq(wli[IBZ] - wri[IBZ])) / (sq(sqrtdl + sqrtdr));
  T y = T(0.5) * (wli[IDN] + wri[IDN]) / rd;
  T pbl = T(0.5) * (bxi * bxi + sq(wli[IBY]) + sq(wli[IBZ]));
  T pbr = T(0.5) * (bxi * bxi + sq(wri[IBY]) + sq(wri[IBZ]));
  T el = wli[IPR] / gm1 + T(0.5) * wli[IDN] * (sq(wli[IVX]) + sq(wli[IVY]) + sq(wli[IVZ])) + pbl;
  T er = wri[IPR] / gm1 + T(0.5) * wri[IDN] * (sq(wri[IVX]) + sq(wri[IVY]) + sq(wri[IVZ])) + pbr;
  T hroe = ((el + wli[IPR] + pbl) / sqrtdl + (er + wri[IPR] + pbr) / sqrtdr) * isdlpdr;
  T cl = fast_speed(wli[IDN], wli[IPR], wli[IBY], wli[IBZ], bxi, gamma);
  T cr = fast_speed(wri[IDN], wri[IPR], wri[IBY], wri[IBZ], bxi, gamma);
  T btsq = sq(rby) + sq(rbz);
  T vaxsq = bxi * bxi / rd;
  T bt_starsq = (gm1 - (gm1 - T(1.0)) * y) * btsq;
  T hp = hroe - (vaxsq + btsq / rd);
  T vsq = sq(rvx) + sq(rvy) + sq(rvz);
  T twid_asq = mx((gm1 * (hp - T(0.5) * vsq) - (gm1 - T(1.0)) * x), T(0.0));
  T ct2 = bt_starsq / rd;
  T tsum = vaxsq + ct2 + twid_asq;
  T tdif = vaxsq + ct2 - twid_asq;
  T cf2_cs2 = sqrt(tdif * tdif + T(4.0) * twid_asq * ct2);
  T cfsq = T(0.5) * (tsum + cf2_cs2);
  T a = sqrt(cfsq);
  T al = mn((rvx - a), (wli[IVX] - cl));
  T ar = mx((rvx + a), (wri[IVX] + cr));
  T bp = ar > T(0.0) ? ar : T(0.0);
  T bm = al < T(0.0) ? al : T(0.0);
  T vxl = wli[IVX] - bm, vxr = wri[IVX] - bp;
  T fl[7], fr[7];
  fl[IDN] = wli[IDN] * vxl; fr[IDN] = wri[IDN] * vxr;
  fl[IVX] = wli[IDN] * wli[IVX] * vxl + pbl - sq(bxi);
  fr[IVX] = wri[IDN] * wri[IVX] * vxr + pbr - sq(bxi);
  fl[IVY] = wli[IDN] * wli[IVY] * vxl - bxi * wli[IBY];
  fr[IVY] = wri[IDN] * wri[IVY] * vxr - bxi * wri[IBY];
  fl[IVZ] = wli[IDN] * wli[IVZ] * vxl - bxi * wli[IBZ];
  fr[IVZ] = wri[IDN] * wri[IVZ] * vxr - bxi * wri[IBZ];
  fl[IVX] += wli[IPR]; fr[IVX] += wri[IPR];
  fl[IEN] = el * vxl + wli[IVX] * (wli[IPR] + pbl - bxi * bxi);
  fr[IEN] = er * vxr + wri[IVX] * (wri[IPR] + pbr - bxi * bxi);
  fl[IEN] -= bxi * (wli[IBY] * wli[IVY] + wli[IBZ] * wli[IVZ]);
  fr[IEN] -= bxi * (wri[IBY] * wri[IVY] + wri[IBZ] * wri[IVZ]);
  fl[IBY] = wli[IBY] * vxl - bxi * wli[IVY];
  fr[IBY] = wri[IBY] * vxr - bxi * wri[IVY];
  fl[IBZ] = wli[IBZ] * vxl - bxi * wli[IVZ];
  fr[IBZ] = wri[IBZ] * vxr - bxi * wri[IVZ];
  T tmp = T(0.0);
  if (bp != bm) tmp = T(0.5) * (bp + bm) / (bp - bm);
#pragma unroll
  for (int n = 0; n < 7; ++n) flxi[n] = T(0.5) * (fl[n] + fr[n]) + (fl[n] - fr[n]) * tmp;
}

template <typename T> struct C1D { T d, mx, my, mz, e, by, bz; };

// HLLD, Miyoshi & Kusano (2005) five-wave solver (hydro/rsolvers/mhd/hlld.cpp:56-371)
template <typename T>
__device__ __forceinline__ void rs_hlld(const T* wli, const T* wri, T bxi, T gamma, T* flxi) {
  const T SMALLN = T(1.0e-8);
  const T igm1 = T(1.0) / (gamma - T(1.0));
  C1D<T> ul, ur, ulst, uldst, urdst, urst, fl, fr;
  T spd[5];
  T bxsq = bxi * bxi;
  T pbl = T(0.5) * (bxsq + (sq(wli[IBY]) + sq(wli[IBZ])));
  T pbr = T(0.5) * (bxsq + (sq(wri[IBY]) + sq(wri[IBZ])));
  T kel = T(0.5) * wli[IDN] * (sq(wli[IVX]) + (sq(wli[IVY]) + sq(wli[IVZ])));
  T ker = T(0.5) * wri[IDN] * (sq(wri[IVX]) + (sq(wri[IVY]) + sq(wri[IVZ])));
  ul.d = wli[IDN]; ul.mx = wli[IVX] * ul.d; ul.my = wli[IVY] * ul.d; ul.mz = wli[IVZ] * ul.d;
  ul.e = wli[IPR] * igm1 + kel + pbl; ul.by = wli[IBY]; ul.bz = wli[IBZ];
  ur.d = wri[IDN]; ur.mx = wri[IVX] * ur.d; ur.my = wri[IVY] * ur.d; ur.mz = wri[IVZ] * ur.d;
  ur.e = wri[IPR] * igm1 + ker + pbr; ur.by = wri[IBY]; ur.bz = wri[IBZ];
  T cfl = fast_speed(wli[IDN], wli[IPR], wli[IBY], wli[IBZ], bxi, gamma);
  T cfr = fast_speed(wri[IDN], wri[IPR], wri[IBY], wri[IBZ], bxi, gamma);
  spd[0] = mn(wli[IVX] - cfl, wri[IVX] - cfr);
  spd[4] = mx(wli[IVX] + cfl, wri[IVX] + cfr);
  T ptl = wli[IPR] + pbl, ptr = wri[IPR] + pbr;
  fl.d = ul.mx;
  fl.mx = ul.mx * wli[IVX] + ptl - bxsq;
  fl.my = ul.my * wli[IVX] - bxi * ul.by;
  fl.mz = ul.mz * wli[IVX] - bxi * ul.bz;
  fl.e = wli[IVX] * (ul.e + ptl - bxsq) - bxi * (wli[IVY] * ul.by + wli[IVZ] * ul.bz);
  fl.by = ul.by * wli[IVX] - bxi * wli[IVY];
  fl.bz = ul.bz * wli[IVX] - bxi * wli[IVZ];
  fr.d = ur.mx;
  fr.mx = ur.mx * wri[IVX] + ptr - bxsq;
  fr.my = ur.my * wri[IVX] - bxi * ur.by;
  fr.mz = ur.mz * wri[IVX] - bxi * ur.bz;
  fr.e = wri[IVX] * (ur.e + ptr - bxsq) - bxi * (wri[IVY] * ur.by + wri[IVZ] * ur.bz);
  fr.by = ur.by * wri[IVX] - bxi * wri[IVY];
  fr.bz = ur.bz * wri[IVX] - bxi * wri[IVZ];
  T sdl = spd[0] - wli[IVX], sdr = spd[4] - wri[IVX];
  spd[2] = (sdr * ur.mx - sdl * ul.mx + (ptl - ptr)) / (sdr * ur.d - sdl * ul.d);
  T sdml = spd[0] - spd[2], sdmr = spd[4] - spd[2];
  T sdml_inv = T(1.0) / sdml, sdmr_inv = T(1.0) / sdmr;
  ulst.d = ul.d * sdl * sdml_inv;
  urst.d = ur.d * sdr * sdmr_inv;
  T ulst_d_inv = T(1.0) / ulst.d, urst_d_inv = T(1.0) / urst.d;
  T sqrtdl = sqrt(ulst.d), sqrtdr = sqrt(urst.d);
  spd[1] = spd[2] - fabs(bxi) / sqrtdl;
  spd[3] = spd[2] + fabs(bxi) / sqrtdr;
  T ptstl = ptl + ul.d * sdl * (spd[2] - wli[IVX]);
  T ptstr = ptr + ur.d * sdr * (spd[2] - wri[IVX]);
  T ptst = T(0.5) * (ptstr + ptstl);
  ulst.mx = ulst.d * spd[2];
  if (fabs(ul.d * sdl * sdml - bxsq) < (SMALLN) * ptst) {
    ulst.my = ulst.d * wli[IVY]; ulst.mz = ulst.d * wli[IVZ];
    ulst.by = ul.by; ulst.bz = ul.bz;
  } else {
    T tmp = bxi * (sdl - sdml) / (ul.d * sdl * sdml - bxsq);
    ulst.my = ulst.d * (wli[IVY] - ul.by * tmp);
    ulst.mz = ulst.d * (wli[IVZ] - ul.bz * tmp);
    tmp = (ul.d * sq(sdl) - bxsq) / (ul.d * sdl * sdml - bxsq);
    ulst.by = ul.by * tmp; ulst.bz = ul.bz * tmp;
  }
  T vbstl = (ulst.mx * bxi + (ulst.my * ulst.by + ulst.mz * ulst.bz)) * ulst_d_inv;
  ulst.e = (sdl * ul.e - ptl * wli[IVX] + ptst * spd[2] +
            bxi * (wli[IVX] * bxi + (wli[IVY] * ul.by + wli[IVZ] * ul.bz) - vbstl)) * sdml_inv;
  urst.mx = urst.d * spd[2];
  if (fabs(ur.d * sdr * sdmr - bxsq) < (SMALLN) * ptst) {
    urst.my = urst.d * wri[IVY]; urst.mz = urst.d * wri[IVZ];
    urst.by = ur.by; urst.bz = ur.bz;
  } else {
    T tmp = bxi * (sdr - sdmr) / (ur.d * sdr * sdmr - bxsq);
    urst.my = urst.d * (wri[IVY] - ur.by * tmp);
    urst.mz = urst.d * (wri[IVZ] - ur.bz * tmp);
    tmp = (ur.d * sq(sdr) - bxsq) / (ur.d * sdr * sdmr - bxsq);
    urst.by = ur.by * tmp; urst.bz = ur.bz * tmp;
  }
  T vbstr = (urst.mx * bxi + (urst.my * urst.by + urst.mz * urst.bz)) * urst_d_inv;
  urst.e = (sdr * ur.e - ptr * wri[IVX] + ptst * spd[2] +
            bxi * (wri[IVX] * bxi + (wri[IVY] * ur.by + wri[IVZ] * ur.bz) - vbstr)) * sdmr_inv;
  if (T(0.5) * bxsq < (SMALLN) * ptst) {
    uldst = ulst; urdst = urst;
  } else {
    T invsumd = T(1.0) / (sqrtdl + sqrtdr);
    T bxsig = (bxi > T(0.0) ? T(1.0) : T(-1.0));
    uldst.d = ulst.d; urdst.d = urst.d;
    uldst.mx = ulst.mx; urdst.mx = urst.mx;
    T tmp = invsumd * (sqrtdl * (ulst.my * ulst_d_inv) + sqrtdr * (urst.my * urst_d_inv) +
                       bxsig * (urst.by - ulst.by));
    uldst.my = uldst.d * tmp; urdst.my = urdst.d * tmp;
    tmp = invsumd * (sqrtdl * (ulst.mz * ulst_d_inv) + sqrtdr * (urst.mz * urst_d_inv) +
                     bxsig * (urst.bz - ulst.bz));
    uldst.mz = uldst.d * tmp; urdst.mz = urdst.d * tmp;
    tmp = invsumd * (sqrtdl * urst.by + sqrtdr * ulst.by +
                     bxsig * sqrtdl * sqrtdr * ((urst.my * urst_d_inv) - (ulst.my * ulst_d_inv)));
    uldst.by = urdst.by = tmp;
    tmp = invsumd * (sqrtdl * urst.bz + sqrtdr * ulst.bz +
                     bxsig * sqrtdl * sqrtdr * ((urst.mz * urst_d_inv) - (ulst.mz * ulst_d_inv)));
    uldst.bz = urdst.bz = tmp;
    tmp = spd[2] * bxi + (uldst.my * uldst.by + uldst.mz * uldst.bz) / uldst.d;
    uldst.e = ulst.e - sqrtdl * bxsig * (vbstl - tmp);
    urdst.e = urst.e + sqrtdr * bxsig * (vbstr - tmp);
  }
  // Select the region of the fan that contains x/t = 0; differences of the
  // intermediate states scaled by the wave speeds are only formed where needed.
  auto dif = [](const C1D<T>& a, const C1D<T>& b, T s, T* o) {
    o[0] = s * (a.d - b.d); o[1] = s * (a.mx - b.mx); o[2] = s * (a.my - b.my);
    o[3] = s * (a.mz - b.mz); o[4] = s * (a.e - b.e); o[5] = s * (a.by - b.by);
    o[6] = s * (a.bz - b.bz);
  };
  T t0[7], t1[7];
  if (spd[0] >= T(0.0)) {
    flxi[IDN] = fl.d; flxi[IVX] = fl.mx; flxi[IVY] = fl.my; flxi[IVZ] = fl.mz;
    flxi[IEN] = fl.e; flxi[IBY] = fl.by; flxi[IBZ] = fl.bz;
  } else if (spd[4] <= T(0.0)) {
    flxi[IDN] = fr.d; flxi[IVX] = fr.mx; flxi[IVY] = fr.my; flxi[IVZ] = fr.mz;
    flxi[IEN] = fr.e; flxi[IBY] = fr.by; flxi[IBZ] = fr.bz;
  } else if (spd[1] >= T(0.0)) {
    dif(ulst, ul, spd[0], t0);
    flxi[IDN] = fl.d + t0[0]; flxi[IVX] = fl.mx + t0[1]; flxi[IVY] = fl.my + t0[2];
    flxi[IVZ] = fl.mz + t0[3]; flxi[IEN] = fl.e + t0[4]; flxi[IBY] = fl.by + t0[5];
    flxi[IBZ] = fl.bz + t0[6];
  } else if (spd[2] >= T(0.0)) {
    dif(ulst, ul, spd[0], t0);
    dif(uldst, ulst, spd[1], t1);
    flxi[IDN] = fl.d + t0[0] + t1[0]; flxi[IVX] = fl.mx + t0[1] + t1[1];
    flxi[IVY] = fl.my + t0[2] + t1[2]; flxi[IVZ] = fl.mz + t0[3] + t1[3];
    flxi[IEN] = fl.e + t0[4] + t1[4]; flxi[IBY] = fl.by + t0[5] + t1[5];
    flxi[IBZ] = fl.bz + t0[6] + t1[6];
  } else if (spd[3] > T(0.0)) {
    dif(urst, ur, spd[4], t0);
    dif(urdst, urst, spd[3], t1);
    flxi[IDN] = fr.d + t0[0] + t1[0]; flxi[IVX] = fr.mx + t0[1] + t1[1];
    flxi[IVY] = fr.my + t0[2] + t1[2]; flxi[IVZ] = fr.mz + t0[3] + t1[3];
    flxi[IEN] = fr.e + t0[4] + t1[4]; flxi[IBY] = fr.by + t0[5] + t1[5];
    flxi[IBZ] = fr.bz + t0[6] + t1[6];
  } else {
    dif(urst, ur, spd[4], t0);
    flxi[IDN] = fr.d + t0[0]; flxi[IVX] = fr.mx + t0[1]; flxi[IVY] = fr.my + t0[2];
    flxi[IVZ] = fr.mz + t0[3]; flxi[IEN] = fr.e + t0[4]; flxi[IBY] = fr.by + t0[5];
    flxi[IBZ] = fr.bz + t0[6];
  }
}

// ---- HLLD on left/right lane pairs ------------------------------------------------------
// Most of HLLD is the same arithmetic on the left and right states, so hlld_lr carries the
// left state in one lane and the right one in the other of a pair type K::P and does the
// L/R-symmetric parts (the conserved states, fast speeds, outer fluxes, single- and
// double-star states, the final flux sums two components at a time) on both lanes at once.
// The few L-R mixed expressions (the contact speed, the double-star averages) and the
// divisions and square roots are per lane. Same formulas as rs_hlld above
// (hydro/rsolvers/mhd/hlld.cpp:56-371); the results agree to the arithmetic's rounding,
// not bit for bit, where a product and a sum are fused.
//
// PkF: FP32, on Blackwell's packed instructions (__fadd2_rn, __fmul2_rn, __ffma2_rn issue
// two FP32 operations per instruction, each lane rounded as the scalar operation). The
// double-float path (athg_df.cu) supplies its own K with pairs of double-float numbers.
struct PkF {
  using S = float;
  using P = float2;
  static __device__ __forceinline__ S sc(double v) { return (float)v; }
  static __device__ __forceinline__ P splat(S s) { return make_float2(s, s); }
  static __device__ __forceinline__ P pair(S l, S r) { return make_float2(l, r); }
  static __device__ __forceinline__ S L(P a) { return a.x; }
  static __device__ __forceinline__ S R(P a) { return a.y; }
  static __device__ __forceinline__ P add(P a, P b) { return __fadd2_rn(a, b); }
  static __device__ __forceinline__ P mul(P a, P b) { return __fmul2_rn(a, b); }
  static __device__ __forceinline__ P fma(P a, P b, P c) { return __ffma2_rn(a, b, c); }
  // a - b, rounded once (b times -1 is exact)
  static __device__ __forceinline__ P sub(P a, P b) { return __ffma2_rn(b, splat(-1.0f), a); }
  static __device__ __forceinline__ P div(P a, P b) { return make_float2(a.x / b.x, a.y / b.y); }
  static __device__ __forceinline__ P sqrt2(P a) { return make_float2(sqrtf(a.x), sqrtf(a.y)); }
  static __device__ __forceinline__ P sel(bool l, bool r, P a, P b) {
    return make_float2(l ? a.x : b.x, r ? a.y : b.y);
  }
  static __device__ __forceinline__ S abs(S a) { return fabsf(a); }
};

template <class K>
__device__ __forceinline__ void hlld_lr(const typename K::S* wli, const typename K::S* wri,
                                        typename K::S bxi, typename K::S gamma,
                                        typename K::S* flxi) {
  using S = typename K::S;
  using P = typename K::P;
  auto sp = [](S v) { return K::splat(v); };
  const S zero = K::sc(0.0), half = K::sc(0.5), one = K::sc(1.0);
  const S SMALLN = K::sc(1.0e-8);
  const S igm1 = one / (gamma - one);
  const S bxsq = bxi * bxi;
  const P d = K::pair(wli[IDN], wri[IDN]), vx = K::pair(wli[IVX], wri[IVX]),
          vy = K::pair(wli[IVY], wri[IVY]), vz = K::pair(wli[IVZ], wri[IVZ]),
          p = K::pair(wli[IPR], wri[IPR]), by = K::pair(wli[IBY], wri[IBY]),
          bz = K::pair(wli[IBZ], wri[IBZ]);
  // magnetic and kinetic energy densities, conserved states
  const P bt2 = K::fma(by, by, K::mul(bz, bz));
  const P pb = K::mul(sp(half), K::add(sp(bxsq), bt2));
  const P ke = K::mul(K::mul(sp(half), d), K::fma(vx, vx, K::fma(vy, vy, K::mul(vz, vz))));
  const P umx = K::mul(vx, d), umy = K::mul(vy, d), umz = K::mul(vz, d);
  const P ue = K::add(K::fma(p, sp(igm1), ke), pb);
  // fast magnetosonic speeds (fast_speed)
  const P asq = K::mul(sp(gamma), p);
  const P qsq = K::add(K::add(sp(bxsq), bt2), asq);
  const P tmq = K::sub(K::add(sp(bxsq), bt2), asq);
  const P disc = K::sqrt2(K::fma(tmq, tmq, K::mul(sp(K::sc(4.0)), K::mul(asq, bt2))));
  const P cf = K::sqrt2(K::div(K::mul(sp(half), K::add(qsq, disc)), d));
  const P vm = K::sub(vx, cf), vp = K::add(vx, cf);
  const S spd0 = mn(K::L(vm), K::R(vm)), spd4 = mx(K::L(vp), K::R(vp));
  const P pt = K::add(p, pb);
  // outer fluxes F(U_L), F(U_R)
  const P nbx = sp(-bxi);
  const P fmx = K::add(K::fma(umx, vx, pt), sp(-bxsq));
  const P fmy = K::fma(umy, vx, K::mul(nbx, by));
  const P fmz = K::fma(umz, vx, K::mul(nbx, bz));
  const P fe = K::fma(vx, K::add(K::add(ue, pt), sp(-bxsq)),
                      K::mul(nbx, K::fma(vy, by, K::mul(vz, bz))));
  const P fby = K::fma(by, vx, K::mul(nbx, vy));
  const P fbz = K::fma(bz, vx, K::mul(nbx, vz));
  // contact speed (L-R mixed: per lane)
  const P sd = K::sub(K::pair(spd0, spd4), vx);  // (sdl, sdr)
  const S spd2 = (K::R(sd) * K::R(umx) - K::L(sd) * K::L(umx) + (K::L(pt) - K::R(pt))) /
                 (K::R(sd) * K::R(d) - K::L(sd) * K::L(d));
  const P sdm = K::sub(K::pair(spd0, spd4), sp(spd2));
  const P sdm_inv = K::div(sp(one), sdm);
  // single-star states
  const P dsd = K::mul(d, sd);
  const P std_ = K::mul(dsd, sdm_inv);  // rho*
  const P std_inv = K::div(sp(one), std_);
  const P sqrtd = K::sqrt2(std_);
  const S abx = K::abs(bxi);
  const S spd1 = spd2 - abx / K::L(sqrtd);
  const S spd3 = spd2 + abx / K::R(sqrtd);
  const P ptstlr = K::fma(dsd, K::sub(sp(spd2), vx), pt);
  const S ptst = half * (K::R(ptstlr) + K::L(ptstlr));
  const P stmx = K::mul(std_, sp(spd2));
  const P den = K::add(K::mul(dsd, sdm), sp(-bxsq));
  const bool degl = K::abs(K::L(den)) < SMALLN * ptst, degr = K::abs(K::R(den)) < SMALLN * ptst;
  const P iden = K::div(sp(one), den);
  const P tmp1 = K::mul(K::mul(sp(bxi), K::sub(sd, sdm)), iden);
  const P tmp2 = K::mul(K::add(K::mul(dsd, sd), sp(-bxsq)), iden);
  const P stmy = K::sel(degl, degr, K::mul(std_, vy), K::mul(std_, K::sub(vy, K::mul(by, tmp1))));
  const P stmz = K::sel(degl, degr, K::mul(std_, vz), K::mul(std_, K::sub(vz, K::mul(bz, tmp1))));
  const P stby = K::sel(degl, degr, by, K::mul(by, tmp2));
  const P stbz = K::sel(degl, degr, bz, K::mul(bz, tmp2));
  const P vbst = K::mul(K::fma(stmx, sp(bxi), K::fma(stmy, stby, K::mul(stmz, stbz))), std_inv);
  const P vbu = K::fma(vy, by, K::mul(vz, bz));
  const P ste = K::mul(K::add(K::add(K::sub(K::mul(sd, ue), K::mul(pt, vx)), sp(ptst * spd2)),
                              K::mul(sp(bxi), K::sub(K::fma(vx, sp(bxi), vbu), vbst))),
                       sdm_inv);
  // double-star states (L-R averages: per lane where they mix)
  P dsmy = stmy, dsmz = stmz, dsby = stby, dsbz = stbz, dse = ste;
  if (!(half * bxsq < SMALLN * ptst)) {
    const S invsumd = one / (K::L(sqrtd) + K::R(sqrtd));
    const S bxsig = (bxi > zero ? one : -one);
    const P vyst = K::mul(stmy, std_inv), vzst = K::mul(stmz, std_inv);
    const S ty = invsumd * (K::L(sqrtd) * K::L(vyst) + K::R(sqrtd) * K::R(vyst) +
                            bxsig * (K::R(stby) - K::L(stby)));
    const S tz = invsumd * (K::L(sqrtd) * K::L(vzst) + K::R(sqrtd) * K::R(vzst) +
                            bxsig * (K::R(stbz) - K::L(stbz)));
    dsmy = K::mul(std_, sp(ty));
    dsmz = K::mul(std_, sp(tz));
    const S sq2 = bxsig * K::L(sqrtd) * K::R(sqrtd);
    const S tby = invsumd * (K::L(sqrtd) * K::R(stby) + K::R(sqrtd) * K::L(stby) +
                             sq2 * (K::R(vyst) - K::L(vyst)));
    const S tbz = invsumd * (K::L(sqrtd) * K::R(stbz) + K::R(sqrtd) * K::L(stbz) +
                             sq2 * (K::R(vzst) - K::L(vzst)));
    dsby = sp(tby);
    dsbz = sp(tbz);
    const S tv = spd2 * bxi + (K::L(dsmy) * tby + K::L(dsmz) * tbz) / K::L(std_);
    const P sgn = K::pair(-K::L(sqrtd) * bxsig, K::R(sqrtd) * bxsig);
    dse = K::fma(sgn, K::sub(vbst, sp(tv)), ste);
  }
  // the region of the fan that contains x/t = 0
  if (spd0 >= zero) {
    flxi[IDN] = K::L(umx); flxi[IVX] = K::L(fmx); flxi[IVY] = K::L(fmy); flxi[IVZ] = K::L(fmz);
    flxi[IEN] = K::L(fe); flxi[IBY] = K::L(fby); flxi[IBZ] = K::L(fbz);
    return;
  }
  if (spd4 <= zero) {
    flxi[IDN] = K::R(umx); flxi[IVX] = K::R(fmx); flxi[IVY] = K::R(fmy); flxi[IVZ] = K::R(fmz);
    flxi[IEN] = K::R(fe); flxi[IBY] = K::R(fby); flxi[IBZ] = K::R(fbz);
    return;
  }
  // one side's outer state U, star state U*, double-star state U**, outer flux F and the
  // wave speeds: F + s_o (U* - U) [+ s_i (U** - U*)], two components per operation
  const bool left = spd2 >= zero;
  const bool inner = left ? !(spd1 >= zero) : (spd3 > zero);
  const S so = left ? spd0 : spd4, si = left ? spd1 : spd3;
  auto pick = [&](P a) { return left ? K::L(a) : K::R(a); };
  const P u01 = K::pair(pick(d), pick(umx)), u23 = K::pair(pick(umy), pick(umz)),
          u45 = K::pair(pick(ue), pick(by)), u6 = K::pair(pick(bz), zero);
  const P s01 = K::pair(pick(std_), pick(stmx)), s23 = K::pair(pick(stmy), pick(stmz)),
          s45 = K::pair(pick(ste), pick(stby)), s6 = K::pair(pick(stbz), zero);
  const P f01 = K::pair(pick(umx), pick(fmx)), f23 = K::pair(pick(fmy), pick(fmz)),
          f45 = K::pair(pick(fe), pick(fby)), f6 = K::pair(pick(fbz), zero);
  P r01 = K::fma(sp(so), K::sub(s01, u01), f01), r23 = K::fma(sp(so), K::sub(s23, u23), f23),
    r45 = K::fma(sp(so), K::sub(s45, u45), f45), r6 = K::fma(sp(so), K::sub(s6, u6), f6);
  if (inner) {
    const P d01 = K::pair(pick(std_), pick(stmx)), d23 = K::pair(pick(dsmy), pick(dsmz)),
            d45 = K::pair(pick(dse), pick(dsby)), d6 = K::pair(pick(dsbz), zero);
    r01 = K::fma(sp(si), K::sub(d01, s01), r01);
    r23 = K::fma(sp(si), K::sub(d23, s23), r23);
    r45 = K::fma(sp(si), K::sub(d45, s45), r45);
    r6 = K::fma(sp(si), K::sub(d6, s6), r6);
  }
  flxi[IDN] = K::L(r01); flxi[IVX] = K::R(r01); flxi[IVY] = K::L(r23); flxi[IVZ] = K::R(r23);
  flxi[IEN] = K::L(r45); flxi[IBY] = K::R(r45); flxi[IBZ] = K::L(r6);
}

template <>
__device__ __forceinline__ void rs_hlld<float>(const float* wli, const float* wri, float bxi,
                                               float gamma, float* flxi) {
  hlld_lr<PkF>(wli, wri, bxi, gamma, flxi);
}

// LHLLC, the fork's low-dissipation HLLC (hydro/rsolvers/hydro/lhllc.cpp:26-180): PVRS
// wave speeds, the shock detector th = min(1, (cmax - min(dvn,0)) / (cmax - min(dvt,0)))^4
// on the pressure jump of the contact speed and the low-Mach factor phi = chi (2 - chi) on
// the contact pressure. dvn, dvt: Hydro::CalculateVelocityDifferences at the face.
template <typename T>
__device__ __forceinline__ void rs_lhllc(const T* wli, const T* wri, T gamma, T dvn,
                     T dvt, T* flxi) {
  T gm1 = gamma - T(1.0), igm1 = T(1.0) / gm1;
  T fl[5], fr[5];
  T cl = sqrt(gamma * wli[IPR] / wli[IDN]);
  T cr = sqrt(gamma * wri[IPR] / wri[IDN]);
  T vsql = sq(wli[IVX]) + sq(wli[IVY]) + sq(wli[IVZ]);
  T vsqr = sq(wri[IVX]) + sq(wri[IVY]) + sq(wri[IVZ]);
  T el = wli[IPR] * igm1 + T(0.5) * wli[IDN] * vsql;
  T er = wri[IPR] * igm1 + T(0.5) * wri[IDN] * vsqr;
  T rhoa = T(.5) * (wli[IDN] + wri[IDN]);
  T ca = T(.5) * (cl + cr);
  T pmid = T(.5) * (wli[IPR] + wri[IPR] + (wli[IVX] - wri[IVX]) * rhoa * ca);
  T umid = T(.5) * (wli[IVX] + wri[IVX] + (wli[IPR] - wri[IPR]) / (rhoa * ca));
  T rhol = wli[IDN] + (wli[IVX] - umid) * rhoa / ca;
  T rhor = wri[IDN] + (umid - wri[IVX]) * rhoa / ca;
  (void)rhol; (void)rhor;
  T ql = (pmid <= wli[IPR]) ? T(1.0)
              : sqrt(T(1.0) + (gamma + T(1)) / (T(2) * gamma) * (pmid / wli[IPR] - T(1.0)));
  T qr = (pmid <= wri[IPR]) ? T(1.0)
              : sqrt(T(1.0) + (gamma + T(1)) / (T(2) * gamma) * (pmid / wri[IPR] - T(1.0)));
  T al = wli[IVX] - cl * ql;
  T ar = wri[IVX] + cr * qr;
  T bp = ar > T(0.0) ? ar : T(1.0e-20);
  T bm = al < T(0.0) ? al : -T(1.0e-20);
  T vxl = al - wli[IVX], vxr = ar - wri[IVX];
  T ml = wli[IDN] * vxl, mr = wri[IDN] * vxr;
  T cmax = mx(cl, cr);
  T th1 = mn(T(1.0), (cmax - mn(dvn, T(0.0))) / (cmax - mn(dvt, T(0.0))));
  T th = th1 * th1 * th1 * th1;
  T am = (mr * wri[IVX] - ml * wli[IVX] - th * (wri[IPR] - wli[IPR])) / (mr - ml);
  T chi = mn(T(1.0), sqrt(mx(vsql, vsqr)) / cmax);
  T phi = chi * (T(2.0) - chi);
  T cp = (mr * wli[IPR] - ml * wri[IPR] + phi * mr * ml * (wri[IVX] - wli[IVX])) / (mr - ml);
  cp = cp > T(0.0) ? cp : T(0.0);
  T uxl = wli[IVX] - bm, uxr = wri[IVX] - bp;
  fl[IDN] = wli[IDN] * uxl; fr[IDN] = wri[IDN] * uxr;
  fl[IVX] = wli[IDN] * wli[IVX] * uxl + wli[IPR]; fr[IVX] = wri[IDN] * wri[IVX] * uxr + wri[IPR];
  fl[IVY] = wli[IDN] * wli[IVY] * uxl; fr[IVY] = wri[IDN] * wri[IVY] * uxr;
  fl[IVZ] = wli[IDN] * wli[IVZ] * uxl; fr[IVZ] = wri[IDN] * wri[IVZ] * uxr;
  fl[IEN] = el * uxl + wli[IPR] * wli[IVX]; fr[IEN] = er * uxr + wri[IPR] * wri[IVX];
  T sl, sr, sm;
  if (am >= T(0.0)) { sl = am / (am - bm); sr = T(0.0); sm = -bm / (am - bm); }
  else { sl = T(0.0); sr = -am / (bp - am); sm = bp / (bp - am); }
  flxi[IDN] = sl * fl[IDN] + sr * fr[IDN];
  flxi[IVX] = sl * fl[IVX] + sr * fr[IVX] + sm * cp;
  flxi[IVY] = sl * fl[IVY] + sr * fr[IVY];
  flxi[IVZ] = sl * fl[IVZ] + sr * fr[IVZ];
  flxi[IEN] = sl * fl[IEN] + sr * fr[IEN] + sm * cp * am;
}

// LHLLD, the fork's low-dissipation HLLD (hydro/rsolvers/mhd/lhlld.cpp:36-388): HLLD with
// the shock detector on the total-pressure jump of S_M and phi in the star total pressure.
template <typename T>
__device__ __forceinline__ void rs_lhlld(const T* wli, const T* wri, T bxi, T gamma,
                     T dvn, T dvt, T* flxi) {
  T igm1 = T(1.0) / (gamma - T(1.0));
  C1D<T> ul, ur, ulst, uldst, urdst, urst, fl, fr;
  T spd[5];
  T bxsq = bxi * bxi;
  T pbl = T(0.5) * (bxsq + (sq(wli[IBY]) + sq(wli[IBZ])));
  T pbr = T(0.5) * (bxsq + (sq(wri[IBY]) + sq(wri[IBZ])));
  T kel = T(0.5) * wli[IDN] * (sq(wli[IVX]) + (sq(wli[IVY]) + sq(wli[IVZ])));
  T ker = T(0.5) * wri[IDN] * (sq(wri[IVX]) + (sq(wri[IVY]) + sq(wri[IVZ])));
  ul.d = wli[IDN]; ul.mx = wli[IVX] * ul.d; ul.my = wli[IVY] * ul.d; ul.mz = wli[IVZ] * ul.d;
  ul.e = wli[IPR] * igm1 + kel + pbl; ul.by = wli[IBY]; ul.bz = wli[IBZ];
  ur.d = wri[IDN]; ur.mx = wri[IVX] * ur.d; ur.my = wri[IVY] * ur.d; ur.mz = wri[IVZ] * ur.d;
  ur.e = wri[IPR] * igm1 + ker + pbr; ur.by = wri[IBY]; ur.bz = wri[IBZ];
  T cfl = fast_speed(wli[IDN], wli[IPR], wli[IBY], wli[IBZ], bxi, gamma);
  T cfr = fast_speed(wri[IDN], wri[IPR], wri[IBY], wri[IBZ], bxi, gamma);
  spd[0] = mn(wli[IVX] - cfl, wri[IVX] - cfr);
  spd[4] = mx(wli[IVX] + cfl, wri[IVX] + cfr);
  T cfmax = mx(cfl, cfr);
  T ptl = wli[IPR] + pbl, ptr = wri[IPR] + pbr;
  fl.d = ul.mx;
  fl.mx = ul.mx * wli[IVX] + ptl - bxsq;
  fl.my = ul.my * wli[IVX] - bxi * ul.by;
  fl.mz = ul.mz * wli[IVX] - bxi * ul.bz;
  fl.e = wli[IVX] * (ul.e + ptl - bxsq) - bxi * (wli[IVY] * ul.by + wli[IVZ] * ul.bz);
  fl.by = ul.by * wli[IVX] - bxi * wli[IVY];
  fl.bz = ul.bz * wli[IVX] - bxi * wli[IVZ];
  fr.d = ur.mx;
  fr.mx = ur.mx * wri[IVX] + ptr - bxsq;
  fr.my = ur.my * wri[IVX] - bxi * ur.by;
  fr.mz = ur.mz * wri[IVX] - bxi * ur.bz;
  fr.e = wri[IVX] * (ur.e + ptr - bxsq) - bxi * (wri[IVY] * ur.by + wri[IVZ] * ur.bz);
  fr.by = ur.by * wri[IVX] - bxi * wri[IVY];
  fr.bz = ur.bz * wri[IVX] - bxi * wri[IVZ];
  T sdl = spd[0] - wli[IVX], sdr = spd[4] - wri[IVX];
  T sdld = sdl * ul.d, sdrd = sdr * ur.d;
  T th1 = mn(T(1.0), (cfmax - mn(dvn, T(0.0))) / (cfmax - mn(dvt, T(0.0))));
  T th = th1 * th1 * th1 * th1;
  spd[2] = (sdr * ur.mx - sdl * ul.mx + th * (ptl - ptr)) / (sdrd - sdld);
  T sdml = spd[0] - spd[2], sdmr = spd[4] - spd[2];
  T sdml_inv = T(1.0) / sdml, sdmr_inv = T(1.0) / sdmr;
  ulst.d = sdld * sdml_inv;
  urst.d = sdrd * sdmr_inv;
  T ulst_d_inv = T(1.0) / ulst.d, urst_d_inv = T(1.0) / urst.d;
  T sqrtdl = sqrt(ulst.d), sqrtdr = sqrt(urst.d);
  spd[1] = spd[2] - fabs(bxi) / sqrtdl;
  spd[3] = spd[2] + fabs(bxi) / sqrtdr;
  T clsq = ((pbl + kel) + sqrt(sq(pbl + kel) - T(2.0) * kel * bxsq)) / ul.d;
  T crsq = ((pbr + ker) + sqrt(sq(pbr + ker) - T(2.0) * ker * bxsq)) / ur.d;
  T chi = mn(T(1.0), sqrt(mx(clsq, crsq)) / cfmax);
  T phi = chi * (T(2.0) - chi);
  T ptst = (sdrd * ptl - sdld * ptr + phi * sdrd * sdld * (wri[IVX] - wli[IVX])) /
                (sdrd - sdld);
  ulst.mx = ulst.d * spd[2];
  if (fabs(sdld * sdml - bxsq) < T(1.0e-8) * ptst) {
    ulst.my = ulst.d * wli[IVY]; ulst.mz = ulst.d * wli[IVZ];
    ulst.by = ul.by; ulst.bz = ul.bz;
  } else {
    T tmp = bxi * (sdl - sdml) / (sdld * sdml - bxsq);
    ulst.my = ulst.d * (wli[IVY] - ul.by * tmp);
    ulst.mz = ulst.d * (wli[IVZ] - ul.bz * tmp);
    tmp = (sdld * sdl - bxsq) / (sdld * sdml - bxsq);
    ulst.by = ul.by * tmp; ulst.bz = ul.bz * tmp;
  }
  T vbstl = (ulst.mx * bxi + (ulst.my * ulst.by + ulst.mz * ulst.bz)) * ulst_d_inv;
  ulst.e = (sdl * ul.e - ptl * wli[IVX] + ptst * spd[2] +
            bxi * (wli[IVX] * bxi + (wli[IVY] * ul.by + wli[IVZ] * ul.bz) - vbstl)) * sdml_inv;
  urst.mx = urst.d * spd[2];
  if (fabs(sdrd * sdmr - bxsq) < T(1.0e-8) * ptst) {
    urst.my = urst.d * wri[IVY]; urst.mz = urst.d * wri[IVZ];
    urst.by = ur.by; urst.bz = ur.bz;
  } else {
    T tmp = bxi * (sdr - sdmr) / (sdrd * sdmr - bxsq);
    urst.my = urst.d * (wri[IVY] - ur.by * tmp);
    urst.mz = urst.d * (wri[IVZ] - ur.bz * tmp);
    tmp = (sdrd * sdr - bxsq) / (sdrd * sdmr - bxsq);
    urst.by = ur.by * tmp; urst.bz = ur.bz * tmp;
  }
  T vbstr = (urst.mx * bxi + (urst.my * urst.by + urst.mz * urst.bz)) * urst_d_inv;
  urst.e = (sdr * ur.e - ptr * wri[IVX] + ptst * spd[2] +
            bxi * (wri[IVX] * bxi + (wri[IVY] * ur.by + wri[IVZ] * ur.bz) - vbstr)) * sdmr_inv;
  if (T(0.5) * bxsq < T(1.0e-8) * ptst) {
    uldst = ulst; urdst = urst;
  } else {
    T invsumd = T(1.0) / (sqrtdl + sqrtdr);
    T bxsig = (bxi > T(0.0) ? T(1.0) : -T(1.0));
    uldst.d = ulst.d; urdst.d = urst.d;
    uldst.mx = ulst.mx; urdst.mx = urst.mx;
    T tmp = invsumd * (sqrtdl * (ulst.my * ulst_d_inv) + sqrtdr * (urst.my * urst_d_inv) +
                            bxsig * (urst.by - ulst.by));
    uldst.my = uldst.d * tmp; urdst.my = urdst.d * tmp;
    tmp = invsumd * (sqrtdl * (ulst.mz * ulst_d_inv) + sqrtdr * (urst.mz * urst_d_inv) +
                     bxsig * (urst.bz - ulst.bz));
    uldst.mz = uldst.d * tmp; urdst.mz = urdst.d * tmp;
    tmp = invsumd * (sqrtdl * urst.by + sqrtdr * ulst.by +
                     bxsig * sqrtdl * sqrtdr * ((urst.my * urst_d_inv) - (ulst.my * ulst_d_inv)));
    uldst.by = urdst.by = tmp;
    tmp = invsumd * (sqrtdl * urst.bz + sqrtdr * ulst.bz +
                     bxsig * sqrtdl * sqrtdr * ((urst.mz * urst_d_inv) - (ulst.mz * ulst_d_inv)));
    uldst.bz = urdst.bz = tmp;
    tmp = spd[2] * bxi + (uldst.my * uldst.by + uldst.mz * uldst.bz) / uldst.d;
    uldst.e = ulst.e - sqrtdl * bxsig * (vbstl - tmp);
    urdst.e = urst.e + sqrtdr * bxsig * (vbstr - tmp);
  }
#define DIFFW(dst, a, b, sp) \
  dst.d = sp * (a.d - b.d); dst.mx = sp * (a.mx - b.mx); dst.my = sp * (a.my - b.my); \
  dst.mz = sp * (a.mz - b.mz); dst.e = sp * (a.e - b.e); dst.by = sp * (a.by - b.by); \
  dst.bz = sp * (a.bz - b.bz);
  C1D<T> t1, t0, t3, t4;
  DIFFW(t1, uldst, ulst, spd[1]);
  DIFFW(t0, ulst, ul, spd[0]);
  DIFFW(t3, urdst, urst, spd[3]);
  DIFFW(t4, urst, ur, spd[4]);
#undef DIFFW
  if (spd[0] >= T(0.0)) {
    flxi[IDN] = fl.d; flxi[IVX] = fl.mx; flxi[IVY] = fl.my; flxi[IVZ] = fl.mz;
    flxi[IEN] = fl.e; flxi[IBY] = fl.by; flxi[IBZ] = fl.bz;
  } else if (spd[4] <= T(0.0)) {
    flxi[IDN] = fr.d; flxi[IVX] = fr.mx; flxi[IVY] = fr.my; flxi[IVZ] = fr.mz;
    flxi[IEN] = fr.e; flxi[IBY] = fr.by; flxi[IBZ] = fr.bz;
  } else if (spd[1] >= T(0.0)) {
    flxi[IDN] = fl.d + t0.d; flxi[IVX] = fl.mx + t0.mx; flxi[IVY] = fl.my + t0.my;
    flxi[IVZ] = fl.mz + t0.mz; flxi[IEN] = fl.e + t0.e; flxi[IBY] = fl.by + t0.by;
    flxi[IBZ] = fl.bz + t0.bz;
  } else if (spd[2] >= T(0.0)) {
    flxi[IDN] = fl.d + t0.d + t1.d; flxi[IVX] = fl.mx + t0.mx + t1.mx;
    flxi[IVY] = fl.my + t0.my + t1.my; flxi[IVZ] = fl.mz + t0.mz + t1.mz;
    flxi[IEN] = fl.e + t0.e + t1.e; flxi[IBY] = fl.by + t0.by + t1.by;
    flxi[IBZ] = fl.bz + t0.bz + t1.bz;
  } else if (spd[3] > T(0.0)) {
    flxi[IDN] = fr.d + t4.d + t3.d; flxi[IVX] = fr.mx + t4.mx + t3.mx;
    flxi[IVY] = fr.my + t4.my + t3.my; flxi[IVZ] = fr.mz + t4.mz + t3.mz;
    flxi[IEN] = fr.e + t4.e + t3.e; flxi[IBY] = fr.by + t4.by + t3.by;
    flxi[IBZ] = fr.bz + t4.bz + t3.bz;
  } else {
    flxi[IDN] = fr.d + t4.d; flxi[IVX] = fr.mx + t4.mx; flxi[IVY] = fr.my + t4.my;
    flxi[IVZ] = fr.mz + t4.mz; flxi[IEN] = fr.e + t4.e; flxi[IBY] = fr.by + t4.by;
    flxi[IBZ] = fr.bz + t4.bz;
  }
}

}  // namespace athg

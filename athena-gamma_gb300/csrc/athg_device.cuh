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

// ---- HLLD for the FP32 flux path on packed FP32 instructions ---------------------------
// Blackwell issues two FP32 additions, multiplications or FMAs per instruction on float2
// operands (__fadd2_rn, __fmul2_rn, __ffma2_rn; each lane rounds as the scalar operation
// does). Most of HLLD is the same arithmetic on the left and right states, so here lane x
// carries the left state and lane y the right one, and the L/R-symmetric parts (the
// conserved states, fast speeds, outer fluxes, single- and double-star states) take half
// the issue slots. Divisions and square roots stay scalar; the few L-R mixed expressions
// (the contact speed, the double-star averages) are scalar too. Same formulas as rs_hlld
// above (hydro/rsolvers/mhd/hlld.cpp:56-371); the results agree to FP32 rounding (the FP32
// flux path's tolerance), not bit for bit, because products that the scalar code rounds
// separately may be fused here.
namespace pk {
__device__ __forceinline__ float2 S(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 P(float l, float r) { return make_float2(l, r); }
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
// a - b, rounded once (b times -1 is exact)
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return __ffma2_rn(b, S(-1.0f), a); }
__device__ __forceinline__ float2 rcp(float2 a) { return make_float2(1.0f / a.x, 1.0f / a.y); }
__device__ __forceinline__ float2 sqrt2(float2 a) { return make_float2(sqrtf(a.x), sqrtf(a.y)); }
__device__ __forceinline__ float2 sel(bool l, bool r, float2 a, float2 b) {
  return make_float2(l ? a.x : b.x, r ? a.y : b.y);
}
}  // namespace pk

template <>
__device__ __forceinline__ void rs_hlld<float>(const float* wli, const float* wri, float bxi,
                                               float gamma, float* flxi) {
  using namespace pk;
  const float SMALLN = 1.0e-8f;
  const float igm1 = 1.0f / (gamma - 1.0f);
  const float bxsq = bxi * bxi;
  const float2 d = P(wli[IDN], wri[IDN]), vx = P(wli[IVX], wri[IVX]),
               vy = P(wli[IVY], wri[IVY]), vz = P(wli[IVZ], wri[IVZ]),
               p = P(wli[IPR], wri[IPR]), by = P(wli[IBY], wri[IBY]), bz = P(wli[IBZ], wri[IBZ]);
  // magnetic and kinetic energy densities, conserved states
  const float2 bt2 = fma(by, by, mul(bz, bz));
  const float2 pb = mul(S(0.5f), add(S(bxsq), bt2));
  const float2 ke = mul(mul(S(0.5f), d), fma(vx, vx, fma(vy, vy, mul(vz, vz))));
  const float2 umx = mul(vx, d), umy = mul(vy, d), umz = mul(vz, d);
  const float2 ue = add(fma(p, S(igm1), ke), pb);
  // fast magnetosonic speeds (fast_speed)
  const float2 asq = mul(S(gamma), p);
  const float2 qsq = add(add(S(bxsq), bt2), asq);
  const float2 tmq = sub(add(S(bxsq), bt2), asq);
  const float2 disc = sqrt2(fma(tmq, tmq, mul(S(4.0f), mul(asq, bt2))));
  const float2 cf2 = mul(S(0.5f), add(qsq, disc));
  const float2 cf = sqrt2(P(cf2.x / d.x, cf2.y / d.y));
  const float2 vm = sub(vx, cf), vp = add(vx, cf);
  const float spd0 = mn(vm.x, vm.y), spd4 = mx(vp.x, vp.y);
  const float2 pt = add(p, pb);
  // outer fluxes F(U_L), F(U_R)
  const float2 nbx = S(-bxi);
  const float2 fmx = add(fma(umx, vx, pt), S(-bxsq));
  const float2 fmy = fma(umy, vx, mul(nbx, by));
  const float2 fmz = fma(umz, vx, mul(nbx, bz));
  const float2 fe = fma(vx, add(add(ue, pt), S(-bxsq)), mul(nbx, fma(vy, by, mul(vz, bz))));
  const float2 fby = fma(by, vx, mul(nbx, vy));
  const float2 fbz = fma(bz, vx, mul(nbx, vz));
  // contact speed (L-R mixed: scalar)
  const float2 sd = sub(P(spd0, spd4), vx);  // (sdl, sdr)
  const float spd2 = (sd.y * umx.y - sd.x * umx.x + (pt.x - pt.y)) / (sd.y * d.y - sd.x * d.x);
  const float2 sdm = sub(P(spd0, spd4), S(spd2));
  const float2 sdm_inv = rcp(sdm);
  // single-star states
  const float2 dsd = mul(d, sd);
  const float2 std_ = mul(dsd, sdm_inv);  // rho*
  const float2 std_inv = rcp(std_);
  const float2 sqrtd = sqrt2(std_);
  const float abx = fabsf(bxi);
  const float spd1 = spd2 - abx / sqrtd.x;
  const float spd3 = spd2 + abx / sqrtd.y;
  const float2 ptstlr = fma(dsd, sub(S(spd2), vx), pt);
  const float ptst = 0.5f * (ptstlr.y + ptstlr.x);
  const float2 stmx = mul(std_, S(spd2));
  const float2 den = add(mul(dsd, sdm), S(-bxsq));
  const bool degl = fabsf(den.x) < SMALLN * ptst, degr = fabsf(den.y) < SMALLN * ptst;
  const float2 iden = rcp(den);
  const float2 tmp1 = mul(mul(S(bxi), sub(sd, sdm)), iden);
  const float2 tmp2 = mul(add(mul(dsd, sd), S(-bxsq)), iden);
  const float2 stmy = sel(degl, degr, mul(std_, vy), mul(std_, sub(vy, mul(by, tmp1))));
  const float2 stmz = sel(degl, degr, mul(std_, vz), mul(std_, sub(vz, mul(bz, tmp1))));
  const float2 stby = sel(degl, degr, by, mul(by, tmp2));
  const float2 stbz = sel(degl, degr, bz, mul(bz, tmp2));
  const float2 vbst = mul(fma(stmx, S(bxi), fma(stmy, stby, mul(stmz, stbz))), std_inv);
  const float2 vbu = fma(vy, by, mul(vz, bz));
  const float2 ste = mul(add(add(sub(mul(sd, ue), mul(pt, vx)), S(ptst * spd2)),
                             mul(S(bxi), sub(fma(vx, S(bxi), vbu), vbst))),
                         sdm_inv);
  // double-star states (L-R averages: scalar where they mix)
  float2 dsmy = stmy, dsmz = stmz, dsby = stby, dsbz = stbz, dse = ste;
  if (!(0.5f * bxsq < SMALLN * ptst)) {
    const float invsumd = 1.0f / (sqrtd.x + sqrtd.y);
    const float bxsig = (bxi > 0.0f ? 1.0f : -1.0f);
    const float2 vyst = mul(stmy, std_inv), vzst = mul(stmz, std_inv);
    const float ty = invsumd * (sqrtd.x * vyst.x + sqrtd.y * vyst.y + bxsig * (stby.y - stby.x));
    const float tz = invsumd * (sqrtd.x * vzst.x + sqrtd.y * vzst.y + bxsig * (stbz.y - stbz.x));
    dsmy = mul(std_, S(ty));
    dsmz = mul(std_, S(tz));
    const float sq2 = bxsig * sqrtd.x * sqrtd.y;
    const float tby = invsumd * (sqrtd.x * stby.y + sqrtd.y * stby.x + sq2 * (vyst.y - vyst.x));
    const float tbz = invsumd * (sqrtd.x * stbz.y + sqrtd.y * stbz.x + sq2 * (vzst.y - vzst.x));
    dsby = S(tby);
    dsbz = S(tbz);
    const float tv = spd2 * bxi + (dsmy.x * tby + dsmz.x * tbz) / std_.x;
    const float2 sgn = P(-sqrtd.x * bxsig, sqrtd.y * bxsig);
    dse = fma(sgn, sub(vbst, S(tv)), ste);
  }
  // the region of the fan that contains x/t = 0
  const bool left = spd2 >= 0.0f;
  auto L = [](float2 a) { return a.x; };
  auto R = [](float2 a) { return a.y; };
  if (spd0 >= 0.0f) {
    flxi[IDN] = umx.x; flxi[IVX] = fmx.x; flxi[IVY] = fmy.x; flxi[IVZ] = fmz.x;
    flxi[IEN] = fe.x; flxi[IBY] = fby.x; flxi[IBZ] = fbz.x;
    return;
  }
  if (spd4 <= 0.0f) {
    flxi[IDN] = umx.y; flxi[IVX] = fmx.y; flxi[IVY] = fmy.y; flxi[IVZ] = fmz.y;
    flxi[IEN] = fe.y; flxi[IBY] = fby.y; flxi[IBZ] = fbz.y;
    return;
  }
  // one side's outer state U, star state U*, double-star state U**, outer flux F and the
  // wave speeds: F + s_o (U* - U) [+ s_i (U** - U*)], two components per instruction
  const bool inner = left ? !(spd1 >= 0.0f) : (spd3 > 0.0f);
  const float so = left ? spd0 : spd4, si = left ? spd1 : spd3;
  auto pick = [&](float2 a) { return left ? L(a) : R(a); };
  const float2 u01 = P(pick(d), pick(umx)), u23 = P(pick(umy), pick(umz)),
               u45 = P(pick(ue), pick(by)), u6 = P(pick(bz), 0.0f);
  const float2 s01 = P(pick(std_), pick(stmx)), s23 = P(pick(stmy), pick(stmz)),
               s45 = P(pick(ste), pick(stby)), s6 = P(pick(stbz), 0.0f);
  const float2 f01 = P(pick(umx), pick(fmx)), f23 = P(pick(fmy), pick(fmz)),
               f45 = P(pick(fe), pick(fby)), f6 = P(pick(fbz), 0.0f);
  float2 r01 = fma(S(so), sub(s01, u01), f01), r23 = fma(S(so), sub(s23, u23), f23),
         r45 = fma(S(so), sub(s45, u45), f45), r6 = fma(S(so), sub(s6, u6), f6);
  if (inner) {
    const float2 d01 = P(pick(std_), pick(stmx)), d23 = P(pick(dsmy), pick(dsmz)),
                 d45 = P(pick(dse), pick(dsby)), d6 = P(pick(dsbz), 0.0f);
    r01 = fma(S(si), sub(d01, s01), r01);
    r23 = fma(S(si), sub(d23, s23), r23);
    r45 = fma(S(si), sub(d45, s45), r45);
    r6 = fma(S(si), sub(d6, s6), r6);
  }
  flxi[IDN] = r01.x; flxi[IVX] = r01.y; flxi[IVY] = r23.x; flxi[IVZ] = r23.y;
  flxi[IEN] = r45.x; flxi[IBY] = r45.y; flxi[IBZ] = r6.x;
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

// athg_stage.cuh -- per-stage kernels of the finite-volume (M)HD update, templated on
// the arithmetic type T of primitives/fluxes (double: plain FP64 path, float: mixed
// path). Conserved variables, face fields and the CT update are FP64 in both paths.
//
// Each launch covers every MeshBlock of the pool (grid.z runs over k and blocks).
#pragma once
#include "athg_device.cuh"

namespace athg {

// Pointers of the block pool handed to the stage kernels.
template <typename T>
struct StagePtrs {
  double *u, *u1;            // conserved registers [nb][5][cells]
  double *b1, *b2, *b3;      // face field          [nb][faces]
  double *r1, *r2, *r3;      // face-field register
  T *w, *bcc;                // primitives [nb][5][cells], cell-centred B [nb][3][cells]
  T *flx[3];                 // per direction [nb][NF][faces]; NF = 5 (hydro) or 8 (MHD:
                             // 5 fluxes, ey, ez, CT weight)
  double *edge;              // corner EMFs [nb][3][edges]
  const BlockGeo *geo;       // [nb]
  const double *coef;        // PLM interface coefficients [nb][3][2][ncmax]
  const double *dt;          // current time step (device scalar)
};

// Index box of one launch: every (i,j) of the box is flattened onto grid.x (so ranges
// like is..ie+1 do not leave idle half-warps), grid.y runs over k, grid.z over blocks.
struct Box {
  int il, jl, kl, ni, nj, nk;
};
__device__ __forceinline__ bool box_coords(const Box& bx, int& i, int& j, int& k, int& b) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= bx.ni * bx.nj) return false;
  int jj = t / bx.ni;
  i = bx.il + (t - jj * bx.ni);
  j = bx.jl + jj;
  k = bx.kl + blockIdx.y;
  b = blockIdx.z;
  return true;
}

// Wave variable n of cell c for a sweep along DIR (transverse B in the cyclic order of
// reference src/reconstruct/plm.cpp:44-55 (x1), :156-170 (x2), :268-282 (x3)).
template <typename T, int DIR>
__device__ __forceinline__ T wave_var(const T* __restrict__ w, const T* __restrict__ bcc,
                                      int64_t nc, int n, int64_t c) {
  if (n < NHYD) return w[n * nc + c];
  constexpr int by = DIR == 0 ? 1 : (DIR == 1 ? 2 : 0);
  constexpr int bz = DIR == 0 ? 2 : (DIR == 1 ? 0 : 1);
  return bcc[(n == IBY ? by : bz) * nc + c];
}

// Face-flux kernel: one thread per face. Reconstruction (donor cell or van Leer PLM,
// reference src/reconstruct/dc.cpp, src/reconstruct/plm.cpp uniform branch) fused with
// the Riemann solve. Face (k,j,i) along DIR separates cell index-1 from cell index.
// Loop extents per direction follow src/hydro/calculate_fluxes.cpp:63-74,164-172,274-279.
template <typename T, int DIR, int ORDER, int SOLVER, bool MHD>
__global__ void __launch_bounds__(128)
k_flux(Geom g, StagePtrs<T> p, Box bx, Phys ph) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  constexpr int NW = MHD ? 7 : 5;
  constexpr int NF = MHD ? 8 : 5;
  const int64_t nc = g.ncell;
  const T* __restrict__ w = p.w + (int64_t)b * NHYD * nc;
  const T* __restrict__ bcc = MHD ? p.bcc + (int64_t)b * 3 * nc : nullptr;
  const int64_t st = DIR == 0 ? 1 : (DIR == 1 ? (int64_t)g.nc1 : (int64_t)g.nc1 * g.nc2);
  const int64_t c = cidx(g, k, j, i);   // cell on the right of the face
  const int f = DIR == 0 ? i : (DIR == 1 ? j : k);
  T wl[7], wr[7];
  if (ORDER == 1) {
#pragma unroll
    for (int n = 0; n < NW; ++n) {
      wl[n] = wave_var<T, DIR>(w, bcc, nc, n, c - st);
      wr[n] = wave_var<T, DIR>(w, bcc, nc, n, c);
    }
  } else {
    const double* cf = p.coef + ((int64_t)b * 3 + DIR) * 2 * g.ncmax;
    const T cpL = (T)cf[f - 1];              // (x_f(c+1) - x_v(c)) / dx  for c = f-1
    const T cmR = (T)cf[g.ncmax + f];        // (x_v(c) - x_f(c)) / dx    for c = f
#pragma unroll
    for (int n = 0; n < NW; ++n) {
      T a0 = wave_var<T, DIR>(w, bcc, nc, n, c - 2 * st);
      T a1 = wave_var<T, DIR>(w, bcc, nc, n, c - st);
      T a2 = wave_var<T, DIR>(w, bcc, nc, n, c);
      T a3 = wave_var<T, DIR>(w, bcc, nc, n, c + st);
      T dwl = (a1 - a0), dwr = (a2 - a1);
      T dw2 = dwl * dwr;
      T dwm = T(2.0) * dw2 / (dwl + dwr);
      if (dw2 <= T(0.0)) dwm = T(0.0);
      wl[n] = a1 + cpL * dwm;
      dwl = (a2 - a1); dwr = (a3 - a2);
      dw2 = dwl * dwr;
      dwm = T(2.0) * dw2 / (dwl + dwr);
      if (dw2 <= T(0.0)) dwm = T(0.0);
      wr[n] = a2 - cmR * dwm;
    }
  }
  constexpr int ivx = IVX + DIR, ivy = IVX + (DIR + 1) % 3, ivz = IVX + (DIR + 2) % 3;
  T wli[7], wri[7], fx[7];
  wli[IDN] = wl[IDN]; wli[IVX] = wl[ivx]; wli[IVY] = wl[ivy]; wli[IVZ] = wl[ivz];
  wli[IPR] = wl[IPR];
  wri[IDN] = wr[IDN]; wri[IVX] = wr[ivx]; wri[IVY] = wr[ivy]; wri[IVZ] = wr[ivz];
  wri[IPR] = wr[IPR];
  const int64_t nf = fsize<DIR>(g);
  const int64_t fi = fidx<DIR>(g, k, j, i);
  T* __restrict__ out = p.flx[DIR] + (int64_t)b * NF * nf;
  const T gam = (T)ph.gamma;
  if constexpr (MHD) {
    wli[IBY] = wl[IBY]; wli[IBZ] = wl[IBZ];
    wri[IBY] = wr[IBY]; wri[IBZ] = wr[IBZ];
    const double* bn = DIR == 0 ? p.b1 + (int64_t)b * g.nf1
                                : (DIR == 1 ? p.b2 + (int64_t)b * g.nf2 : p.b3 + (int64_t)b * g.nf3);
    const T bxi = (T)bn[fi];
    if (SOLVER == HLLD) rs_hlld<T>(wli, wri, bxi, gam, fx);
    else rs_hlle_mhd<T>(wli, wri, bxi, gam, fx);
    out[5 * nf + fi] = -fx[IBY];
    out[6 * nf + fi] = fx[IBZ];
    out[7 * nf + fi] = ct_weight<T>(fx[IDN], wli[IDN], wri[IDN], (T)p.geo[b].dx[DIR], (T)(*p.dt));
  } else {
    if (SOLVER == HLLC) rs_hllc<T>(wli, wri, gam, fx);
    else rs_hlle_hydro<T>(wli, wri, gam, fx);
  }
  out[IDN * nf + fi] = fx[IDN];
  out[ivx * nf + fi] = fx[IVX];
  out[ivy * nf + fi] = fx[IVY];
  out[ivz * nf + fi] = fx[IVZ];
  out[IEN * nf + fi] = fx[IEN];
}

// Corner EMFs (Gardiner & Stone upwind integration), one thread per corner location
// (k,j,i) in [ks,ke+1]x[js,je+1]x[is,ie+1] computing e1, e2, e3 there.
// Reference src/field/calculate_corner_e.cpp:129-229 (3-D, Newtonian). The cell-centred
// E = -v x B is recomputed from W and bcc where needed instead of being stored.
template <typename T>
__global__ void __launch_bounds__(128) k_corner_emf(Geom g, StagePtrs<T> p, Box bx) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  const int64_t nc = g.ncell;
  const T* w = p.w + (int64_t)b * NHYD * nc;
  const T* bc = p.bcc + (int64_t)b * 3 * nc;
  auto cce = [&](int n, int kk, int jj, int ii) -> T {
    int64_t c = cidx(g, kk, jj, ii);
    T vx = w[IVX * nc + c], vy = w[IVY * nc + c], vz = w[IVZ * nc + c];
    T bx1 = bc[c], by1 = bc[nc + c], bz1 = bc[2 * nc + c];
    if (n == 0) return vz * by1 - vy * bz1;
    if (n == 1) return vx * bz1 - vz * bx1;
    return vy * bx1 - vx * by1;
  };
  const int64_t n1 = g.nf1, n2 = g.nf2, n3 = g.nf3;
  const T* F1 = p.flx[0] + (int64_t)b * 8 * n1;
  const T* F2 = p.flx[1] + (int64_t)b * 8 * n2;
  const T* F3 = p.flx[2] + (int64_t)b * 8 * n3;
  // face EMFs: x1 faces carry (e3, e2), x2 faces (e1, e3), x3 faces (e2, e1)
  auto e3x1 = [&](int kk, int jj, int ii) { return F1[5 * n1 + f1idx(g, kk, jj, ii)]; };
  auto e2x1 = [&](int kk, int jj, int ii) { return F1[6 * n1 + f1idx(g, kk, jj, ii)]; };
  auto wx1 = [&](int kk, int jj, int ii) { return F1[7 * n1 + f1idx(g, kk, jj, ii)]; };
  auto e1x2 = [&](int kk, int jj, int ii) { return F2[5 * n2 + f2idx(g, kk, jj, ii)]; };
  auto e3x2 = [&](int kk, int jj, int ii) { return F2[6 * n2 + f2idx(g, kk, jj, ii)]; };
  auto wx2 = [&](int kk, int jj, int ii) { return F2[7 * n2 + f2idx(g, kk, jj, ii)]; };
  auto e2x3 = [&](int kk, int jj, int ii) { return F3[5 * n3 + f3idx(g, kk, jj, ii)]; };
  auto e1x3 = [&](int kk, int jj, int ii) { return F3[6 * n3 + f3idx(g, kk, jj, ii)]; };
  auto wx3 = [&](int kk, int jj, int ii) { return F3[7 * n3 + f3idx(g, kk, jj, ii)]; };
  const T one = T(1.0), q = T(0.25);
  double* E = p.edge + (int64_t)b * 3 * g.ne;
  const int64_t ei = eidx(g, k, j, i);
  {
    T de1_l3 = (one - wx2(k - 1, j, i)) * (e1x3(k, j, i) - cce(0, k - 1, j, i)) +
               (wx2(k - 1, j, i)) * (e1x3(k, j - 1, i) - cce(0, k - 1, j - 1, i));
    T de1_r3 = (one - wx2(k, j, i)) * (e1x3(k, j, i) - cce(0, k, j, i)) +
               (wx2(k, j, i)) * (e1x3(k, j - 1, i) - cce(0, k, j - 1, i));
    T de1_l2 = (one - wx3(k, j - 1, i)) * (e1x2(k, j, i) - cce(0, k, j - 1, i)) +
               (wx3(k, j - 1, i)) * (e1x2(k - 1, j, i) - cce(0, k - 1, j - 1, i));
    T de1_r2 = (one - wx3(k, j, i)) * (e1x2(k, j, i) - cce(0, k, j, i)) +
               (wx3(k, j, i)) * (e1x2(k - 1, j, i) - cce(0, k - 1, j, i));
    E[ei] = (double)(q * (de1_l3 + de1_r3 + de1_l2 + de1_r2 + e1x2(k - 1, j, i) +
                          e1x2(k, j, i) + e1x3(k, j - 1, i) + e1x3(k, j, i)));
  }
  {
    T de2_l3 = (one - wx1(k - 1, j, i)) * (e2x3(k, j, i) - cce(1, k - 1, j, i)) +
               (wx1(k - 1, j, i)) * (e2x3(k, j, i - 1) - cce(1, k - 1, j, i - 1));
    T de2_r3 = (one - wx1(k, j, i)) * (e2x3(k, j, i) - cce(1, k, j, i)) +
               (wx1(k, j, i)) * (e2x3(k, j, i - 1) - cce(1, k, j, i - 1));
    T de2_l1 = (one - wx3(k, j, i - 1)) * (e2x1(k, j, i) - cce(1, k, j, i - 1)) +
               (wx3(k, j, i - 1)) * (e2x1(k - 1, j, i) - cce(1, k - 1, j, i - 1));
    T de2_r1 = (one - wx3(k, j, i)) * (e2x1(k, j, i) - cce(1, k, j, i)) +
               (wx3(k, j, i)) * (e2x1(k - 1, j, i) - cce(1, k - 1, j, i));
    E[g.ne + ei] = (double)(q * (de2_l3 + de2_r3 + de2_l1 + de2_r1 + e2x3(k, j, i - 1) +
                                 e2x3(k, j, i) + e2x1(k - 1, j, i) + e2x1(k, j, i)));
  }
  {
    T de3_l2 = (one - wx1(k, j - 1, i)) * (e3x2(k, j, i) - cce(2, k, j - 1, i)) +
               (wx1(k, j - 1, i)) * (e3x2(k, j, i - 1) - cce(2, k, j - 1, i - 1));
    T de3_r2 = (one - wx1(k, j, i)) * (e3x2(k, j, i) - cce(2, k, j, i)) +
               (wx1(k, j, i)) * (e3x2(k, j, i - 1) - cce(2, k, j, i - 1));
    T de3_l1 = (one - wx2(k, j, i - 1)) * (e3x1(k, j, i) - cce(2, k, j, i - 1)) +
               (wx2(k, j, i - 1)) * (e3x1(k, j - 1, i) - cce(2, k, j - 1, i - 1));
    T de3_r1 = (one - wx2(k, j, i)) * (e3x1(k, j, i) - cce(2, k, j, i)) +
               (wx2(k, j, i)) * (e3x1(k, j - 1, i) - cce(2, k, j - 1, i));
    E[2 * g.ne + ei] = (double)(q * (de3_l1 + de3_r1 + de3_l2 + de3_r2 + e3x2(k, j, i - 1) +
                                     e3x2(k, j, i) + e3x1(k, j - 1, i) + e3x1(k, j, i)));
  }
}

// Register averaging + flux divergence + CT, fused. One thread per location
// (k,j,i) in [ks,ke+1]x[js,je+1]x[is,ie+1]: the cell (if interior) and the three faces
// whose lower corner is (k,j,i) (if owned). FP64 throughout; fluxes are widened from T.
//   u1 <- u1 + delta*u                    (mesh/weighted_ave.cpp, wght[0]==1 branch)
//   u  <- swap ? u1 : g1*u + g2*u1        (time_integrator.cpp:1580-1584)
//   u  <- u - beta*dt*div(F)/vol          (hydro/add_flux_divergence.cpp:53-92)
//   b  likewise, then b -= beta*dt*curl(E) (field/ct.cpp:38-113)
// The registers keep fixed roles (no pointer swap): with swap set, the averaged value
// u1 is written into u, which is what the reference's swap leaves in u.
template <typename T, bool MHD>
__global__ void __launch_bounds__(128) k_update(Geom g, StagePtrs<T> p, Box bx, StageW sw) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  const double wght = sw.beta * (*p.dt);
  const BlockGeo geo = p.geo[b];
  const double dx1 = geo.dx[0], dx2 = geo.dx[1], dx3 = geo.dx[2];
  if (i <= g.ie && j <= g.je && k <= g.ke) {
    const int64_t nc = g.ncell;
    double* u = p.u + (int64_t)b * NHYD * nc;
    double* u1 = p.u1 + (int64_t)b * NHYD * nc;
    constexpr int NF = MHD ? 8 : 5;
    const T* F1 = p.flx[0] + (int64_t)b * NF * g.nf1;
    const T* F2 = p.flx[1] + (int64_t)b * NF * g.nf2;
    const T* F3 = p.flx[2] + (int64_t)b * NF * g.nf3;
    const double a1 = dx2 * dx3, a2 = dx1 * dx3, a3 = dx1 * dx2;
    const double vol = dx1 * dx2 * dx3;
    const int64_t c = cidx(g, k, j, i);
    const int64_t q1 = f1idx(g, k, j, i), q2 = f2idx(g, k, j, i), q3 = f3idx(g, k, j, i);
    const int64_t s2 = g.nc1, s3 = (int64_t)g.nc1 * g.nc2;
#pragma unroll
    for (int n = 0; n < NHYD; ++n) {
      double uo = u[n * nc + c];
      double r = sw.zero_reg ? 0.0 : u1[n * nc + c];
      if (sw.delta != 0.0) { r += sw.delta * uo; u1[n * nc + c] = r; }
      double base = sw.swap ? r : sw.g1 * uo + sw.g2 * r;
      double d = (a1 * (double)F1[n * g.nf1 + q1 + 1] - a1 * (double)F1[n * g.nf1 + q1]);
      d += (a2 * (double)F2[n * g.nf2 + q2 + s2] - a2 * (double)F2[n * g.nf2 + q2]);
      d += (a3 * (double)F3[n * g.nf3 + q3 + s3] - a3 * (double)F3[n * g.nf3 + q3]);
      u[n * nc + c] = base - wght * d / vol;
    }
  }
  if constexpr (MHD) {
    const double* E1 = p.edge + (int64_t)b * 3 * g.ne;
    const double* E2 = E1 + g.ne;
    const double* E3 = E2 + g.ne;
    const double ar1 = dx2 * dx3, ar2 = dx1 * dx3, ar3 = dx1 * dx2;
    const double l1 = dx1, l2 = dx2, l3 = dx3;
    const int64_t e = eidx(g, k, j, i);
    const int64_t ej = (int64_t)g.nc1 + 1, ek = ((int64_t)g.nc1 + 1) * (g.nc2 + 1);
    // applies "-= (w/a)*curl_m" and "+= (w/a)*curl_p" in the reference's order
    auto face = [&](double* bb, double* rr, int64_t q, double curl_m, double curl_p,
                    double ar, bool plus_first) {
      double bo = bb[q];
      double r = sw.zero_reg ? 0.0 : rr[q];
      if (sw.delta != 0.0) { r += sw.delta * bo; rr[q] = r; }
      double v = sw.swap ? r : sw.g1 * bo + sw.g2 * r;
      if (plus_first) {
        v += (wght / ar) * curl_p;
        v -= (wght / ar) * curl_m;
      } else {
        v -= (wght / ar) * curl_m;
        v += (wght / ar) * curl_p;
      }
      bb[q] = v;
    };
    if (j <= g.je && k <= g.ke) {  // B1 at (k,j,i), i in [is, ie+1]
      int64_t q = (int64_t)b * g.nf1 + f1idx(g, k, j, i);
      face(p.b1, p.r1, q, (l3 * E3[e + ej] - l3 * E3[e]), (l2 * E2[e + ek] - l2 * E2[e]), ar1,
           false);
    }
    if (i <= g.ie && k <= g.ke) {  // B2 at (k,j,i), j in [js, je+1]
      int64_t q = (int64_t)b * g.nf2 + f2idx(g, k, j, i);
      // ct.cpp:80-93: b2 += (w/a)*(curl e3 along i) first, then b2 -= (w/a)*(curl e1 along k)
      face(p.b2, p.r2, q, (l1 * E1[e + ek] - l1 * E1[e]), (l3 * E3[e + 1] - l3 * E3[e]), ar2,
           true);
    }
    if (i <= g.ie && j <= g.je) {  // B3 at (k,j,i), k in [ks, ke+1]
      int64_t q = (int64_t)b * g.nf3 + f3idx(g, k, j, i);
      face(p.b3, p.r3, q, (l2 * E2[e + 1] - l2 * E2[e]), (l1 * E1[e + ej] - l1 * E1[e]), ar3,
           false);
    }
  }
}

// Conserved -> primitive with floors over every cell of every block (interior and
// ghosts). Reference src/eos/adiabatic_mhd.cpp:41-90 (adiabatic_hydro.cpp:39-81) and the
// uniform cell-centred field average of src/field/field.cpp:112-180. The EOS arithmetic
// is FP64 in both paths; W and bcc are stored as T.
template <typename T, bool MHD>
__global__ void __launch_bounds__(256) k_c2p(Geom g, StagePtrs<T> p, Box bx, Phys ph) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  const int64_t nc = g.ncell;
  const int64_t c = cidx(g, k, j, i);
  double* u = p.u + (int64_t)b * NHYD * nc;
  T* w = p.w + (int64_t)b * NHYD * nc;
  const double gm1 = ph.gamma - 1.0;
  double pb = 0.0;
  if constexpr (MHD) {
    const double* b1 = p.b1 + (int64_t)b * g.nf1;
    const double* b2 = p.b2 + (int64_t)b * g.nf2;
    const double* b3 = p.b3 + (int64_t)b * g.nf3;
    double bc1 = 0.5 * b1[f1idx(g, k, j, i)] + 0.5 * b1[f1idx(g, k, j, i + 1)];
    double bc2 = 0.5 * b2[f2idx(g, k, j, i)] + 0.5 * b2[f2idx(g, k, j + 1, i)];
    double bc3 = 0.5 * b3[f3idx(g, k, j, i)] + 0.5 * b3[f3idx(g, k + 1, j, i)];
    T* bcc = p.bcc + (int64_t)b * 3 * nc;
    bcc[c] = (T)bc1; bcc[nc + c] = (T)bc2; bcc[2 * nc + c] = (T)bc3;
    pb = 0.5 * (bc1 * bc1 + bc2 * bc2 + bc3 * bc3);
  }
  double ud = u[c], m1 = u[nc + c], m2 = u[2 * nc + c], m3 = u[3 * nc + c], ue = u[4 * nc + c];
  ud = (ud > ph.dfloor) ? ud : ph.dfloor;
  u[c] = ud;
  double di = 1.0 / ud;
  double e_k = 0.5 * di * (m1 * m1 + m2 * m2 + m3 * m3);
  double wp = MHD ? gm1 * (ue - e_k - pb) : gm1 * (ue - e_k);
  if (!(wp > ph.pfloor)) {
    u[4 * nc + c] = MHD ? ((ph.pfloor / gm1) + e_k + pb) : ((ph.pfloor / gm1) + e_k);
    wp = ph.pfloor;
  }
  w[c] = (T)ud;
  w[nc + c] = (T)(m1 * di);
  w[2 * nc + c] = (T)(m2 * di);
  w[3 * nc + c] = (T)(m3 * di);
  w[4 * nc + c] = (T)wp;
}

// Per-block CFL limit (src/hydro/new_blockdt.cpp:58-158) reduced over the whole pool
// in one launch: warp-shuffle min, block min, then one 64-bit atomicMin (positive
// doubles order like their bit patterns).
template <typename T, bool MHD>
__global__ void __launch_bounds__(256)
k_block_dt(Geom g, StagePtrs<T> p, Box bx, Phys ph, unsigned long long* dtmin) {
  int i, j, k, b;
  double mindt = 1.79769313486231570815e308;
  if (box_coords(bx, i, j, k, b)) {
    const int64_t nc = g.ncell, c = cidx(g, k, j, i);
    const T* w = p.w + (int64_t)b * NHYD * nc;
    const BlockGeo geo = p.geo[b];
    double d = w[c], vx = w[nc + c], vy = w[2 * nc + c], vz = w[3 * nc + c], pr = w[4 * nc + c];
    double dt1, dt2, dt3;
    if constexpr (MHD) {
      const T* bcc = p.bcc + (int64_t)b * 3 * nc;
      double bc1 = bcc[c], bc2 = bcc[nc + c], bc3 = bcc[2 * nc + c];
      double bx1 = bc1 + fabs(p.b1[(int64_t)b * g.nf1 + f1idx(g, k, j, i)] - bc1);
      double cf = fast_speed<double>(d, pr, bc2, bc3, bx1, ph.gamma);
      dt1 = geo.dx[0] / (fabs(vx) + cf);
      double bx2 = bc2 + fabs(p.b2[(int64_t)b * g.nf2 + f2idx(g, k, j, i)] - bc2);
      cf = fast_speed<double>(d, pr, bc3, bc1, bx2, ph.gamma);
      dt2 = geo.dx[1] / (fabs(vy) + cf);
      double bx3 = bc3 + fabs(p.b3[(int64_t)b * g.nf3 + f3idx(g, k, j, i)] - bc3);
      cf = fast_speed<double>(d, pr, bc1, bc2, bx3, ph.gamma);
      dt3 = geo.dx[2] / (fabs(vz) + cf);
    } else {
      double cs = sqrt(ph.gamma * pr / d);
      dt1 = geo.dx[0] / (fabs(vx) + cs);
      dt2 = geo.dx[1] / (fabs(vy) + cs);
      dt3 = geo.dx[2] / (fabs(vz) + cs);
    }
    mindt = mn(mn(mn(mindt, dt1), dt2), dt3);
  }
  for (int o = 16; o > 0; o >>= 1) mindt = mn(mindt, __shfl_xor_sync(0xffffffffu, mindt, o));
  __shared__ double red[32];
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  const int nt = blockDim.x * blockDim.y;
  if ((tid & 31) == 0) red[tid >> 5] = mindt;
  __syncthreads();
  if (tid < 32) {
    double v = (tid < (nt + 31) / 32) ? red[tid] : 1.79769313486231570815e308;
    for (int o = 16; o > 0; o >>= 1) v = mn(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (tid == 0) atomicMin(dtmin, (unsigned long long)__double_as_longlong(v));
  }
}

}  // namespace athg

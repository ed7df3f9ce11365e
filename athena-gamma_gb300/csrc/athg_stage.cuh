// athg_stage.cuh -- per-stage kernels of the finite-volume (M)HD update, templated on
// the arithmetic type T of primitives/fluxes (double: plain FP64 path, float: mixed
// path). Conserved variables, face fields and the CT update are FP64 in both paths.
//
// Each launch covers every MeshBlock of the pool (grid.z runs over k and blocks).
#pragma once
#include <type_traits>

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
  T *edge;                   // corner EMFs [nb][3][edges]
  T *cce;                    // mixed path: cell-centred E = -v x B [nb][3][cells], written
                             // by k_c2p for k_corner_emf (nullptr in the FP64 path)
  const BlockGeo *geo;       // [nb] cell widths (FP64)
  const T *coef;             // PLM interface coefficients [nb][3][2][ncmax]
  const T *dxT;              // [nb][3] cell widths in T
  const double *dt;          // current time step (device scalar)
  const T *dtT;              // the same time step in T
  const T *bf[3];            // face field as read by the flux kernels: the FP64 field itself,
                             // or its FP32 copy (written by k_c2p) in the mixed path
  T *bfw[3];                 // where k_c2p writes that FP32 copy (mixed path only)
  const MixedGeo *mg;        // [nb] widths of the mixed-path update
};

// The mixed path keeps FP64 work (which runs at a small fraction of the FP32 rate on this
// GPU, conversions included) out of the FP32 kernels.
template <typename T> constexpr bool kMixed = std::is_same<T, float>::value;

// Index box of one launch: every (i,j) of the box is flattened onto grid.x (so ranges
// like is..ie+1 do not leave idle half-warps), grid.y runs over k, grid.z over blocks.
struct Box {
  int il, jl, kl, ni, nj, nk;
  FastDiv dni;  // division by ni
};
inline Box box_make(int il, int iu, int jl, int ju, int kl, int ku) {
  Box b;
  b.il = il; b.jl = jl; b.kl = kl;
  b.ni = iu - il + 1; b.nj = ju - jl + 1; b.nk = ku - kl + 1;
  b.dni = fastdiv_make((uint32_t)b.ni);
  return b;
}
__device__ __forceinline__ bool box_coords(const Box& bx, int& i, int& j, int& k, int& b) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= bx.ni * bx.nj) return false;
  int jj = fastdiv(t, bx.dni);
  i = bx.il + (t - jj * bx.ni);
  j = bx.jl + jj;
  k = bx.kl + blockIdx.y;
  b = blockIdx.z;
  return true;
}

// Block sizes of a launch: compile-time constants for SNC > 0 (blocks of SNC^3 cells, ghosts
// included, so strides fold into the loads' immediate offsets), else the context's.
template <int SNC>
struct BlockDims {
  int64_t nc1, nc2, ncell, nf1, nf2, nf3, ne;
  __device__ __forceinline__ explicit BlockDims(const Geom& g) {
    if constexpr (SNC > 0) {
      constexpr int64_t S = SNC;
      nc1 = S; nc2 = S; ncell = S * S * S;
      nf1 = nf2 = nf3 = S * S * (S + 1);
      ne = (S + 1) * (S + 1) * (S + 1);
    } else {
      nc1 = g.nc1; nc2 = g.nc2; ncell = g.ncell;
      nf1 = g.nf1; nf2 = g.nf2; nf3 = g.nf3; ne = g.ne;
    }
  }
  __device__ __forceinline__ int64_t cell(int k, int j, int i) const {
    return ((int64_t)k * nc2 + j) * nc1 + i;
  }
  __device__ __forceinline__ int64_t f1(int k, int j, int i) const {
    return ((int64_t)k * nc2 + j) * (nc1 + 1) + i;
  }
  __device__ __forceinline__ int64_t f2(int k, int j, int i) const {
    return ((int64_t)k * (nc2 + 1) + j) * nc1 + i;
  }
  __device__ __forceinline__ int64_t edge(int k, int j, int i) const {
    return ((int64_t)k * (nc2 + 1) + j) * (nc1 + 1) + i;
  }
};

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

// Hydro::CalculateVelocityDifferences (hydro/calculate_velocity_differences.cpp:20-52,
// 3-D) at face (k,j,i) of a DIR sweep: the normal velocity jump and the smallest
// transverse velocity difference around the face (the LHLLC/LHLLD shock detector).
template <typename T, int DIR>
__device__ __forceinline__ void velocity_differences(const Geom& g, const T* __restrict__ w,
                                                     int k, int j, int i, T& dvn, T& dvt) {
  const int64_t nc = g.ncell;
  const T* vx = w + IVX * nc;
  const T* vy = w + IVY * nc;
  const T* vz = w + IVZ * nc;
  auto W = [&](const T* a, int kk, int jj, int ii) { return a[cidx(g, kk, jj, ii)]; };
  T dvl, dvr, dwl, dwr;
  if (DIR == 0) {
    dvn = W(vx, k, j, i) - W(vx, k, j, i - 1);
    dvl = mn(W(vy, k, j + 1, i - 1) - W(vy, k, j, i - 1), W(vy, k, j, i - 1) - W(vy, k, j - 1, i - 1));
    dvr = mn(W(vy, k, j + 1, i) - W(vy, k, j, i), W(vy, k, j, i) - W(vy, k, j - 1, i));
    dwl = mn(W(vz, k + 1, j, i - 1) - W(vz, k, j, i - 1), W(vz, k, j, i - 1) - W(vz, k - 1, j, i - 1));
    dwr = mn(W(vz, k + 1, j, i) - W(vz, k, j, i), W(vz, k, j, i) - W(vz, k - 1, j, i));
  } else if (DIR == 1) {
    dvn = W(vy, k, j, i) - W(vy, k, j - 1, i);
    dvl = mn(W(vz, k + 1, j - 1, i) - W(vz, k, j - 1, i), W(vz, k, j - 1, i) - W(vz, k - 1, j - 1, i));
    dvr = mn(W(vz, k + 1, j, i) - W(vz, k, j, i), W(vz, k, j, i) - W(vz, k - 1, j, i));
    dwl = mn(W(vx, k, j - 1, i + 1) - W(vx, k, j - 1, i), W(vx, k, j - 1, i) - W(vx, k, j - 1, i - 1));
    dwr = mn(W(vx, k, j, i + 1) - W(vx, k, j, i), W(vx, k, j, i) - W(vx, k, j, i - 1));
  } else {
    dvn = W(vz, k, j, i) - W(vz, k - 1, j, i);
    dvl = mn(W(vx, k - 1, j, i + 1) - W(vx, k - 1, j, i), W(vx, k - 1, j, i) - W(vx, k - 1, j, i - 1));
    dvr = mn(W(vx, k, j, i + 1) - W(vx, k, j, i), W(vx, k, j, i) - W(vx, k, j, i - 1));
    dwl = mn(W(vy, k - 1, j + 1, i) - W(vy, k - 1, j, i), W(vy, k - 1, j, i) - W(vy, k - 1, j - 1, i));
    dwr = mn(W(vy, k, j + 1, i) - W(vy, k, j, i), W(vy, k, j, i) - W(vy, k, j - 1, i));
  }
  dvt = mn(mn(dvl, dvr), mn(dwl, dwr));
}

// Face-flux kernel: one thread per face. Reconstruction (donor cell or van Leer PLM,
// reference src/reconstruct/dc.cpp, src/reconstruct/plm.cpp uniform branch) fused with
// the Riemann solve. Face (k,j,i) along DIR separates cell index-1 from cell index.
// Loop extents per direction follow src/hydro/calculate_fluxes.cpp:63-74,164-172,274-279.
// SNC > 0: blocks of SNC^3 cells (BlockDims), compile-time strides.
template <typename T, int DIR, int ORDER, int SOLVER, bool MHD, int SNC = 0>
__global__ void __launch_bounds__(128)
k_flux(Geom g, StagePtrs<T> p, Box bx, Phys ph) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  constexpr int NW = MHD ? 7 : 5;
  constexpr int NF = MHD ? 8 : 5;
  const BlockDims<SNC> d(g);
  const int64_t nc = d.ncell;
  const T* __restrict__ w = p.w + (int64_t)b * NHYD * nc;
  const T* __restrict__ bcc = MHD ? p.bcc + (int64_t)b * 3 * nc : nullptr;
  const int64_t st = DIR == 0 ? 1 : (DIR == 1 ? d.nc1 : d.nc1 * d.nc2);
  const int64_t c = d.cell(k, j, i);   // cell on the right of the face
  const int f = DIR == 0 ? i : (DIR == 1 ? j : k);
  T wl[7], wr[7];
  if (ORDER == 1) {
#pragma unroll
    for (int n = 0; n < NW; ++n) {
      wl[n] = wave_var<T, DIR>(w, bcc, nc, n, c - st);
      wr[n] = wave_var<T, DIR>(w, bcc, nc, n, c);
    }
  } else if (ORDER == 3) {
#pragma unroll
    for (int n = 0; n < NW; ++n) {
      T v0 = wave_var<T, DIR>(w, bcc, nc, n, c - 3 * st);
      T v1 = wave_var<T, DIR>(w, bcc, nc, n, c - 2 * st);
      T v2 = wave_var<T, DIR>(w, bcc, nc, n, c - st);
      T v3 = wave_var<T, DIR>(w, bcc, nc, n, c);
      T v4 = wave_var<T, DIR>(w, bcc, nc, n, c + st);
      T v5 = wave_var<T, DIR>(w, bcc, nc, n, c + 2 * st);
      T qm, qp, unused;
      ppm_cell<T>(v0, v1, v2, v3, v4, unused, qp);
      ppm_cell<T>(v1, v2, v3, v4, v5, qm, unused);
      wl[n] = qp;
      wr[n] = qm;
    }
    // density and pressure floors on the PPM states (ppm.cpp:326-332)
    const T df = ph_dfloor<T>(ph), pf = ph_pfloor<T>(ph);
    wl[IDN] = (wl[IDN] > df) ? wl[IDN] : df; wl[IPR] = (wl[IPR] > pf) ? wl[IPR] : pf;
    wr[IDN] = (wr[IDN] > df) ? wr[IDN] : df; wr[IPR] = (wr[IPR] > pf) ? wr[IPR] : pf;
  } else {
    const T* cf = p.coef + ((int64_t)b * 3 + DIR) * 2 * g.ncmax;
    const T cpL = cf[f - 1];                 // (x_f(c+1) - x_v(c)) / dx  for c = f-1
    const T cmR = cf[g.ncmax + f];           // (x_v(c) - x_f(c)) / dx    for c = f
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
  constexpr int64_t S = SNC;
  const int64_t nf = SNC ? S * S * (S + 1) : fsize<DIR>(g);
  const int64_t fi = DIR == 0 ? d.f1(k, j, i) : (DIR == 1 ? d.f2(k, j, i) : d.cell(k, j, i));
  T* __restrict__ out = p.flx[DIR] + (int64_t)b * NF * nf;
  const T gam = ph_gamma<T>(ph);
  if constexpr (MHD) {
    wli[IBY] = wl[IBY]; wli[IBZ] = wl[IBZ];
    wri[IBY] = wr[IBY]; wri[IBZ] = wr[IBZ];
    const T bxi = p.bf[DIR][(int64_t)b * nf + fi];
    if (SOLVER == HLLD) {
      rs_hlld<T>(wli, wri, bxi, gam, fx);
    } else if (SOLVER == LHLLD) {
      T dvn, dvt;
      velocity_differences<T, DIR>(g, p.w + (int64_t)b * NHYD * g.ncell, k, j, i, dvn, dvt);
      rs_lhlld<T>(wli, wri, bxi, gam, dvn, dvt, fx);
    } else {
      rs_hlle_mhd<T>(wli, wri, bxi, gam, fx);
    }
    out[5 * nf + fi] = -fx[IBY];
    out[6 * nf + fi] = fx[IBZ];
    out[7 * nf + fi] = ct_weight<T>(fx[IDN], wli[IDN], wri[IDN], p.dxT[b * 3 + DIR], *p.dtT);
  } else {
    if (SOLVER == HLLC) {
      rs_hllc<T>(wli, wri, gam, fx);
    } else if (SOLVER == LHLLC) {
      T dvn, dvt;
      velocity_differences<T, DIR>(g, p.w + (int64_t)b * NHYD * g.ncell, k, j, i, dvn, dvt);
      rs_lhllc<T>(wli, wri, gam, dvn, dvt, fx);
    } else {
      rs_hlle_hydro<T>(wli, wri, gam, fx);
    }
  }
  out[IDN * nf + fi] = fx[IDN];
  out[ivx * nf + fi] = fx[IVX];
  out[ivy * nf + fi] = fx[IVY];
  out[ivz * nf + fi] = fx[IVZ];
  out[IEN * nf + fi] = fx[IEN];
}

// Riemann solve of one face from reconstructed states in the unrotated order, storing the
// flux (and for MHD the face EMFs and CT weight) like k_flux.
template <typename T, int DIR, int SOLVER, bool MHD, int SNC = 0>
__device__ __forceinline__ void face_solve(const Geom& g, const StagePtrs<T>& p, const Phys& ph,
                                           int b, int64_t fi, const T* wl, const T* wr,
                                           int k, int j, int i) {
  constexpr int64_t S = SNC;
  constexpr int NF = MHD ? 8 : 5;
  constexpr int ivx = IVX + DIR, ivy = IVX + (DIR + 1) % 3, ivz = IVX + (DIR + 2) % 3;
  T wli[7], wri[7], fx[7];
  wli[IDN] = wl[IDN]; wli[IVX] = wl[ivx]; wli[IVY] = wl[ivy]; wli[IVZ] = wl[ivz];
  wli[IPR] = wl[IPR];
  wri[IDN] = wr[IDN]; wri[IVX] = wr[ivx]; wri[IVY] = wr[ivy]; wri[IVZ] = wr[ivz];
  wri[IPR] = wr[IPR];
  const int64_t nf = SNC ? S * S * (S + 1) : fsize<DIR>(g);
  T* __restrict__ out = p.flx[DIR] + (int64_t)b * NF * nf;
  const T gam = ph_gamma<T>(ph);
  if constexpr (MHD) {
    wli[IBY] = wl[IBY]; wli[IBZ] = wl[IBZ];
    wri[IBY] = wr[IBY]; wri[IBZ] = wr[IBZ];
    const T bxi = p.bf[DIR][(int64_t)b * nf + fi];
    if (SOLVER == HLLD) {
      rs_hlld<T>(wli, wri, bxi, gam, fx);
    } else if (SOLVER == LHLLD) {
      T dvn, dvt;
      velocity_differences<T, DIR>(g, p.w + (int64_t)b * NHYD * g.ncell, k, j, i, dvn, dvt);
      rs_lhlld<T>(wli, wri, bxi, gam, dvn, dvt, fx);
    } else {
      rs_hlle_mhd<T>(wli, wri, bxi, gam, fx);
    }
    out[5 * nf + fi] = -fx[IBY];
    out[6 * nf + fi] = fx[IBZ];
    out[7 * nf + fi] = ct_weight<T>(fx[IDN], wli[IDN], wri[IDN], p.dxT[b * 3 + DIR], *p.dtT);
  } else {
    if (SOLVER == HLLC) {
      rs_hllc<T>(wli, wri, gam, fx);
    } else if (SOLVER == LHLLC) {
      T dvn, dvt;
      velocity_differences<T, DIR>(g, p.w + (int64_t)b * NHYD * g.ncell, k, j, i, dvn, dvt);
      rs_lhllc<T>(wli, wri, gam, dvn, dvt, fx);
    } else {
      rs_hlle_hydro<T>(wli, wri, gam, fx);
    }
  }
  out[IDN * nf + fi] = fx[IDN];
  out[ivx * nf + fi] = fx[IVX];
  out[ivy * nf + fi] = fx[IVY];
  out[ivz * nf + fi] = fx[IVZ];
  out[IEN * nf + fi] = fx[IEN];
}

// x1 PPM sweep in two phases: a thread block takes `rows` whole i-rows of the face box;
// first one thread per cell reconstructs the cell once (ppm_cell gives the states at both
// of its faces) into shared memory, then one thread per face takes the left state from
// the cell below and the right state from the cell above and solves. k_flux instead
// reconstructs both cells of every face, so each cell twice; the states, and so the
// fluxes, are the same values bit for bit. Shared memory: 2 * rows * NW * (ni + 1) values.
// (For PLM, whose slope is cheap, the extra pass through shared memory costs more than
// the second slope: measured slower in FP32 and no faster in FP64.)
template <typename T, int SOLVER, bool MHD>
__global__ void __launch_bounds__(256)
k_flux_x1_ppm(Geom g, StagePtrs<T> p, Box bx, Phys ph, int rows) {
  constexpr int NW = MHD ? 7 : 5;
  const int W = bx.ni;     // faces il .. il + W - 1 of a row
  const int C = W + 1;     // cells il - 1 .. il + W - 1
  extern __shared__ unsigned char x1_smem[];
  T* qm = reinterpret_cast<T*>(x1_smem);  // [rows][NW][C]: state at the cell's lower face
  T* qp = qm + (int64_t)rows * NW * C;    //                 state at its upper face
  const int b = blockIdx.z;
  const int nrows = bx.nj * bx.nk;
  const int r0 = blockIdx.x * rows;
  const int64_t nc = g.ncell;
  const T* __restrict__ w = p.w + (int64_t)b * NHYD * nc;
  const T* __restrict__ bcc = MHD ? p.bcc + (int64_t)b * 3 * nc : nullptr;
  for (int t = threadIdx.x; t < rows * C; t += blockDim.x) {
    const int rr = t / C, cc = t - rr * C;
    const int row = r0 + rr;
    if (row >= nrows) continue;
    const int j = bx.jl + row % bx.nj, k = bx.kl + row / bx.nj;
    const int64_t c = cidx(g, k, j, bx.il - 1 + cc);
#pragma unroll
    for (int n = 0; n < NW; ++n) {
      const T v0 = wave_var<T, 0>(w, bcc, nc, n, c - 2), v1 = wave_var<T, 0>(w, bcc, nc, n, c - 1),
              v2 = wave_var<T, 0>(w, bcc, nc, n, c), v3 = wave_var<T, 0>(w, bcc, nc, n, c + 1),
              v4 = wave_var<T, 0>(w, bcc, nc, n, c + 2);
      T m, q;
      ppm_cell<T>(v0, v1, v2, v3, v4, m, q);
      qm[((int64_t)rr * NW + n) * C + cc] = m;
      qp[((int64_t)rr * NW + n) * C + cc] = q;
    }
  }
  __syncthreads();
  const T df = ph_dfloor<T>(ph), pf = ph_pfloor<T>(ph);
  for (int t = threadIdx.x; t < rows * W; t += blockDim.x) {
    const int rr = t / W, ff = t - rr * W;
    const int row = r0 + rr;
    if (row >= nrows) continue;
    const int j = bx.jl + row % bx.nj, k = bx.kl + row / bx.nj, i = bx.il + ff;
    T wl[7], wr[7];
#pragma unroll
    for (int n = 0; n < NW; ++n) {
      wl[n] = qp[((int64_t)rr * NW + n) * C + ff];      // cell i - 1
      wr[n] = qm[((int64_t)rr * NW + n) * C + ff + 1];  // cell i
    }
    // density and pressure floors on the PPM states (ppm.cpp:326-332)
    wl[IDN] = (wl[IDN] > df) ? wl[IDN] : df; wl[IPR] = (wl[IPR] > pf) ? wl[IPR] : pf;
    wr[IDN] = (wr[IDN] > df) ? wr[IDN] : df; wr[IPR] = (wr[IPR] > pf) ? wr[IPR] : pf;
    face_solve<T, 0, SOLVER, MHD>(g, p, ph, b, fidx<0>(g, k, j, i), wl, wr, k, j, i);
  }
}

// Marching face-flux kernel for the j (DIR=1) and k (DIR=2) sweeps: one thread per
// pencil along DIR (consecutive threads on consecutive i, so every load is coalesced),
// walking faces fs..fe with a register window of three cells. Each cell is loaded once
// and its limited slope computed once, giving the right state of its lower face and the
// left state of its upper face -- the same row-by-row reuse as the reference's
// wl_/wlb_ swap in hydro/calculate_fluxes.cpp:174-212 and :278-316.
// The box describes the transverse pencil set (i, and k or j) and the face range (nk).
// The FP32 instantiation (kernels_f32.cu, ATHG_MARCH_MIN_BLOCKS 5) is held to five blocks of
// 128 per SM, at most 96 registers: 2.4% faster PLM sweeps on a GB300 at 256^3. The FP64
// one keeps the compiler's allocation (held to five blocks it ran 1.8% slower, and even an
// explicit minimum of one block changes its register allocation).
#ifdef ATHG_MARCH_MIN_BLOCKS
#define ATHG_MARCH_BOUNDS __launch_bounds__(128, ATHG_MARCH_MIN_BLOCKS)
#else
#define ATHG_MARCH_BOUNDS __launch_bounds__(128)
#endif
template <typename T, int DIR, int ORDER, int SOLVER, bool MHD, int SNC = 0>
__global__ void ATHG_MARCH_BOUNDS
k_flux_march(Geom g, StagePtrs<T> p, Box bx, Phys ph, int fs, int fe) {
  static_assert(DIR == 1 || DIR == 2, "marching sweeps are transverse to i");
  int i, a, unused, b;
  {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= bx.ni * bx.nj) return;
    int aa = t / bx.ni;
    i = bx.il + (t - aa * bx.ni);
    a = bx.jl + aa;  // the other transverse index: k for DIR=1, j for DIR=2
    b = blockIdx.z;
    (void)unused;
  }
  // grid.y splits each pencil into segments (shorter dependency chains, more threads);
  // every segment rebuilds its window from the cells before its first face
  {
    const int len = (fe - fs + (int)gridDim.y) / (int)gridDim.y;
    const int s0 = fs + (int)blockIdx.y * len;
    const int s1 = min(fe, s0 + len - 1);
    if (s0 > s1) return;
    fs = s0;
    fe = s1;
  }
  constexpr int NW = MHD ? 7 : 5;
  const BlockDims<SNC> d(g);
  const int64_t nc = d.ncell;
  const T* __restrict__ w = p.w + (int64_t)b * NHYD * nc;
  const T* __restrict__ bcc = MHD ? p.bcc + (int64_t)b * 3 * nc : nullptr;
  const int64_t st = DIR == 1 ? d.nc1 : d.nc1 * d.nc2;
  // cell index of pencil position f
  auto cell_at = [&](int f) -> int64_t {
    return DIR == 1 ? d.cell(a, f, i) : d.cell(f, a, i);
  };
  auto face_at = [&](int f) -> int64_t {
    return DIR == 1 ? d.f2(a, f, i) : d.cell(f, a, i);
  };
  const T* cf = p.coef + ((int64_t)b * 3 + DIR) * 2 * g.ncmax;
  T cm1[7], c0[7], cp1[7], wlnext[7], wr[7];
  if (ORDER == 1) {
    int64_t c = cell_at(fs - 1);
#pragma unroll
    for (int n = 0; n < NW; ++n) wlnext[n] = wave_var<T, DIR>(w, bcc, nc, n, c);
    for (int f = fs; f <= fe; ++f) {
      int64_t cc = c + st;
#pragma unroll
      for (int n = 0; n < NW; ++n) wr[n] = wave_var<T, DIR>(w, bcc, nc, n, cc);
      face_solve<T, DIR, SOLVER, MHD, SNC>(g, p, ph, b, face_at(f), wlnext, wr, DIR == 1 ? a : f,
                                      DIR == 1 ? f : a, i);
#pragma unroll
      for (int n = 0; n < NW; ++n) wlnext[n] = wr[n];
      c = cc;
    }
    return;
  }
  if (ORDER == 3) {
    // PPM: window of five cells; cell f gives the right state of face f (qminus) and
    // the left state of face f+1 (qplus)
    const T df = ph_dfloor<T>(ph), pf = ph_pfloor<T>(ph);
    T win[5][7];
    int64_t c = cell_at(fs - 1);
#pragma unroll
    for (int n = 0; n < NW; ++n) {
#pragma unroll
      for (int q = 0; q < 5; ++q) win[q][n] = wave_var<T, DIR>(w, bcc, nc, n, c + (q - 2) * st);
      T unused;
      ppm_cell<T>(win[0][n], win[1][n], win[2][n], win[3][n], win[4][n], unused, wlnext[n]);
    }
    for (int f = fs; f <= fe; ++f) {
      c += st;  // cell f
#pragma unroll
      for (int n = 0; n < NW; ++n) {
        win[0][n] = win[1][n]; win[1][n] = win[2][n]; win[2][n] = win[3][n];
        win[3][n] = win[4][n];
        win[4][n] = wave_var<T, DIR>(w, bcc, nc, n, c + 2 * st);
        T qm, qp;
        ppm_cell<T>(win[0][n], win[1][n], win[2][n], win[3][n], win[4][n], qm, qp);
        wr[n] = qm;
        cm1[n] = wlnext[n];
        wlnext[n] = qp;
      }
      cm1[IDN] = (cm1[IDN] > df) ? cm1[IDN] : df; cm1[IPR] = (cm1[IPR] > pf) ? cm1[IPR] : pf;
      wr[IDN] = (wr[IDN] > df) ? wr[IDN] : df; wr[IPR] = (wr[IPR] > pf) ? wr[IPR] : pf;
      face_solve<T, DIR, SOLVER, MHD, SNC>(g, p, ph, b, face_at(f), cm1, wr, DIR == 1 ? a : f,
                                      DIR == 1 ? f : a, i);
    }
    return;
  }
  // prologue: cells fs-2, fs-1, fs -> left state of face fs from the slope of cell fs-1
  {
    int64_t c = cell_at(fs - 1);
    const T cp = cf[fs - 1];
#pragma unroll
    for (int n = 0; n < NW; ++n) {
      cm1[n] = wave_var<T, DIR>(w, bcc, nc, n, c - st);
      c0[n] = wave_var<T, DIR>(w, bcc, nc, n, c);
      cp1[n] = wave_var<T, DIR>(w, bcc, nc, n, c + st);
      T dwl = (c0[n] - cm1[n]), dwr = (cp1[n] - c0[n]);
      T dw2 = dwl * dwr;
      T dwm = T(2.0) * dw2 / (dwl + dwr);
      if (dw2 <= T(0.0)) dwm = T(0.0);
      wlnext[n] = c0[n] + cp * dwm;
    }
  }
  // The cell a face step needs next is loaded one step ahead, before the Riemann solve of
  // the current face, so its load latency is spent under the solve (measured: 6.6% off the
  // PLM sweeps; the donor-cell sweeps, whose extra registers cost a block per SM, keep
  // loading in step).
  int64_t c = cell_at(fs);  // c0 <- cell fs (window shifts at loop start)
  T ahead[7];                // cell fs + 1, then one cell ahead of each step
#pragma unroll
  for (int n = 0; n < NW; ++n) ahead[n] = wave_var<T, DIR>(w, bcc, nc, n, c + st);
  for (int f = fs; f <= fe; ++f) {
    const T cmR = cf[g.ncmax + f], cpR = cf[f];
#pragma unroll
    for (int n = 0; n < NW; ++n) {
      cm1[n] = c0[n];
      c0[n] = cp1[n];
      cp1[n] = ahead[n];
      T dwl = (c0[n] - cm1[n]), dwr = (cp1[n] - c0[n]);
      T dw2 = dwl * dwr;
      T dwm = T(2.0) * dw2 / (dwl + dwr);
      if (dw2 <= T(0.0)) dwm = T(0.0);
      wr[n] = c0[n] - cmR * dwm;
      cm1[n] = wlnext[n];                 // reuse the slot: left state of face f
      wlnext[n] = c0[n] + cpR * dwm;      // left state of face f+1
    }
    if (f < fe) {
#pragma unroll
      for (int n = 0; n < NW; ++n) ahead[n] = wave_var<T, DIR>(w, bcc, nc, n, c + 2 * st);
    }
    face_solve<T, DIR, SOLVER, MHD, SNC>(g, p, ph, b, face_at(f), cm1, wr, DIR == 1 ? a : f,
                                    DIR == 1 ? f : a, i);
    c += st;
  }
}

// Corner EMFs (Gardiner & Stone upwind integration), one thread per corner location
// (k,j,i) in [ks,ke+1]x[js,je+1]x[is,ie+1] computing e1, e2, e3 there.
// Reference src/field/calculate_corner_e.cpp:129-229 (3-D, Newtonian). The cell-centred
// E = -v x B is recomputed from W and bcc where needed instead of being stored (the mixed
// path reads it from cce, written by the update).
// SNC > 0: blocks of SNC^3 cells (ghosts included), a compile-time size, so the strides
// fold into the loads' immediate offsets; 0: any size (the same arithmetic either way).
template <typename T, int SNC>
__global__ void __launch_bounds__(128) k_corner_emf(Geom g, StagePtrs<T> p, Box bx) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  const int nc1 = SNC ? SNC : g.nc1, nc2 = SNC ? SNC : g.nc2;
  constexpr int64_t S = SNC;
  const int64_t nc = SNC ? S * S * S : g.ncell;
  const T* w = p.w + (int64_t)b * NHYD * nc;
  const T* bc = p.bcc + (int64_t)b * 3 * nc;
  const T* ce = kMixed<T> ? p.cce + (int64_t)b * 3 * nc : nullptr;
  // Every value sits at this corner's index or one below it along some axes: the
  // accessors take those offsets (0 or -1 per axis), so each load is a base pointer plus
  // a stride combination formed once, not a fresh 64-bit index polynomial.
  const int64_t c0 = ((int64_t)k * nc2 + j) * nc1 + i;
  const int64_t q1 = ((int64_t)k * nc2 + j) * (nc1 + 1) + i;
  const int64_t q2 = ((int64_t)k * (nc2 + 1) + j) * nc1 + i;
  const int64_t jc = nc1, kc = (int64_t)nc1 * nc2;             // cells, x3 faces
  const int64_t j1 = nc1 + 1, k1 = (int64_t)(nc1 + 1) * nc2;   // x1 faces
  const int64_t j2 = nc1, k2 = (int64_t)nc1 * (nc2 + 1);       // x2 faces
  auto cce = [&](int n, int dk, int dj, int di) -> T {
    const int64_t c = c0 + dk * kc + dj * jc + di;
    if constexpr (kMixed<T>) return ce[n * nc + c];
    T vx = w[IVX * nc + c], vy = w[IVY * nc + c], vz = w[IVZ * nc + c];
    T bx1 = bc[c], by1 = bc[nc + c], bz1 = bc[2 * nc + c];
    if (n == 0) return vz * by1 - vy * bz1;
    if (n == 1) return vx * bz1 - vz * bx1;
    return vy * bx1 - vx * by1;
  };
  const int64_t n1 = SNC ? S * S * (S + 1) : g.nf1, n2 = SNC ? S * S * (S + 1) : g.nf2,
                n3 = SNC ? S * S * (S + 1) : g.nf3;
  const T* F1 = p.flx[0] + (int64_t)b * 8 * n1 + q1;
  const T* F2 = p.flx[1] + (int64_t)b * 8 * n2 + q2;
  const T* F3 = p.flx[2] + (int64_t)b * 8 * n3 + c0;
  // face EMFs: x1 faces carry (e3, e2), x2 faces (e1, e3), x3 faces (e2, e1)
  auto o1 = [&](int dk, int dj, int di) { return dk * k1 + dj * j1 + di; };
  auto o2 = [&](int dk, int dj, int di) { return dk * k2 + dj * j2 + di; };
  auto o3 = [&](int dk, int dj, int di) { return dk * kc + dj * jc + di; };
  auto e3x1 = [&](int dk, int dj, int di) { return F1[5 * n1 + o1(dk, dj, di)]; };
  auto e2x1 = [&](int dk, int dj, int di) { return F1[6 * n1 + o1(dk, dj, di)]; };
  auto wx1 = [&](int dk, int dj, int di) { return F1[7 * n1 + o1(dk, dj, di)]; };
  auto e1x2 = [&](int dk, int dj, int di) { return F2[5 * n2 + o2(dk, dj, di)]; };
  auto e3x2 = [&](int dk, int dj, int di) { return F2[6 * n2 + o2(dk, dj, di)]; };
  auto wx2 = [&](int dk, int dj, int di) { return F2[7 * n2 + o2(dk, dj, di)]; };
  auto e2x3 = [&](int dk, int dj, int di) { return F3[5 * n3 + o3(dk, dj, di)]; };
  auto e1x3 = [&](int dk, int dj, int di) { return F3[6 * n3 + o3(dk, dj, di)]; };
  auto wx3 = [&](int dk, int dj, int di) { return F3[7 * n3 + o3(dk, dj, di)]; };
  const T one = T(1.0), q = T(0.25);
  const int64_t ne = SNC ? (S + 1) * (S + 1) * (S + 1) : g.ne;
  T* E = p.edge + (int64_t)b * 3 * ne;
  const int64_t ei = ((int64_t)k * (nc2 + 1) + j) * (nc1 + 1) + i;
  {
    T de1_l3 = (one - wx2(-1, 0, 0)) * (e1x3(0, 0, 0) - cce(0, -1, 0, 0)) +
               (wx2(-1, 0, 0)) * (e1x3(0, -1, 0) - cce(0, -1, -1, 0));
    T de1_r3 = (one - wx2(0, 0, 0)) * (e1x3(0, 0, 0) - cce(0, 0, 0, 0)) +
               (wx2(0, 0, 0)) * (e1x3(0, -1, 0) - cce(0, 0, -1, 0));
    T de1_l2 = (one - wx3(0, -1, 0)) * (e1x2(0, 0, 0) - cce(0, 0, -1, 0)) +
               (wx3(0, -1, 0)) * (e1x2(-1, 0, 0) - cce(0, -1, -1, 0));
    T de1_r2 = (one - wx3(0, 0, 0)) * (e1x2(0, 0, 0) - cce(0, 0, 0, 0)) +
               (wx3(0, 0, 0)) * (e1x2(-1, 0, 0) - cce(0, -1, 0, 0));
    E[ei] = q * (de1_l3 + de1_r3 + de1_l2 + de1_r2 + e1x2(-1, 0, 0) +
                 e1x2(0, 0, 0) + e1x3(0, -1, 0) + e1x3(0, 0, 0));
  }
  {
    T de2_l3 = (one - wx1(-1, 0, 0)) * (e2x3(0, 0, 0) - cce(1, -1, 0, 0)) +
               (wx1(-1, 0, 0)) * (e2x3(0, 0, -1) - cce(1, -1, 0, -1));
    T de2_r3 = (one - wx1(0, 0, 0)) * (e2x3(0, 0, 0) - cce(1, 0, 0, 0)) +
               (wx1(0, 0, 0)) * (e2x3(0, 0, -1) - cce(1, 0, 0, -1));
    T de2_l1 = (one - wx3(0, 0, -1)) * (e2x1(0, 0, 0) - cce(1, 0, 0, -1)) +
               (wx3(0, 0, -1)) * (e2x1(-1, 0, 0) - cce(1, -1, 0, -1));
    T de2_r1 = (one - wx3(0, 0, 0)) * (e2x1(0, 0, 0) - cce(1, 0, 0, 0)) +
               (wx3(0, 0, 0)) * (e2x1(-1, 0, 0) - cce(1, -1, 0, 0));
    E[ne + ei] = q * (de2_l3 + de2_r3 + de2_l1 + de2_r1 + e2x3(0, 0, -1) +
                        e2x3(0, 0, 0) + e2x1(-1, 0, 0) + e2x1(0, 0, 0));
  }
  {
    T de3_l2 = (one - wx1(0, -1, 0)) * (e3x2(0, 0, 0) - cce(2, 0, -1, 0)) +
               (wx1(0, -1, 0)) * (e3x2(0, 0, -1) - cce(2, 0, -1, -1));
    T de3_r2 = (one - wx1(0, 0, 0)) * (e3x2(0, 0, 0) - cce(2, 0, 0, 0)) +
               (wx1(0, 0, 0)) * (e3x2(0, 0, -1) - cce(2, 0, 0, -1));
    T de3_l1 = (one - wx2(0, 0, -1)) * (e3x1(0, 0, 0) - cce(2, 0, 0, -1)) +
               (wx2(0, 0, -1)) * (e3x1(0, -1, 0) - cce(2, 0, -1, -1));
    T de3_r1 = (one - wx2(0, 0, 0)) * (e3x1(0, 0, 0) - cce(2, 0, 0, 0)) +
               (wx2(0, 0, 0)) * (e3x1(0, -1, 0) - cce(2, 0, -1, 0));
    E[2 * ne + ei] = q * (de3_l1 + de3_r1 + de3_l2 + de3_r2 + e3x2(0, 0, -1) +
                            e3x2(0, 0, 0) + e3x1(0, -1, 0) + e3x1(0, 0, 0));
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
  if constexpr (kMixed<T>) {
    // Mixed path. Every face flux enters the update pre-multiplied by the FP32 weight
    // beta dt / dx (the same rounded value in both neighbouring cells), the six weighted
    // fluxes of a cell are summed without rounding error into a pair hi + lo, and only
    // the final U - (hi + lo) runs in FP64. The face fields take the same route with
    // edge-integrated EMFs (beta dt dx_e E), so each face's flux change is an exact sum
    // of shared edge values and div B stays at FP64 round-off.
    // Every input is loaded before the first store (restrict-qualified, read-only path),
    // so a thread keeps all its ~50 loads in flight at once.
    const MixedGeo mg = p.mg[b];
    const float wf = __fmul_rn(sw.betaf, __ldg(p.dtT));
    const bool cell = (i <= g.ie && j <= g.je && k <= g.ke);
    const int64_t nc = g.ncell;
    double* __restrict__ u = p.u + (int64_t)b * NHYD * nc;
    double* __restrict__ u1 = p.u1 + (int64_t)b * NHYD * nc;
    const int64_t c = cidx(g, k, j, i);
    float fx[NHYD][6];
    double uo[NHYD], ro[NHYD];
    if (cell) {
      constexpr int NF = MHD ? 8 : 5;
      const T* __restrict__ F1 = p.flx[0] + (int64_t)b * NF * g.nf1;
      const T* __restrict__ F2 = p.flx[1] + (int64_t)b * NF * g.nf2;
      const T* __restrict__ F3 = p.flx[2] + (int64_t)b * NF * g.nf3;
      const int64_t q1 = f1idx(g, k, j, i), q2 = f2idx(g, k, j, i), q3 = f3idx(g, k, j, i);
      const int64_t s2 = g.nc1, s3 = (int64_t)g.nc1 * g.nc2;
#pragma unroll
      for (int n = 0; n < NHYD; ++n) {
        fx[n][0] = __ldg(F1 + n * g.nf1 + q1 + 1);
        fx[n][1] = __ldg(F1 + n * g.nf1 + q1);
        fx[n][2] = __ldg(F2 + n * g.nf2 + q2 + s2);
        fx[n][3] = __ldg(F2 + n * g.nf2 + q2);
        fx[n][4] = __ldg(F3 + n * g.nf3 + q3 + s3);
        fx[n][5] = __ldg(F3 + n * g.nf3 + q3);
        uo[n] = u[n * nc + c];
        ro[n] = (sw.copy_reg || sw.zero_reg) ? 0.0 : u1[n * nc + c];
      }
    }
    // face fields: base values and the four edge EMFs of each face
    double bo[3] = {0.0, 0.0, 0.0}, rb[3] = {0.0, 0.0, 0.0};
    float ed[3][4];
    int64_t qf[3] = {0, 0, 0};
    bool own[3] = {false, false, false};
    if constexpr (MHD) {
      const T* __restrict__ E1 = p.edge + (int64_t)b * 3 * g.ne;
      const T* __restrict__ E2 = E1 + g.ne;
      const T* __restrict__ E3 = E2 + g.ne;
      const int64_t e = eidx(g, k, j, i);
      const int64_t ej = (int64_t)g.nc1 + 1, ek = ((int64_t)g.nc1 + 1) * (g.nc2 + 1);
      own[0] = (j <= g.je && k <= g.ke);
      own[1] = (i <= g.ie && k <= g.ke);
      own[2] = (i <= g.ie && j <= g.je);
      qf[0] = (int64_t)b * g.nf1 + f1idx(g, k, j, i);
      qf[1] = (int64_t)b * g.nf2 + f2idx(g, k, j, i);
      qf[2] = (int64_t)b * g.nf3 + f3idx(g, k, j, i);
      double* __restrict__ bb[3] = {p.b1, p.b2, p.b3};
      double* __restrict__ rr[3] = {p.r1, p.r2, p.r3};
      // dPhi1 = (eps3(j) - eps3(j+1)) + (eps2(k+1) - eps2(k))
      // dPhi2 = (eps3(i+1) - eps3(i)) + (eps1(k) - eps1(k+1))
      // dPhi3 = (eps2(i) - eps2(i+1)) + (eps1(j+1) - eps1(j))
      const T* __restrict__ ea[3][2] = {{E3, E2}, {E3, E1}, {E2, E1}};
      const int64_t eo[3][4] = {{e, e + ej, e + ek, e}, {e + 1, e, e, e + ek},
                                {e, e + 1, e + ej, e}};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if (!own[d]) continue;
        bo[d] = bb[d][qf[d]];
        rb[d] = (sw.copy_reg || sw.zero_reg) ? 0.0 : rr[d][qf[d]];
        ed[d][0] = __ldg(ea[d][0] + eo[d][0]);
        ed[d][1] = __ldg(ea[d][0] + eo[d][1]);
        ed[d][2] = __ldg(ea[d][1] + eo[d][2]);
        ed[d][3] = __ldg(ea[d][1] + eo[d][3]);
      }
    }
    auto base_of = [&](double vo, double& r) -> double {
      if (sw.copy_reg) {  // first stage: register = state exactly
        r = vo;
        return sw.swap ? vo : sw.g1 * vo + sw.g2 * vo;
      }
      if (sw.has_delta) r += sw.delta * vo;
      return sw.swap ? r : sw.g1 * vo + sw.g2 * r;
    };
    if (cell) {
      const float cw1 = __fmul_rn(wf, mg.idx[0]), cw2 = __fmul_rn(wf, mg.idx[1]),
                  cw3 = __fmul_rn(wf, mg.idx[2]);
#pragma unroll
      for (int n = 0; n < NHYD; ++n) {
        double r = ro[n];
        const double base = base_of(uo[n], r);
        if (sw.copy_reg || sw.has_delta) u1[n * nc + c] = r;
        float hi, lo;
        sum3diff(__fmul_rn(cw1, fx[n][0]), __fmul_rn(cw1, fx[n][1]),
                 __fmul_rn(cw2, fx[n][2]), __fmul_rn(cw2, fx[n][3]),
                 __fmul_rn(cw3, fx[n][4]), __fmul_rn(cw3, fx[n][5]), hi, lo);
        u[n * nc + c] = (base - f2d_int(hi)) - f2d_int(lo);
      }
    }
    if constexpr (MHD) {
      const float we[3] = {__fmul_rn(wf, mg.dx[0]), __fmul_rn(wf, mg.dx[1]),
                           __fmul_rn(wf, mg.dx[2])};
      // the EMF component of each term: face 1 uses (e3, e2), face 2 (e3, e1), face 3 (e2, e1)
      const int comp[3][2] = {{2, 1}, {2, 0}, {1, 0}};
      double* __restrict__ bb[3] = {p.b1, p.b2, p.b3};
      double* __restrict__ rr[3] = {p.r1, p.r2, p.r3};
#pragma unroll
      for (int d = 0; d < 3; ++d) {
        if (!own[d]) continue;
        double r = rb[d];
        const double v = base_of(bo[d], r);
        if (sw.copy_reg || sw.has_delta) rr[d][qf[d]] = r;
        const float wa = we[comp[d][0]], wb = we[comp[d][1]];
        float hi, lo;
        sum2diff(__fmul_rn(wa, ed[d][0]), __fmul_rn(wa, ed[d][1]), __fmul_rn(wb, ed[d][2]),
                 __fmul_rn(wb, ed[d][3]), hi, lo);
        bb[d][qf[d]] = fma(f2d_int(lo), mg.ia[d], fma(f2d_int(hi), mg.ia[d], v));
      }
    }
  } else {
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
      const T* E1 = p.edge + (int64_t)b * 3 * g.ne;
      const T* E2 = E1 + g.ne;
      const T* E3 = E2 + g.ne;
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
}

// Conserved -> primitive with floors over every cell of every block (interior and
// ghosts). Reference src/eos/adiabatic_mhd.cpp:41-90 (adiabatic_hydro.cpp:39-81) and the
// uniform cell-centred field average of src/field/field.cpp:112-180. The EOS arithmetic
// is FP64 in both paths; W and bcc are stored as T.
template <typename T, bool MHD>
__global__ void __launch_bounds__(256) k_c2p(Geom g, StagePtrs<T> p, Box bx, Phys ph) {
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  if constexpr (kMixed<T>) {
    // Mixed path. The FP64 state is split exactly (integer pipe) into double-float pairs
    // and the internal energy E - m^2/2d - B^2/2 is formed in double-float arithmetic on
    // the FP32 pipe (relative error ~1e-13 of E, the class of the FP64 formula), so no
    // FP64 instruction runs outside the floor branches. Density is floored in place,
    // energy only where the pressure floor acts (the values the reference writes).
    const int64_t nc = g.ncell;
    const int64_t c = cidx(g, k, j, i);
    double* __restrict__ u = p.u + (int64_t)b * NHYD * nc;
    float* __restrict__ w = p.w + (int64_t)b * NHYD * nc;
    // the conserved state first: its loads are issued before any store of this thread
    double ud = u[c];
    const double m1 = u[nc + c], m2 = u[2 * nc + c], m3 = u[3 * nc + c], ue = u[4 * nc + c];
    ff ss = {0.0f, 0.0f};  // (2 Bcc)^2
    if constexpr (MHD) {
      const double* __restrict__ b1 = p.b1 + (int64_t)b * g.nf1;
      const double* __restrict__ b2 = p.b2 + (int64_t)b * g.nf2;
      const double* __restrict__ b3 = p.b3 + (int64_t)b * g.nf3;
      const int64_t q1 = f1idx(g, k, j, i), q2 = f2idx(g, k, j, i), q3 = f3idx(g, k, j, i);
      const ff f1 = split_ff(__ldg(b1 + q1)), f2 = split_ff(__ldg(b2 + q2)),
               f3 = split_ff(__ldg(b3 + q3));
      const ff s1 = ff_add(f1, split_ff(__ldg(b1 + q1 + 1)));
      const ff s2 = ff_add(f2, split_ff(__ldg(b2 + q2 + g.nc1)));
      const ff s3 = ff_add(f3, split_ff(__ldg(b3 + q3 + (int64_t)g.nc1 * g.nc2)));
      float* bcc = p.bcc + (int64_t)b * 3 * nc;
      bcc[c] = 0.5f * ff_f(s1);
      bcc[nc + c] = 0.5f * ff_f(s2);
      bcc[2 * nc + c] = 0.5f * ff_f(s3);
      // FP32 copy of the lower faces of this cell for the flux kernels; every face index
      // the sweeps read (< nc along the normal) is the lower face of some cell
      p.bfw[0][(int64_t)b * g.nf1 + q1] = f1.hi;
      p.bfw[1][(int64_t)b * g.nf2 + q2] = f2.hi;
      p.bfw[2][(int64_t)b * g.nf3 + q3] = f3.hi;
      ss = ff_add(ff_add(ff_sqr(s1), ff_sqr(s2)), ff_sqr(s3));
    }
    // ud > dfloor on the bit patterns (dfloor > 0; negative, zero and NaN densities floor)
    const uint64_t ub = bits_d(ud);
    if (!((ub >> 63) == 0 && ub > bits_d(ph.dfloor) && ub <= 0x7ff0000000000000ull)) {
      ud = ph.dfloor;
      u[c] = ud;
    }
    const ff dd = split_ff(ud), mx1 = split_ff(m1), mx2 = split_ff(m2), mx3 = split_ff(m3);
    const ff di = ff_recip(dd);
    const ff mm = ff_add(ff_add(ff_sqr(mx1), ff_sqr(mx2)), ff_sqr(mx3));
    ff x = ff_mul(mm, di);  // 2 (e_k + p_B)
    if constexpr (MHD) x = ff_add(x, ff_scale(ss, 0.25f));
    const ff wp = ff_mul(ff_sub(split_ff(ue), ff_scale(x, 0.5f)), ph.gm1f);
    float pf;
    if (!ff_gt(wp, ph.pfloorf)) {
      u[4 * nc + c] = (ph.pfloor / ph.gm1) + 0.5 * (f2d_int(x.hi) + f2d_int(x.lo));
      pf = d2f_int(ph.pfloor);
    } else {
      pf = ff_f(wp);
    }
    const float dif = ff_f(di);
    const float vx = mx1.hi * dif, vy = mx2.hi * dif, vz = mx3.hi * dif;
    w[c] = dd.hi;
    w[nc + c] = vx;
    w[2 * nc + c] = vy;
    w[3 * nc + c] = vz;
    w[4 * nc + c] = pf;
    if constexpr (MHD) {
      // cell-centred EMF of field/calculate_corner_e.cpp:135-200 for the corner kernel
      const float* bcc = p.bcc + (int64_t)b * 3 * nc;
      const float bx = bcc[c], by = bcc[nc + c], bz = bcc[2 * nc + c];
      float* ce = p.cce + (int64_t)b * 3 * nc;
      ce[c] = vz * by - vy * bz;
      ce[nc + c] = vx * bz - vz * bx;
      ce[2 * nc + c] = vy * bx - vx * by;
    }
    return;
  } else {
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
      const double f1 = b1[f1idx(g, k, j, i)], f2 = b2[f2idx(g, k, j, i)], f3 = b3[f3idx(g, k, j, i)];
      double bc1 = 0.5 * f1 + 0.5 * b1[f1idx(g, k, j, i + 1)];
      double bc2 = 0.5 * f2 + 0.5 * b2[f2idx(g, k, j + 1, i)];
      double bc3 = 0.5 * f3 + 0.5 * b3[f3idx(g, k + 1, j, i)];
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
}

// ---------------------------------------------------------------------------------------
// Mixed VL2 stage update with the primitive recovery of the interior fused in.
// Both VL2 stages start from the state at the beginning of the cycle (stage 1: the
// register is a copy of it; stage 2: the swap makes the register the base), so the state
// is read from `in` and the new state written to `out`, and the two buffers trade places
// after each cycle: no register copy, and no thread reads a value another thread writes.
// Each thread updates its cell and the six faces around it (upper faces are recomputed by
// the neighbouring thread, identically; a face is stored only by the cell it lies below,
// or by the block's last cell along its axis), then recovers W, bcc, the FP32 face copies
// and the cell-centred EMF from the values in registers. The arithmetic is that of
// k_update and k_c2p in the mixed path.
struct StateBufs {
  const double* u_in;
  const double* b_in[3];
  double* u_out;
  double* b_out[3];
};

// (a.hi + a.lo) - (b.hi + b.lo) rounded to binary32: TwoSum of the leading parts, so the
// difference of two nearby FP64 potentials keeps its FP32 precision
__device__ __forceinline__ float pair_diff(float2 a, float2 b) {
  float s, e;
  two_sum(a.x, -b.x, s, e);
  return s + (e + (a.y - b.y));
}

// One cell of k_update_c2p; returns the cell's CFL time step (new_blockdt.cpp:58-158,
// as k_block_dt computes it) when DT, so the last stage folds the time-step kernel in.
// SG: the self-gravity source (hydro/srcterms/self_gravity.cpp:35-125) joins the
// momentum and energy increments before they reach the FP64 state: momentum from the
// potential differences times the stage-start density, energy from this stage's mass
// fluxes. phi2 holds the potential as FP32 pairs hi + lo (one ghost layer), so the
// differences take no FP64 instructions.
template <bool MHD, bool DT, bool SG, int SNC>
__device__ __forceinline__ float update_c2p_cell(const Geom& g, const StagePtrs<float>& p,
                                                 int i, int j, int k, int b, const StageW& sw,
                                                 const Phys& ph, const StateBufs& sb,
                                                 const float2* __restrict__ phi2) {
  const MixedGeo mg = p.mg[b];
  const float wf = __fmul_rn(sw.betaf, __ldg(p.dtT));
  const BlockDims<SNC> d(g);
  const int64_t nc = d.ncell;
  const int64_t c = d.cell(k, j, i);
  const double* __restrict__ uin = sb.u_in + (int64_t)b * NHYD * nc;
  double* __restrict__ uout = sb.u_out + (int64_t)b * NHYD * nc;
  constexpr int NF = MHD ? 8 : 5;
  const float* __restrict__ F1 = p.flx[0] + (int64_t)b * NF * d.nf1;
  const float* __restrict__ F2 = p.flx[1] + (int64_t)b * NF * d.nf2;
  const float* __restrict__ F3 = p.flx[2] + (int64_t)b * NF * d.nf3;
  const int64_t q1 = d.f1(k, j, i), q2 = d.f2(k, j, i), q3 = c;
  const int64_t s2 = d.nc1, s3 = d.nc1 * d.nc2;
  const float cw1 = __fmul_rn(wf, mg.idx[0]), cw2 = __fmul_rn(wf, mg.idx[1]),
              cw3 = __fmul_rn(wf, mg.idx[2]);
  float* __restrict__ w = p.w + (int64_t)b * NHYD * nc;
  float sgs[NHYD] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};  // source terms, subtracted below
  if constexpr (SG) {
    // first, while few values are live: the density the stage's fluxes were computed
    // from (this thread's own cell of W, read before it is overwritten below), the
    // potential differences and the mass fluxes of the six faces
    const float rho = w[c];
    const float2* __restrict__ pp = phi2 + (int64_t)b * nc;
    const float2 pc = __ldg(pp + c);
    const int64_t sd[3] = {1, s2, s3};
    const float cwd[3] = {cw1, cw2, cw3};
    const float* __restrict__ Fd[3] = {F1 + q1, F2 + q2, F3 + q3};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float dl = pair_diff(pc, __ldg(pp + c - sd[a]));
      const float dr = pair_diff(__ldg(pp + c + sd[a]), pc);
      sgs[1 + a] = cwd[a] * rho * (0.5f * (dl + dr));
      sgs[4] += cwd[a] * (0.5f * (__ldg(Fd[a]) * dl + __ldg(Fd[a] + sd[a]) * dr));
    }
  }
  float fx[NHYD][6];
  double uo[NHYD];
#pragma unroll
  for (int n = 0; n < NHYD; ++n) {
    fx[n][0] = __ldg(F1 + n * d.nf1 + q1 + 1);
    fx[n][1] = __ldg(F1 + n * d.nf1 + q1);
    fx[n][2] = __ldg(F2 + n * d.nf2 + q2 + s2);
    fx[n][3] = __ldg(F2 + n * d.nf2 + q2);
    fx[n][4] = __ldg(F3 + n * d.nf3 + q3 + s3);
    fx[n][5] = __ldg(F3 + n * d.nf3 + q3);
    uo[n] = __ldg(uin + n * nc + c);
  }
  // faces (lower, upper) per direction, base values and edge EMFs
  double bl[3] = {0.0, 0.0, 0.0}, bu[3] = {0.0, 0.0, 0.0};
  float E1[2][2], E2[2][2], E3[2][2];  // E1[dk][dj], E2[dk][di], E3[dj][di]
  int64_t fl[3] = {0, 0, 0}, fu[3] = {0, 0, 0};
  if constexpr (MHD) {
    fl[0] = (int64_t)b * d.nf1 + q1;      fu[0] = fl[0] + 1;
    fl[1] = (int64_t)b * d.nf2 + q2;      fu[1] = fl[1] + d.nc1;
    fl[2] = (int64_t)b * d.nf3 + q3;      fu[2] = fl[2] + d.nc1 * d.nc2;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      bl[d] = __ldg(sb.b_in[d] + fl[d]);
      bu[d] = __ldg(sb.b_in[d] + fu[d]);
    }
    const float* __restrict__ Ea = p.edge + (int64_t)b * 3 * d.ne;
    const int64_t e = d.edge(k, j, i);
    const int64_t ej = d.nc1 + 1, ek = (d.nc1 + 1) * (d.nc2 + 1);
#pragma unroll
    for (int x = 0; x < 2; ++x)
#pragma unroll
      for (int y = 0; y < 2; ++y) {
        E1[x][y] = __ldg(Ea + e + x * ek + y * ej);
        E2[x][y] = __ldg(Ea + d.ne + e + x * ek + y);
        E3[x][y] = __ldg(Ea + 2 * d.ne + e + x * ej + y);
      }
  }
  // conserved update (base = the state at the start of the cycle)
  double un[NHYD];
#pragma unroll
  for (int n = 0; n < NHYD; ++n) {
    float hi, lo;
    sum3diff(__fmul_rn(cw1, fx[n][0]), __fmul_rn(cw1, fx[n][1]), __fmul_rn(cw2, fx[n][2]),
             __fmul_rn(cw2, fx[n][3]), __fmul_rn(cw3, fx[n][4]), __fmul_rn(cw3, fx[n][5]), hi, lo);
    if (SG && n > 0) {
      float e;
      two_sum(hi, sgs[n], hi, e);
      lo += e;
    }
    un[n] = (uo[n] - f2d_int(hi)) - f2d_int(lo);
  }
  ff ss = {0.0f, 0.0f};
  float* __restrict__ bcc = p.bcc + (int64_t)b * 3 * nc;
  float fl32[3] = {0.0f, 0.0f, 0.0f};  // FP32 copies of the lower faces
  if constexpr (MHD) {
    const float we1 = __fmul_rn(wf, mg.dx[0]), we2 = __fmul_rn(wf, mg.dx[1]),
                we3 = __fmul_rn(wf, mg.dx[2]);
    auto upd = [&](double base, float a, float b0, float c0, float d0, float wa, float wb,
                   double ia) {
      float hi, lo;
      sum2diff(__fmul_rn(wa, a), __fmul_rn(wa, b0), __fmul_rn(wb, c0), __fmul_rn(wb, d0), hi, lo);
      return fma(f2d_int(lo), ia, fma(f2d_int(hi), ia, base));
    };
    // dPhi1 = (eps3(j) - eps3(j+1)) + (eps2(k+1) - eps2(k)) at i and i+1
    const double n1l = upd(bl[0], E3[0][0], E3[1][0], E2[1][0], E2[0][0], we3, we2, mg.ia[0]);
    const double n1u = upd(bu[0], E3[0][1], E3[1][1], E2[1][1], E2[0][1], we3, we2, mg.ia[0]);
    // dPhi2 = (eps3(i+1) - eps3(i)) + (eps1(k) - eps1(k+1)) at j and j+1
    const double n2l = upd(bl[1], E3[0][1], E3[0][0], E1[0][0], E1[1][0], we3, we1, mg.ia[1]);
    const double n2u = upd(bu[1], E3[1][1], E3[1][0], E1[0][1], E1[1][1], we3, we1, mg.ia[1]);
    // dPhi3 = (eps2(i) - eps2(i+1)) + (eps1(j+1) - eps1(j)) at k and k+1
    const double n3l = upd(bl[2], E2[0][0], E2[0][1], E1[0][1], E1[0][0], we2, we1, mg.ia[2]);
    const double n3u = upd(bu[2], E2[1][0], E2[1][1], E1[1][1], E1[1][0], we2, we1, mg.ia[2]);
    const ff f1 = split_ff(n1l), f2 = split_ff(n2l), f3 = split_ff(n3l);
    sb.b_out[0][fl[0]] = n1l;
    sb.b_out[1][fl[1]] = n2l;
    sb.b_out[2][fl[2]] = n3l;
    p.bfw[0][fl[0]] = f1.hi;
    p.bfw[1][fl[1]] = f2.hi;
    p.bfw[2][fl[2]] = f3.hi;
    fl32[0] = f1.hi; fl32[1] = f2.hi; fl32[2] = f3.hi;
    const ff u1f = split_ff(n1u), u2f = split_ff(n2u), u3f = split_ff(n3u);
    if (i == g.ie) { sb.b_out[0][fu[0]] = n1u; p.bfw[0][fu[0]] = u1f.hi; }
    if (j == g.je) { sb.b_out[1][fu[1]] = n2u; p.bfw[1][fu[1]] = u2f.hi; }
    if (k == g.ke) { sb.b_out[2][fu[2]] = n3u; p.bfw[2][fu[2]] = u3f.hi; }
    const ff s1 = ff_add(f1, u1f), s2f = ff_add(f2, u2f), s3f = ff_add(f3, u3f);
    bcc[c] = 0.5f * ff_f(s1);
    bcc[nc + c] = 0.5f * ff_f(s2f);
    bcc[2 * nc + c] = 0.5f * ff_f(s3f);
    ss = ff_add(ff_add(ff_sqr(s1), ff_sqr(s2f)), ff_sqr(s3f));
  }
  // primitive recovery (the mixed k_c2p)
  double ud = un[0];
  const uint64_t ub = bits_d(ud);
  if (!((ub >> 63) == 0 && ub > bits_d(ph.dfloor) && ub <= 0x7ff0000000000000ull)) ud = ph.dfloor;
  const ff dd = split_ff(ud), mx1 = split_ff(un[1]), mx2 = split_ff(un[2]), mx3 = split_ff(un[3]);
  const ff di = ff_recip(dd);
  const ff mm = ff_add(ff_add(ff_sqr(mx1), ff_sqr(mx2)), ff_sqr(mx3));
  ff x = ff_mul(mm, di);
  if constexpr (MHD) x = ff_add(x, ff_scale(ss, 0.25f));
  const ff wp = ff_mul(ff_sub(split_ff(un[4]), ff_scale(x, 0.5f)), ph.gm1f);
  double ue = un[4];
  float pf;
  if (!ff_gt(wp, ph.pfloorf)) {
    ue = (ph.pfloor / ph.gm1) + 0.5 * (f2d_int(x.hi) + f2d_int(x.lo));
    pf = d2f_int(ph.pfloor);
  } else {
    pf = ff_f(wp);
  }
  uout[c] = ud;
  uout[nc + c] = un[1];
  uout[2 * nc + c] = un[2];
  uout[3 * nc + c] = un[3];
  uout[4 * nc + c] = ue;
  const float dif = ff_f(di);
  const float vx = mx1.hi * dif, vy = mx2.hi * dif, vz = mx3.hi * dif;
  w[c] = dd.hi;
  w[nc + c] = vx;
  w[2 * nc + c] = vy;
  w[3 * nc + c] = vz;
  w[4 * nc + c] = pf;
  float bx = 0.0f, by = 0.0f, bz = 0.0f;
  if constexpr (MHD) {
    bx = bcc[c]; by = bcc[nc + c]; bz = bcc[2 * nc + c];
    float* __restrict__ ce = p.cce + (int64_t)b * 3 * nc;
    ce[c] = vz * by - vy * bz;
    ce[nc + c] = vx * bz - vz * bx;
    ce[2 * nc + c] = vy * bx - vx * by;
  }
  if constexpr (DT) {
    const float dx1 = p.dxT[b * 3], dx2 = p.dxT[b * 3 + 1], dx3 = p.dxT[b * 3 + 2];
    const float gam = ph.gammas, d = dd.hi;
    float dt1, dt2, dt3;
    if constexpr (MHD) {
      float cf = fast_speed<float>(d, pf, by, bz, bx + fabsf(fl32[0] - bx), gam);
      dt1 = dx1 / (fabsf(vx) + cf);
      cf = fast_speed<float>(d, pf, bz, bx, by + fabsf(fl32[1] - by), gam);
      dt2 = dx2 / (fabsf(vy) + cf);
      cf = fast_speed<float>(d, pf, bx, by, bz + fabsf(fl32[2] - bz), gam);
      dt3 = dx3 / (fabsf(vz) + cf);
    } else {
      const float cs = sqrtf(gam * pf / d);
      dt1 = dx1 / (fabsf(vx) + cs);
      dt2 = dx2 / (fabsf(vy) + cs);
      dt3 = dx3 / (fabsf(vz) + cs);
    }
    return mn(mn(mn(3.402823466e38f, dt1), dt2), dt3);
  }
  return 3.402823466e38f;
}

// Seven blocks of 128 per SM: up to 73 registers a thread. On a GB300 at 256^3 that ran
// 1.027 / 1.069 ms per launch (without / with the time step) against 1.097 / 1.152 ms with
// eight blocks and 64 registers, where the kernel spilled.
template <bool MHD, bool DT, bool SG, int SNC>
__global__ void __launch_bounds__(128, 7)
k_update_c2p(Geom g, StagePtrs<float> p, Box bx, StageW sw, Phys ph, StateBufs sb,
             unsigned long long* dtmin, const float2* __restrict__ phi2) {
  int i, j, k, b;
  const bool active = box_coords(bx, i, j, k, b);
  float mindt = 3.402823466e38f;
  if (active) mindt = update_c2p_cell<MHD, DT, SG, SNC>(g, p, i, j, k, b, sw, ph, sb, phi2);
  if constexpr (DT) {  // block minimum, then one 64-bit atomicMin (as k_block_dt)
    for (int o = 16; o > 0; o >>= 1) mindt = mn(mindt, __shfl_xor_sync(0xffffffffu, mindt, o));
    __shared__ float red[32];
    const int tid = threadIdx.x;
    if ((tid & 31) == 0) red[tid >> 5] = mindt;
    __syncthreads();
    if (tid < 32) {
      float v = (tid < (int)((blockDim.x + 31) / 32)) ? red[tid] : 3.402823466e38f;
      for (int o = 16; o > 0; o >>= 1) v = mn(v, __shfl_xor_sync(0xffffffffu, v, o));
      if (tid == 0) {
        const double vd = (v == 3.402823466e38f) ? 1.79769313486231570815e308 : f2d_int(v);
        atomicMin(dtmin, (unsigned long long)__double_as_longlong(vd));
      }
    }
  }
}

// Self-gravity source (hydro/srcterms/self_gravity.cpp:35-125): momentum from the face
// potentials, energy from the mass fluxes of this stage, applied after the flux
// divergence with the stage weight beta dt. phi is the block pool's potential (one ghost
// layer filled from the multigrid solution). The FP64 path keeps the reference's order
// (x1, x2, x3 passes, each a read-modify-write of U); the mixed path forms the potential
// differences in FP64 and the products in FP32.
template <typename T, bool MHD>
__global__ void __launch_bounds__(128)
k_self_gravity(Geom g, StagePtrs<T> p, Box bx, StageW sw, const double* __restrict__ phi_pool) {
  constexpr int NF = MHD ? 8 : 5;
  int i, j, k, b;
  if (!box_coords(bx, i, j, k, b)) return;
  const int64_t nc = g.ncell;
  const int64_t c = cidx(g, k, j, i);
  double* u = p.u + (int64_t)b * NHYD * nc;
  const T* w = p.w + (int64_t)b * NHYD * nc;
  const double* phi = phi_pool + (int64_t)b * nc;
  const T* F1 = p.flx[0] + (int64_t)b * NF * g.nf1;
  const T* F2 = p.flx[1] + (int64_t)b * NF * g.nf2;
  const T* F3 = p.flx[2] + (int64_t)b * NF * g.nf3;
  const int64_t st[3] = {1, (int64_t)g.nc1, (int64_t)g.nc1 * g.nc2};
  const int64_t fl[3] = {f1idx(g, k, j, i), f2idx(g, k, j, i), f3idx(g, k, j, i)};
  const int64_t fr[3] = {f1idx(g, k, j, i + 1), f2idx(g, k, j + 1, i), f3idx(g, k + 1, j, i)};
  const T* F[3] = {F1, F2, F3};
  if constexpr (kMixed<T>) {
    const MixedGeo mg = p.mg[b];
    const float wf = __fmul_rn(sw.betaf, *p.dtT);
    const float rho = w[c];
    float de = 0.0f;
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const float dtodx = wf * mg.idx[d];
      const float dl = d2f_int(phi[c] - phi[c - st[d]]);
      const float dr = d2f_int(phi[c + st[d]] - phi[c]);
      const float dm = dtodx * rho * (0.5f * (dl + dr));
      u[(1 + d) * nc + c] -= f2d_int(dm);
      de += dtodx * (0.5f * (F[d][fl[d]] * dl + F[d][fr[d]] * dr));
    }
    u[4 * nc + c] -= f2d_int(de);
  } else {
    const double dt = sw.beta * (*p.dt);
    const BlockGeo geo = p.geo[b];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const double dtodx = dt / geo.dx[d];
      const double phic = phi[c];
      const double phil = 0.5 * (phi[c - st[d]] + phi[c]);
      const double phir = 0.5 * (phi[c] + phi[c + st[d]]);
      u[(1 + d) * nc + c] -= dtodx * w[c] * (phir - phil);
      u[4 * nc + c] -= dtodx * (F[d][fl[d]] * (phic - phil) + F[d][fr[d]] * (phir - phic));
    }
  }
}

// Per-block CFL limit (src/hydro/new_blockdt.cpp:58-158) reduced over the whole pool
// in one launch: warp-shuffle min, block min, then one 64-bit atomicMin (positive
// doubles order like their bit patterns).
template <typename T, bool MHD>
__global__ void __launch_bounds__(256)
k_block_dt(Geom g, StagePtrs<T> p, Box bx, Phys ph, unsigned long long* dtmin) {
  // the reduction runs in T: FP32 in the mixed path (relative change of dt ~1e-7)
  int i, j, k, b;
  const T kBig = kMixed<T> ? T(3.402823466e38f) : T(1.79769313486231570815e308);
  T mindt = kBig;
  if (box_coords(bx, i, j, k, b)) {
    const int64_t nc = g.ncell, c = cidx(g, k, j, i);
    const T* w = p.w + (int64_t)b * NHYD * nc;
    T d = w[c], vx = w[nc + c], vy = w[2 * nc + c], vz = w[3 * nc + c], pr = w[4 * nc + c];
    T dx1, dx2, dx3;
    if constexpr (kMixed<T>) {
      dx1 = p.dxT[b * 3]; dx2 = p.dxT[b * 3 + 1]; dx3 = p.dxT[b * 3 + 2];
    } else {
      const BlockGeo geo = p.geo[b];
      dx1 = geo.dx[0]; dx2 = geo.dx[1]; dx3 = geo.dx[2];
    }
    const T gam = ph_gamma<T>(ph);
    T dt1, dt2, dt3;
    if constexpr (MHD) {
      const T* bcc = p.bcc + (int64_t)b * 3 * nc;
      T bc1 = bcc[c], bc2 = bcc[nc + c], bc3 = bcc[2 * nc + c];
      T bx1 = bc1 + fabs(p.bf[0][(int64_t)b * g.nf1 + f1idx(g, k, j, i)] - bc1);
      T cf = fast_speed<T>(d, pr, bc2, bc3, bx1, gam);
      dt1 = dx1 / (fabs(vx) + cf);
      T bx2 = bc2 + fabs(p.bf[1][(int64_t)b * g.nf2 + f2idx(g, k, j, i)] - bc2);
      cf = fast_speed<T>(d, pr, bc3, bc1, bx2, gam);
      dt2 = dx2 / (fabs(vy) + cf);
      T bx3 = bc3 + fabs(p.bf[2][(int64_t)b * g.nf3 + f3idx(g, k, j, i)] - bc3);
      cf = fast_speed<T>(d, pr, bc1, bc2, bx3, gam);
      dt3 = dx3 / (fabs(vz) + cf);
    } else {
      T cs = sqrt(gam * pr / d);
      dt1 = dx1 / (fabs(vx) + cs);
      dt2 = dx2 / (fabs(vy) + cs);
      dt3 = dx3 / (fabs(vz) + cs);
    }
    mindt = mn(mn(mn(mindt, dt1), dt2), dt3);
  }
  for (int o = 16; o > 0; o >>= 1) mindt = mn(mindt, __shfl_xor_sync(0xffffffffu, mindt, o));
  __shared__ T red[32];
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  const int nt = blockDim.x * blockDim.y;
  if ((tid & 31) == 0) red[tid >> 5] = mindt;
  __syncthreads();
  if (tid < 32) {
    T v = (tid < (nt + 31) / 32) ? red[tid] : kBig;
    for (int o = 16; o > 0; o >>= 1) v = mn(v, __shfl_xor_sync(0xffffffffu, v, o));
    if (tid == 0) {
      const double vd = (v == kBig) ? 1.79769313486231570815e308 : (double)v;
      atomicMin(dtmin, (unsigned long long)__double_as_longlong(vd));
    }
  }
}

}  // namespace athg

// athg_single_pass.cu -- one launch per stage of the mixed-precision VL2 MHD update on a
// uniform mesh: reconstruction + Riemann fluxes of all three directions, face and corner
// EMFs, flux divergence, constrained transport and the primitive recovery of the interior,
// with every intermediate kept on chip.
//
// The reference's stage is one pass over a MeshBlock (Hydro::CalculateFluxes,
// hydro/calculate_fluxes.cpp:36-378; Field::ComputeCornerE, field/calculate_corner_e.cpp:
// 129-229; the stage tasks of task_list/time_integrator.cpp:1460-1653). The separate
// kernels of athg_stage.cuh run it as x1, x2, x3 sweeps, corner EMFs and the update, each
// round-tripping its results through HBM. Here a thread block owns a 32 x 8 column of cells
// of one block and marches it along k:
//
//   * the FP32 primitives and cell-centred field (W, bcc) of a 36 x 12 plane (the column
//     plus two ghost cells each side) arrive by TMA (cp.async.bulk.tensor, one box for the
//     five W components and one for the three bcc components) into a ring of four planes
//     in shared memory, completed on an mbarrier per slot, three planes ahead of their use;
//   * per plane step k the block solves the x1 and x2 faces of plane k+1 and the x3 faces
//     between planes k and k+1 (PLM or donor cell + HLLD/HLLE, the arithmetic of k_flux and
//     k_flux_march), forms the corner EMFs e3 of plane k+1 and e1, e2 of the face plane
//     k+1/2 (k_corner_emf's arithmetic, the cell-centred EMF recomputed from W and bcc),
//     and then updates plane k: flux divergence and CT in the exact FP32 sums of
//     k_update_c2p, FP64 state read once and written once, and W, bcc and the FP32 face
//     copies of the new state written for the next stage;
//   * the face-plane quantities shared by consecutive steps stay in shared memory (two
//     planes of face EMFs and corner EMFs) or in registers (the x3 flux and the new x3
//     face field below each cell, the x1/x2 part of each cell's flux sum).
//
// W and bcc are read from one set of FP32 arrays and written to a second set (the next
// stage reads what this one wrote, after the ghost exchange), because neighbouring thread
// blocks read a plane's halo while others write its interior.
//
// Every wait on an mbarrier is bounded: a load that does not complete sets bit 0 of the
// device error word and the block stops issuing work (no hang, no fault).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <string>

#include "athg_single_pass.h"
#include "athg_stage.cuh"

namespace athg {

namespace {

constexpr int TI = SP_TILE_I, TJ = SP_TILE_J, NT = TI * TJ;
constexpr int WI = TI + 4, WJ = TJ + 4, PL = WI * WJ;  // W box of one plane: 36 x 12
// a ring slot: the W box (5 x PL floats) then the bcc box (3 x PL floats), each padded to
// a multiple of 128 bytes (TMA destination alignment)
constexpr int W_FLOATS = ((5 * PL * 4 + 127) / 128) * 128 / 4;
constexpr int B_FLOATS = ((3 * PL * 4 + 127) / 128) * 128 / 4;
constexpr int SLOT = W_FLOATS + B_FLOATS;
constexpr int RING = 4;
constexpr uint32_t W_BYTES = 5u * PL * 4u, B_BYTES = 3u * PL * 4u;
// face sets of one plane: x1 faces i in [i0, i0+TI], rows j in [j0-1, j0+TJ];
// x2 faces columns i in [i0-1, i0+TI], j in [j0, j0+TJ]; x3 faces and the cell-centred
// EMF on the rectangle i in [i0-1, i0+TI], j in [j0-1, j0+TJ]
constexpr int N1W = TI + 1, N1H = TJ + 2, N1 = N1W * N1H;
constexpr int N2W = TI + 2, N2H = TJ + 1, N2 = N2W * N2H;
constexpr int XW = TI + 2, XH = TJ + 2, N3 = XW * XH;
constexpr int N3B = N3 - NT;             // rectangle border (not a tile column)
constexpr int NFACE = N3B + N1 + N2;     // faces of rounds after the tile's own x3 faces
constexpr int NE3 = (TI + 1) * (TJ + 1), NE1 = TI * (TJ + 1), NE2 = (TI + 1) * TJ;

struct Smem {
  float w[RING][SLOT];
  float x3l[7][N3];        // left state of the next x3 face (rotated order), per column
  float x1e[2][3][N1];     // x1 faces: e3, e2, CT weight; two planes
  float x2e[2][3][N2];     // x2 faces: e1, e3, CT weight
  float x3e[3][N3];        // x3 faces of the current face plane: e2, e1, CT weight
  float x1h[5][TJ][N1W];   // hydro fluxes of the x1 faces of the tile rows (one plane)
  float x2h[5][N2H][TI];   // hydro fluxes of the x2 faces of the tile columns
  float e1[2][TJ + 1][TI];     // corner EMFs along x1 at two face planes
  float e2[2][TJ][TI + 1];     // along x2
  float e3[2][TJ + 1][TI + 1]; // along x3 at two cell planes
  float cc[2][3][N3];          // cell-centred E = -v x B on the rectangle, two cell planes
  unsigned long long bar[RING];
};

// ---- TMA and mbarrier (inline PTX) ----------------------------------------------------
__device__ __forceinline__ uint32_t sa(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void bar_init(unsigned long long* b) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(sa(b)) : "memory");
}
__device__ __forceinline__ void fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void bar_expect(unsigned long long* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(b)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void tma_4d(void* dst, const CUtensorMap* map, unsigned long long* b,
                                       int x, int y, int z, int v) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(sa(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(v), "r"(sa(b))
      : "memory");
}
__device__ __forceinline__ bool bar_try(unsigned long long* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}" : "=r"(ok) : "r"(sa(b)), "r"(parity) : "memory");
  return ok != 0;
}
// bounded wait: false if the phase did not complete within the limit
__device__ __forceinline__ bool bar_wait(unsigned long long* b, uint32_t parity) {
  for (int it = 0; it < (1 << 20); ++it)
    if (bar_try(b, parity)) return true;
  return false;
}

// ---- per-face arithmetic ----------------------------------------------------------------
// van Leer slope of a cell from its two neighbours (plm.cpp uniform branch, as k_flux)
__device__ __forceinline__ float vl_slope(float am, float a0, float ap) {
  const float dwl = (a0 - am), dwr = (ap - a0);
  const float dw2 = dwl * dwr;
  float dwm = 2.0f * dw2 / (dwl + dwr);
  if (dw2 <= 0.0f) dwm = 0.0f;
  return dwm;
}

// source variable (0..7: W then bcc) of rotated wave variable m for a sweep along d
__device__ __forceinline__ int wave_src(int d, int m) {
  if (m == 0) return 0;
  if (m == 4) return 4;
  if (m < 4) return 1 + (d + m - 1) % 3;          // vn, vt1, vt2
  return 5 + (m == 5 ? (d + 1) % 3 : (d + 2) % 3);  // by, bz (cyclic, plm.cpp:44-55)
}

__device__ __forceinline__ const float* slot_var(const Smem& s, int slot, int v) {
  return v < 5 ? &s.w[slot][v * PL] : &s.w[slot][W_FLOATS + (v - 5) * PL];
}

// Riemann solve of one face from rotated states; fx (rotated) and the face EMFs / weight
template <int SOLVER>
__device__ __forceinline__ void solve_face(const float* wl, const float* wr, float bx, float gam,
                                           float dxd, float dt, float* fx, float* em) {
  if (SOLVER == HLLD) rs_hlld<float>(wl, wr, bx, gam, fx);
  else rs_hlle_mhd<float>(wl, wr, bx, gam, fx);
  em[0] = -fx[IBY];
  em[1] = fx[IBZ];
  em[2] = ct_weight<float>(fx[IDN], wl[IDN], wr[IDN], dxd, dt);
}

// the arithmetic of one corner EMF (k_corner_emf): a, b are the two face-EMF terms of the
// upwind integration, each (1 - w) (e - c) + w (e' - c')
__device__ __forceinline__ float up(float w, float e, float c, float e2, float c2) {
  return (1.0f - w) * (e - c) + (w) * (e2 - c2);
}

struct SpArgs {
  Geom g;
  StagePtrs<float> p;  // read set: w, bcc, bf; geometry, dt
  float* w_out;
  float* bcc_out;
  float* bf_out[3];
  StateBufs sb;
  StageW sw;
  Phys ph;
  unsigned long long* dtmin;
  unsigned int* err;
  int nseg;
};

template <int ORDER, int SOLVER, bool DT>
__global__ void __launch_bounds__(NT, 2)
k_single_pass(const __grid_constant__ CUtensorMap tw, const __grid_constant__ CUtensorMap tb,
              SpArgs A) {
  extern __shared__ unsigned char smem_raw[];
  Smem& S = *reinterpret_cast<Smem*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~(uintptr_t)127);
  const Geom& g = A.g;
  const StagePtrs<float>& p = A.p;
  const int tid = threadIdx.x;
  const int tiles_i = g.nx1 / TI;
  const int i0 = g.is + (blockIdx.x % tiles_i) * TI;   // padded index of the first column
  const int j0 = g.js + (blockIdx.x / tiles_i) * TJ;
  const int b = blockIdx.z;
  const int seg = g.nx3 / A.nseg;
  const int ks0 = g.ks + blockIdx.y * seg, ke0 = ks0 + seg - 1;
  const int p0 = ks0 - 2;                              // first plane of the ring
  const int ti = tid % TI, tj = tid / TI;              // this thread's column
  const int ci = i0 + ti, cj = j0 + tj;

  if (tid == 0) {
    for (int s = 0; s < RING; ++s) bar_init(&S.bar[s]);
    fence_init();
  }
  __syncthreads();
  auto issue = [&](int plane) {  // thread 0: TMA of plane `plane` into its slot
    const int r = plane - p0, s = r & 3;
    fence_async_smem();
    bar_expect(&S.bar[s], W_BYTES + B_BYTES);
    tma_4d(&S.w[s][0], &tw, &S.bar[s], i0 - 2, j0 - 2, plane, b * 5);
    tma_4d(&S.w[s][W_FLOATS], &tb, &S.bar[s], i0 - 2, j0 - 2, plane, b * 3);
  };
  if (tid == 0)
    for (int q = 0; q < RING; ++q) issue(p0 + q);
  bool failed = false;
  int waited = p0 - 1, issued = p0 + RING - 1;  // last plane waited for / issued
  auto wait_plane = [&](int plane) {
    const int r = plane - p0;
    const bool ok = bar_wait(&S.bar[r & 3], (uint32_t)((r >> 2) & 1));
    if (ok) waited = plane;
    if (__syncthreads_or(!ok)) {
      if (tid == 0) atomicOr(A.err, kErrTmaTimeout);
      failed = true;
    }
  };

  const float gam = ph_gamma<float>(A.ph);
  const float dtf = __ldg(p.dtT);
  const float* __restrict__ cf1 = p.coef + ((int64_t)b * 3 + 0) * 2 * g.ncmax;
  const float* __restrict__ cf2 = p.coef + ((int64_t)b * 3 + 1) * 2 * g.ncmax;
  const float* __restrict__ cf3 = p.coef + ((int64_t)b * 3 + 2) * 2 * g.ncmax;
  const float dx1 = p.dxT[b * 3], dx2 = p.dxT[b * 3 + 1], dx3 = p.dxT[b * 3 + 2];
  const float* __restrict__ bf1 = p.bf[0] + (int64_t)b * g.nf1;
  const float* __restrict__ bf2 = p.bf[1] + (int64_t)b * g.nf2;
  const float* __restrict__ bf3 = p.bf[2] + (int64_t)b * g.nf3;
  const MixedGeo mg = p.mg[b];
  const float wf = __fmul_rn(A.sw.betaf, dtf);
  const float cw1 = __fmul_rn(wf, mg.idx[0]), cw2 = __fmul_rn(wf, mg.idx[1]),
              cw3 = __fmul_rn(wf, mg.idx[2]);
  const float we1 = __fmul_rn(wf, mg.dx[0]), we2 = __fmul_rn(wf, mg.dx[1]),
              we3 = __fmul_rn(wf, mg.dx[2]);
  const int64_t nc = g.ncell;

  // carried from step to step for this thread's column
  float f3lo[NHYD];                 // x3 flux of the face below the cell (raw)
  float pt[NHYD], pe12[NHYD], pe4[NHYD];  // x1/x2 part of the cell's exact flux sum
  double b3lo = 0.0;                // new x3 face field below the cell
  float mindt = 3.402823466e38f;

  for (int k = ks0 - 2; k <= ke0 && !failed; ++k) {
    const bool pre = (k == ks0 - 2);
    const bool upd = (k >= ks0);
    // the plane three ahead goes into the slot of plane k-1, free since the last step
    if (!pre && k + 3 <= ke0 + 2) {
      if (tid == 0) issue(k + 3);
      issued = k + 3;
    }
    if (pre) { wait_plane(k); if (failed) break; wait_plane(k + 1); if (failed) break; }
    wait_plane(k + 2);
    if (failed) break;
    const int sk = (k - p0) & 3, sk1 = (k + 1 - p0) & 3, sk2 = (k + 2 - p0) & 3;
    const int pn = (k + 1) & 1, po = k & 1;  // buffers of plane / face plane k+1 and k

    // FP64 state of this thread's cell (consumed after the face and EMF phases)
    double uo[NHYD], bl1 = 0.0, bu1 = 0.0, bl2 = 0.0, bu2 = 0.0, bu3 = 0.0;
    const int64_t c = cidx(g, k, cj, ci);
    if (upd) {
      const double* __restrict__ uin = A.sb.u_in + (int64_t)b * NHYD * nc;
#pragma unroll
      for (int n = 0; n < NHYD; ++n) uo[n] = __ldg(uin + n * nc + c);
      const int64_t q1 = (int64_t)b * g.nf1 + f1idx(g, k, cj, ci);
      const int64_t q2 = (int64_t)b * g.nf2 + f2idx(g, k, cj, ci);
      const int64_t q3 = (int64_t)b * g.nf3 + f3idx(g, k + 1, cj, ci);
      bl1 = __ldg(A.sb.b_in[0] + q1); bu1 = __ldg(A.sb.b_in[0] + q1 + 1);
      bl2 = __ldg(A.sb.b_in[1] + q2); bu2 = __ldg(A.sb.b_in[1] + q2 + g.nc1);
      bu3 = __ldg(A.sb.b_in[2] + q3);
    }

    // ---- faces: round 0 the x3 face above this thread's own cell, then the rest ----
    float f3up[NHYD];
    // item -1: the x3 face above this thread's own cell; then items tid, tid + NT, ... of
    // the flat list (rectangle border x3 faces, x1 faces, x2 faces): one solver call site
    const int nit = 1 + (NFACE - tid + NT - 1) / NT;
    for (int it = 0; it < nit; ++it) {
      const int q = it == 0 ? -1 : tid + (it - 1) * NT;
      int dir, xi = 0, xj = 0;
      if (q < 0) { dir = 2; xi = ti + 1; xj = tj + 1; }
      else if (q < N3B) {
        dir = 2;
        if (q < XW) { xi = q; xj = 0; }
        else if (q < 2 * XW) { xi = q - XW; xj = XH - 1; }
        else { const int r = q - 2 * XW; xj = 1 + (r >> 1); xi = (r & 1) ? XW - 1 : 0; }
      } else if (q < N3B + N1) { dir = 0; xi = (q - N3B) % N1W; xj = (q - N3B) / N1W; }
      else { dir = 1; xi = (q - N3B - N1) % N2W; xj = (q - N3B - N1) / N2W; }
      float wl[7], wr[7], bx;
      float dxd;
      int fk, fj, fi;  // padded face index (k, j, i) of this face
      if (dir == 2) {
        // column (i0-1+xi, j0-1+xj); box coordinates (xi+1, xj+1); cell k+1's slope gives
        // the right state of face k+1 and the left state of face k+2
        fi = i0 - 1 + xi; fj = j0 - 1 + xj; fk = k + 1;
        const int o = (xj + 1) * WI + (xi + 1);
        const int r = xj * XW + xi;
        const float cmR = cf3[g.ncmax + fk], cpR = cf3[fk];
#pragma unroll
        for (int m = 0; m < 7; ++m) {
          const int v = wave_src(2, m);
          const float a0 = slot_var(S, sk1, v)[o];
          float wrm, wln;
          if (ORDER == 1) {
            wrm = a0; wln = a0;
          } else {
            const float dwm = vl_slope(slot_var(S, sk, v)[o], a0, slot_var(S, sk2, v)[o]);
            wrm = a0 - cmR * dwm;
            wln = a0 + cpR * dwm;
          }
          wl[m] = S.x3l[m][r];
          wr[m] = wrm;
          S.x3l[m][r] = wln;
        }
        {  // cell-centred E of cell k+1 of this column (the mixed k_c2p's expression)
          const float vx = slot_var(S, sk1, 1)[o], vy = slot_var(S, sk1, 2)[o],
                      vz = slot_var(S, sk1, 3)[o];
          const float bxc = slot_var(S, sk1, 5)[o], byc = slot_var(S, sk1, 6)[o],
                      bzc = slot_var(S, sk1, 7)[o];
          S.cc[pn][0][r] = vz * byc - vy * bzc;
          S.cc[pn][1][r] = vx * bzc - vz * bxc;
          S.cc[pn][2][r] = vy * bxc - vx * byc;
        }
        if (pre) continue;
        bx = __ldg(bf3 + f3idx(g, fk, fj, fi));
        dxd = dx3;
      } else {
        // in-plane faces of plane k+1: right cell at box (bi, bj), stencil stride st
        int bi, bj, st;
        if (dir == 0) { fi = i0 + xi; fj = j0 - 1 + xj; bi = xi + 2; bj = xj + 1; st = 1; }
        else { fi = i0 - 1 + xi; fj = j0 + xj; bi = xi + 1; bj = xj + 2; st = WI; }
        fk = k + 1;
        const int o = bj * WI + bi;
        const float* cf = dir == 0 ? cf1 : cf2;
        const int f = dir == 0 ? fi : fj;
        const float cpL = cf[f - 1], cmR = cf[g.ncmax + f];
#pragma unroll
        for (int m = 0; m < 7; ++m) {
          const float* a = slot_var(S, sk1, wave_src(dir, m));
          if (ORDER == 1) {
            wl[m] = a[o - st];
            wr[m] = a[o];
          } else {
            const float a0 = a[o - 2 * st], a1 = a[o - st], a2 = a[o], a3 = a[o + st];
            wl[m] = a1 + cpL * vl_slope(a0, a1, a2);
            wr[m] = a2 - cmR * vl_slope(a1, a2, a3);
          }
        }
        bx = dir == 0 ? __ldg(bf1 + f1idx(g, fk, fj, fi)) : __ldg(bf2 + f2idx(g, fk, fj, fi));
        dxd = dir == 0 ? dx1 : dx2;
      }
      float fx[7], em[3];
      solve_face<SOLVER>(wl, wr, bx, gam, dxd, dtf, fx, em);
      // unrotate the hydro flux: (d, m_dir, m_dir+1, m_dir+2, E) -> (d, m1, m2, m3, E)
      float fh[NHYD];
      fh[IDN] = fx[IDN];
      fh[IVX + dir] = fx[IVX];
      fh[IVX + (dir + 1) % 3] = fx[IVY];
      fh[IVX + (dir + 2) % 3] = fx[IVZ];
      fh[IEN] = fx[IEN];
      if (dir == 2) {
        const int r = xj * XW + xi;
        S.x3e[0][r] = em[0]; S.x3e[1][r] = em[1]; S.x3e[2][r] = em[2];
        if (q < 0) {
#pragma unroll
          for (int n = 0; n < NHYD; ++n) f3up[n] = fh[n];
        }
      } else if (dir == 0) {
        const int r = xj * N1W + xi;
        S.x1e[pn][0][r] = em[0]; S.x1e[pn][1][r] = em[1]; S.x1e[pn][2][r] = em[2];
        if (xj >= 1 && xj <= TJ) {
#pragma unroll
          for (int n = 0; n < NHYD; ++n) S.x1h[n][xj - 1][xi] = fh[n];
        }
      } else {
        const int r = xj * N2W + xi;
        S.x2e[pn][0][r] = em[0]; S.x2e[pn][1][r] = em[1]; S.x2e[pn][2][r] = em[2];
        if (xi >= 1 && xi <= TI) {
#pragma unroll
          for (int n = 0; n < NHYD; ++n) S.x2h[n][xj][xi - 1] = fh[n];
        }
      }
    }
    __syncthreads();
    if (pre) continue;

    // ---- corner EMFs: e3 of plane k+1, e1 and e2 of face plane k+1 ----
    // cell-centred E of the rectangle cell at box coordinates (ii, jj) of plane k (slot sk)
    // or k+1 (slot sk1), formed by the faces' x3 items of this step and the last
    auto cce = [&](int slot, int n, int jj, int ii) -> float {
      return S.cc[slot == sk1 ? pn : po][n][(jj - 1) * XW + (ii - 1)];
    };
    for (int q = tid; q < NE3 + NE1 + NE2; q += NT) {
      if (q < NE3) {
        // e3 at (k+1, j, i), i in [i0, i0+TI], j in [j0, j0+TJ]: box (ii = ei+2, jj = ej+2)
        const int ei = q % (TI + 1), ej = q / (TI + 1);
        const int ii = ei + 2, jj = ej + 2;
        const float* E = S.x1e[pn][0];
        const float* W1 = S.x1e[pn][2];
        const float* F = S.x2e[pn][1];
        const float* W2 = S.x2e[pn][2];
        // x1 face (i, j) is item (ej+1)*N1W + ei; x2 face (i, j) is ej*N2W + ei+1
        const int a1 = (ej + 1) * N1W + ei, a1m = ej * N1W + ei;      // rows j, j-1
        const int a2 = ej * N2W + ei + 1, a2m = ej * N2W + ei;         // columns i, i-1
        const float de3_l2 = up(W1[a1m], F[a2], cce(sk1, 2, jj - 1, ii), F[a2m], cce(sk1, 2, jj - 1, ii - 1));
        const float de3_r2 = up(W1[a1], F[a2], cce(sk1, 2, jj, ii), F[a2m], cce(sk1, 2, jj, ii - 1));
        const float de3_l1 = up(W2[a2m], E[a1], cce(sk1, 2, jj, ii - 1), E[a1m], cce(sk1, 2, jj - 1, ii - 1));
        const float de3_r1 = up(W2[a2], E[a1], cce(sk1, 2, jj, ii), E[a1m], cce(sk1, 2, jj - 1, ii));
        S.e3[pn][ej][ei] = 0.25f * (de3_l1 + de3_r1 + de3_l2 + de3_r2 + F[a2m] + F[a2] +
                                    E[a1m] + E[a1]);
      } else if (q < NE3 + NE1) {
        // e1 at face plane k+1, (j, i): i in the tile, j in [j0, j0+TJ]
        const int r = q - NE3, ei = r % TI, ej = r / TI;
        const int ii = ei + 2, jj = ej + 2;
        const int a2 = ej * N2W + ei + 1;                    // x2 face (i, j)
        const int x = (ej + 1) * XW + ei + 1, xm = ej * XW + ei + 1;  // x3 faces (j), (j-1)
        const float* E2n = S.x2e[pn][0];
        const float* E2o = S.x2e[po][0];
        const float w2o = S.x2e[po][2][a2], w2n = S.x2e[pn][2][a2];
        const float* E3 = S.x3e[1];
        const float* W3 = S.x3e[2];
        const float de1_l3 = up(w2o, E3[x], cce(sk, 0, jj, ii), E3[xm], cce(sk, 0, jj - 1, ii));
        const float de1_r3 = up(w2n, E3[x], cce(sk1, 0, jj, ii), E3[xm], cce(sk1, 0, jj - 1, ii));
        const float de1_l2 = up(W3[xm], E2n[a2], cce(sk1, 0, jj - 1, ii), E2o[a2], cce(sk, 0, jj - 1, ii));
        const float de1_r2 = up(W3[x], E2n[a2], cce(sk1, 0, jj, ii), E2o[a2], cce(sk, 0, jj, ii));
        S.e1[pn][ej][ei] = 0.25f * (de1_l3 + de1_r3 + de1_l2 + de1_r2 + E2o[a2] + E2n[a2] +
                                    E3[xm] + E3[x]);
      } else {
        // e2 at face plane k+1, (j, i): i in [i0, i0+TI], j in the tile
        const int r = q - NE3 - NE1, ei = r % (TI + 1), ej = r / (TI + 1);
        const int ii = ei + 2, jj = ej + 2;
        const int a1 = (ej + 1) * N1W + ei;                   // x1 face (i, j)
        const int x = (ej + 1) * XW + ei + 1, xm = (ej + 1) * XW + ei;  // x3 faces (i), (i-1)
        const float* E1n = S.x1e[pn][1];
        const float* E1o = S.x1e[po][1];
        const float w1o = S.x1e[po][2][a1], w1n = S.x1e[pn][2][a1];
        const float* E3 = S.x3e[0];
        const float* W3 = S.x3e[2];
        const float de2_l3 = up(w1o, E3[x], cce(sk, 1, jj, ii), E3[xm], cce(sk, 1, jj, ii - 1));
        const float de2_r3 = up(w1n, E3[x], cce(sk1, 1, jj, ii), E3[xm], cce(sk1, 1, jj, ii - 1));
        const float de2_l1 = up(W3[xm], E1n[a1], cce(sk1, 1, jj, ii - 1), E1o[a1], cce(sk, 1, jj, ii - 1));
        const float de2_r1 = up(W3[x], E1n[a1], cce(sk1, 1, jj, ii), E1o[a1], cce(sk, 1, jj, ii));
        S.e2[pn][ej][ei] = 0.25f * (de2_l3 + de2_r3 + de2_l1 + de2_r1 + E3[xm] + E3[x] +
                                    E1o[a1] + E1n[a1]);
      }
    }
    __syncthreads();

    // ---- update of this thread's cell in plane k ----
    if (upd) {
      // exact flux sum: the x1/x2 part carried from the last step, the two x3 faces now
      double un[NHYD];
#pragma unroll
      for (int n = 0; n < NHYD; ++n) {
        float s3, e3, hi, e5;
        two_sum(__fmul_rn(cw3, f3up[n]), -__fmul_rn(cw3, f3lo[n]), s3, e3);
        two_sum(pt[n], s3, hi, e5);
        const float lo = (pe12[n] + e3) + (pe4[n] + e5);
        un[n] = (uo[n] - f2d_int(hi)) - f2d_int(lo);
      }
      // CT of the faces around the cell: E1[dk][dj], E2[dk][di], E3[dj][di]
      float E1[2][2], E2[2][2], E3[2][2];
#pragma unroll
      for (int x = 0; x < 2; ++x)
#pragma unroll
        for (int y = 0; y < 2; ++y) {
          E1[x][y] = S.e1[x ? pn : po][tj + y][ti];
          E2[x][y] = S.e2[x ? pn : po][tj][ti + y];
          E3[x][y] = S.e3[po][tj + x][ti + y];
        }
      auto ct = [&](double base, float a, float b0, float c0, float d0, float wa, float wb,
                    double ia) {
        float hi, lo;
        sum2diff(__fmul_rn(wa, a), __fmul_rn(wa, b0), __fmul_rn(wb, c0), __fmul_rn(wb, d0), hi, lo);
        return fma(f2d_int(lo), ia, fma(f2d_int(hi), ia, base));
      };
      const double n1l = ct(bl1, E3[0][0], E3[1][0], E2[1][0], E2[0][0], we3, we2, mg.ia[0]);
      const double n1u = ct(bu1, E3[0][1], E3[1][1], E2[1][1], E2[0][1], we3, we2, mg.ia[0]);
      const double n2l = ct(bl2, E3[0][1], E3[0][0], E1[0][0], E1[1][0], we3, we1, mg.ia[1]);
      const double n2u = ct(bu2, E3[1][1], E3[1][0], E1[0][1], E1[1][1], we3, we1, mg.ia[1]);
      const double n3l = b3lo;
      const double n3u = ct(bu3, E2[1][0], E2[1][1], E1[1][1], E1[1][0], we2, we1, mg.ia[2]);
      b3lo = n3u;
      // stores of the new state and its FP32 copies (the write set)
      const int64_t q1 = (int64_t)b * g.nf1 + f1idx(g, k, cj, ci);
      const int64_t q2 = (int64_t)b * g.nf2 + f2idx(g, k, cj, ci);
      const int64_t q3 = (int64_t)b * g.nf3 + f3idx(g, k, cj, ci);
      const ff f1 = split_ff(n1l), f2 = split_ff(n2l), f3 = split_ff(n3l);
      const ff u1f = split_ff(n1u), u2f = split_ff(n2u), u3f = split_ff(n3u);
      A.sb.b_out[0][q1] = n1l;
      A.sb.b_out[1][q2] = n2l;
      A.sb.b_out[2][q3] = n3l;
      A.bf_out[0][q1] = f1.hi;
      A.bf_out[1][q2] = f2.hi;
      A.bf_out[2][q3] = f3.hi;
      if (ci == g.ie) { A.sb.b_out[0][q1 + 1] = n1u; A.bf_out[0][q1 + 1] = u1f.hi; }
      if (cj == g.je) { A.sb.b_out[1][q2 + g.nc1] = n2u; A.bf_out[1][q2 + g.nc1] = u2f.hi; }
      if (k == g.ke) {
        const int64_t qt = q3 + (int64_t)g.nc1 * g.nc2;
        A.sb.b_out[2][qt] = n3u;
        A.bf_out[2][qt] = u3f.hi;
      }
      const ff s1 = ff_add(f1, u1f), s2f = ff_add(f2, u2f), s3f = ff_add(f3, u3f);
      float* __restrict__ bcc = A.bcc_out + (int64_t)b * 3 * nc;
      const float bxc = 0.5f * ff_f(s1), byc = 0.5f * ff_f(s2f), bzc = 0.5f * ff_f(s3f);
      bcc[c] = bxc;
      bcc[nc + c] = byc;
      bcc[2 * nc + c] = bzc;
      const ff ss = ff_add(ff_add(ff_sqr(s1), ff_sqr(s2f)), ff_sqr(s3f));
      // primitive recovery (the mixed k_c2p)
      const Phys& ph = A.ph;
      double ud = un[0];
      const uint64_t ub = bits_d(ud);
      if (!((ub >> 63) == 0 && ub > bits_d(ph.dfloor) && ub <= 0x7ff0000000000000ull)) ud = ph.dfloor;
      const ff dd = split_ff(ud), mx1 = split_ff(un[1]), mx2 = split_ff(un[2]), mx3 = split_ff(un[3]);
      const ff di = ff_recip(dd);
      const ff mm = ff_add(ff_add(ff_sqr(mx1), ff_sqr(mx2)), ff_sqr(mx3));
      ff x = ff_add(ff_mul(mm, di), ff_scale(ss, 0.25f));
      const ff wp = ff_mul(ff_sub(split_ff(un[4]), ff_scale(x, 0.5f)), ph.gm1f);
      double ue = un[4];
      float pf;
      if (!ff_gt(wp, ph.pfloorf)) {
        ue = (ph.pfloor / ph.gm1) + 0.5 * (f2d_int(x.hi) + f2d_int(x.lo));
        pf = d2f_int(ph.pfloor);
      } else {
        pf = ff_f(wp);
      }
      double* __restrict__ uout = A.sb.u_out + (int64_t)b * NHYD * nc;
      uout[c] = ud;
      uout[nc + c] = un[1];
      uout[2 * nc + c] = un[2];
      uout[3 * nc + c] = un[3];
      uout[4 * nc + c] = ue;
      const float dif = ff_f(di);
      const float vx = mx1.hi * dif, vy = mx2.hi * dif, vz = mx3.hi * dif;
      float* __restrict__ w = A.w_out + (int64_t)b * NHYD * nc;
      w[c] = dd.hi;
      w[nc + c] = vx;
      w[2 * nc + c] = vy;
      w[3 * nc + c] = vz;
      w[4 * nc + c] = pf;
      if constexpr (DT) {
        // device error word: a primitive or cell-centred field value that is not finite
        // (the floors replace a non-finite density or energy, not a momentum)
        auto inf_or_nan = [](float x) { return (bits_f(x) & 0x7f800000u) == 0x7f800000u; };
        const bool nf =
            (inf_or_nan(dd.hi) | inf_or_nan(vx) | inf_or_nan(vy) | inf_or_nan(vz) |
             inf_or_nan(pf) | inf_or_nan(bxc) | inf_or_nan(byc) | inf_or_nan(bzc));
        if (nf) atomicOr(A.err, kErrNonFinite);
        const float d = dd.hi;
        float cfs = fast_speed<float>(d, pf, byc, bzc, bxc + fabsf(f1.hi - bxc), gam);
        const float dt1 = dx1 / (fabsf(vx) + cfs);
        cfs = fast_speed<float>(d, pf, bzc, bxc, byc + fabsf(f2.hi - byc), gam);
        const float dt2 = dx2 / (fabsf(vy) + cfs);
        cfs = fast_speed<float>(d, pf, bxc, byc, bzc + fabsf(f3.hi - bzc), gam);
        const float dt3 = dx3 / (fabsf(vz) + cfs);
        mindt = mn(mn(mn(mindt, dt1), dt2), dt3);
      }
#pragma unroll
      for (int n = 0; n < NHYD; ++n) f3lo[n] = f3up[n];
    } else {
      // k = ks0 - 1: the face plane below the first cell of the segment
#pragma unroll
      for (int n = 0; n < NHYD; ++n) f3lo[n] = f3up[n];
      const int64_t q3 = (int64_t)b * g.nf3 + f3idx(g, k + 1, cj, ci);
      const double b3in = __ldg(A.sb.b_in[2] + q3);
      float hi, lo;
      const float a0 = S.e2[pn][tj][ti], a1 = S.e2[pn][tj][ti + 1];
      const float c0 = S.e1[pn][tj + 1][ti], d0 = S.e1[pn][tj][ti];
      sum2diff(__fmul_rn(we2, a0), __fmul_rn(we2, a1), __fmul_rn(we1, c0), __fmul_rn(we1, d0), hi, lo);
      b3lo = fma(f2d_int(lo), mg.ia[2], fma(f2d_int(hi), mg.ia[2], b3in));
    }
    // x1/x2 part of the flux sum of the cell in plane k+1 (faces computed this step)
    if (k + 1 <= ke0) {
#pragma unroll
      for (int n = 0; n < NHYD; ++n) {
        float s1, e1, s2, e2;
        two_sum(__fmul_rn(cw1, S.x1h[n][tj][ti + 1]), -__fmul_rn(cw1, S.x1h[n][tj][ti]), s1, e1);
        two_sum(__fmul_rn(cw2, S.x2h[n][tj + 1][ti]), -__fmul_rn(cw2, S.x2h[n][tj][ti]), s2, e2);
        two_sum(s1, s2, pt[n], pe4[n]);
        pe12[n] = e1 + e2;
      }
    }
    __syncthreads();
  }
  if (failed) {
    // a load did not arrive: wait (bounded) for the copies still in flight into this
    // block's shared memory before it exits
    for (int pl = waited + 1; pl <= issued; ++pl) {
      const int r = pl - p0;
      bar_wait(&S.bar[r & 3], (uint32_t)((r >> 2) & 1));
    }
  }
  if constexpr (DT) {  // block minimum, then one 64-bit atomicMin (as k_update_c2p)
    for (int o = 16; o > 0; o >>= 1) mindt = mn(mindt, __shfl_xor_sync(0xffffffffu, mindt, o));
    __shared__ float red[NT / 32];
    if ((tid & 31) == 0) red[tid >> 5] = mindt;
    __syncthreads();
    if (tid < 32) {
      float v = tid < NT / 32 ? red[tid] : 3.402823466e38f;
      for (int o = 16; o > 0; o >>= 1) v = mn(v, __shfl_xor_sync(0xffffffffu, v, o));
      if (tid == 0 && !failed) {
        const double vd = (v == 3.402823466e38f) ? 1.79769313486231570815e308 : f2d_int(v);
        atomicMin(A.dtmin, (unsigned long long)__double_as_longlong(vd));
      }
    }
  }
}

}  // namespace

size_t single_pass_smem() { return sizeof(Smem) + 128; }

int single_pass_setup() {
  const int sm = (int)single_pass_smem();
  const void* ks[] = {
      (const void*)k_single_pass<1, HLLD, false>, (const void*)k_single_pass<1, HLLD, true>,
      (const void*)k_single_pass<2, HLLD, false>, (const void*)k_single_pass<2, HLLD, true>,
      (const void*)k_single_pass<1, HLLE, false>, (const void*)k_single_pass<1, HLLE, true>,
      (const void*)k_single_pass<2, HLLE, false>, (const void*)k_single_pass<2, HLLE, true>};
  for (const void* k : ks) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, sm);
    if (e != cudaSuccess) return (int)e;
  }
  return 0;
}

int single_pass_maps(const float* w, const float* bcc, const Geom& g, SinglePassMaps* out,
                     std::string* err) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  if (!encode) {
    cudaDriverEntryPointQueryResult q;
    void* fn = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault,
                                         &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
      *err = "cuTensorMapEncodeTiled is not available";
      return -1;
    }
    encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  }
  // [nb * ncomp][nc3][nc2][nc1] floats; box: the 36 x 12 plane of all components
  auto make = [&](const float* base, int ncomp, void* dst) -> bool {
    const cuuint64_t dims[4] = {(cuuint64_t)g.nc1, (cuuint64_t)g.nc2, (cuuint64_t)g.nc3,
                                (cuuint64_t)ncomp * (cuuint64_t)g.nb};
    const cuuint64_t strides[3] = {(cuuint64_t)g.nc1 * 4, (cuuint64_t)g.nc1 * g.nc2 * 4,
                                   (cuuint64_t)g.ncell * 4};
    const cuuint32_t box[4] = {(cuuint32_t)WI, (cuuint32_t)WJ, 1u, (cuuint32_t)ncomp};
    const cuuint32_t es[4] = {1u, 1u, 1u, 1u};
    CUresult r = encode(reinterpret_cast<CUtensorMap*>(dst), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                        const_cast<float*>(base), dims, strides, box, es,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                        CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
  };
  if (!make(w, 5, out->w) || !make(bcc, 3, out->bcc)) {
    *err = "cuTensorMapEncodeTiled failed for the W/bcc arrays";
    return -1;
  }
  return 0;
}

bool single_pass_fits(const Geom& g, int nseg) {
  return g.ng == 2 && g.nx1 % TI == 0 && g.nx2 % TJ == 0 && nseg >= 1 && g.nx3 % nseg == 0 &&
         g.nx3 / nseg >= 1 && g.nb <= 65535;
}

int single_pass_launch(const SinglePassMaps& maps, const Geom& g, const StagePtrs<float>& p,
                       float* w_out, float* bcc_out, float* const bf_out[3], const StateBufs& sb,
                       const StageW& sw, const Phys& ph, unsigned long long* dtmin,
                       unsigned int* err, int order, int solver, int nseg, cudaStream_t st) {
  SpArgs a;
  a.g = g; a.p = p; a.w_out = w_out; a.bcc_out = bcc_out;
  for (int d = 0; d < 3; ++d) a.bf_out[d] = bf_out[d];
  a.sb = sb; a.sw = sw; a.ph = ph; a.dtmin = dtmin; a.err = err; a.nseg = nseg;
  const dim3 grid((unsigned)((g.nx1 / TI) * (g.nx2 / TJ)), (unsigned)nseg, (unsigned)g.nb);
  const size_t sm = single_pass_smem();
  const CUtensorMap* tw = reinterpret_cast<const CUtensorMap*>(maps.w);
  const CUtensorMap* tb = reinterpret_cast<const CUtensorMap*>(maps.bcc);
#define ATHG_SP(O, S, D) k_single_pass<O, S, D><<<grid, NT, sm, st>>>(*tw, *tb, a)
  const bool dt = dtmin != nullptr;
  if (solver == HLLD) {
    if (order == 1) { if (dt) ATHG_SP(1, HLLD, true); else ATHG_SP(1, HLLD, false); }
    else { if (dt) ATHG_SP(2, HLLD, true); else ATHG_SP(2, HLLD, false); }
  } else {
    if (order == 1) { if (dt) ATHG_SP(1, HLLE, true); else ATHG_SP(1, HLLE, false); }
    else { if (dt) ATHG_SP(2, HLLE, true); else ATHG_SP(2, HLLE, false); }
  }
#undef ATHG_SP
  return (int)cudaGetLastError();
}

}  // namespace athg

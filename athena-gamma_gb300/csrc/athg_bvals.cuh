// athg_bvals.cuh -- on-device ghost-zone exchange between MeshBlocks of the same level.
//
// The reference packs each neighbour's ghost region into a buffer, copies it
// (std::memcpy on one rank, MPI otherwise) and unpacks it (src/bvals/bvals_var.cpp:108-330,
// src/bvals/cc/bvals_cc.cpp:201-342, src/bvals/fc/bvals_fc.cpp:344-397). Here all blocks
// live in one device pool, so one launch gathers every ghost value straight from the
// owning neighbour's interior: no buffers, no pack/unpack.
//
// Ownership rule (same as the reference's pack ranges): along a cell axis a block owns
// indices [s, e]; along the normal axis of a face field it owns [s, e+1] (the shared
// face is never exchanged, bvals_fc.cpp:351-353). A ghost location takes the value of
// the neighbour in direction (ox1,ox2,ox3) at the index shifted by -ox*nx.
#pragma once
#include "athg_device.cuh"

namespace athg {

struct GhostPtrs {
  double *u, *b1, *b2, *b3;
  const int* nbr;  // [nb][27], same-level neighbour block id, -1 = none
  int nvar;        // cell variables in u (5)
  int mhd;
};

__device__ __forceinline__ int ghost_dir(int i, int s, int e) {
  return i < s ? -1 : (i > e ? 1 : 0);
}

// The positions (k,j,i) of [0,nc3]x[0,nc2]x[0,nc1] (the edge-sized box, so the last face
// of each axis is included) that hold any ghost value, as three disjoint regions: A, the
// k-ghost planes; B, the j-ghost rows of the interior planes; C, the i-ghost columns of the
// interior rows. One thread per position of the ghost shell instead of the whole box.
__host__ __device__ inline int64_t ghost_shell_size(const Geom& g) {
  const int64_t gk = g.nc3 + 1 - g.nx3, gj = g.nc2 + 1 - g.nx2, gi = g.nc1 + 1 - g.nx1;
  return gk * (g.nc2 + 1) * (g.nc1 + 1) + (int64_t)g.nx3 * gj * (g.nc1 + 1) +
         (int64_t)g.nx3 * g.nx2 * gi;
}
// t < ghost_shell_size(g), which fits 32 bits for any block that fits in memory: 32-bit
// index arithmetic (64-bit division is a long instruction sequence)
__device__ __forceinline__ void ghost_shell_pos(const Geom& g, int t, int& k, int& j, int& i) {
  const int gk = g.nc3 + 1 - g.nx3, gj = g.nc2 + 1 - g.nx2, gi = g.nc1 + 1 - g.nx1;
  const int w1 = g.nc1 + 1, w2 = g.nc2 + 1;
  const int na = gk * w2 * w1;
  const int nbb = g.nx3 * gj * w1;
  // quotients by multiply and shift (FastDiv), remainders from them
  if (t < na) {
    const int r = fastdiv(t, g.dw1);
    i = t - r * w1;
    const int q = fastdiv(r, g.dw2);
    j = r - q * w2;
    k = q < g.ks ? q : q + g.nx3;  // 0..ks-1, then ke+1..nc3
  } else if (t < na + nbb) {
    const int u = t - na;
    const int r = fastdiv(u, g.dw1);
    i = u - r * w1;
    const int rk = fastdiv(r, g.dgj);
    const int q = r - rk * gj;
    j = q < g.js ? q : q + g.nx2;
    k = g.ks + rk;
  } else {
    const int u = t - na - nbb;
    const int r = fastdiv(u, g.dgi);
    const int q = u - r * gi;
    i = q < g.is ? q : q + g.nx1;
    const int rk = fastdiv(r, g.dnx2);
    j = g.js + (r - rk * g.nx2);
    k = g.ks + rk;
  }
}

// One thread per (k,j,i) of the largest (edge-sized) box of every block; each thread
// handles the cell and the three faces that share this index, when they are ghosts.
__global__ void __launch_bounds__(256) k_ghost_same_level(Geom g, GhostPtrs p) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ghost_shell_size(g)) return;
  int k, j, i;
  ghost_shell_pos(g, (int)t, k, j, i);
  const int b = blockIdx.y;
  const int* nb = p.nbr + (int64_t)b * 27;
  // cell-centred variables
  if (i < g.nc1 && j < g.nc2 && k < g.nc3) {
    int o1 = ghost_dir(i, g.is, g.ie), o2 = ghost_dir(j, g.js, g.je), o3 = ghost_dir(k, g.ks, g.ke);
    if (o1 | o2 | o3) {
      int src = nb[(o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)];
      if (src >= 0) {
        int64_t d = cidx(g, k, j, i);
        int64_t s = cidx(g, k - o3 * g.nx3, j - o2 * g.nx2, i - o1 * g.nx1);
        const double* __restrict__ us = p.u + (int64_t)src * NHYD * g.ncell;
        double* __restrict__ ud = p.u + (int64_t)b * NHYD * g.ncell;
        double v[NHYD];
#pragma unroll
        for (int n = 0; n < NHYD; ++n) v[n] = __ldg(us + n * g.ncell + s);
#pragma unroll
        for (int n = 0; n < NHYD; ++n) ud[n * g.ncell + d] = v[n];
      }
    }
  }
  if (!p.mhd) return;
  if (i <= g.nc1 && j < g.nc2 && k < g.nc3) {  // x1 faces
    int o1 = ghost_dir(i, g.is, g.ie + 1), o2 = ghost_dir(j, g.js, g.je), o3 = ghost_dir(k, g.ks, g.ke);
    if (o1 | o2 | o3) {
      int src = nb[(o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)];
      if (src >= 0)
        p.b1[(int64_t)b * g.nf1 + f1idx(g, k, j, i)] =
            p.b1[(int64_t)src * g.nf1 + f1idx(g, k - o3 * g.nx3, j - o2 * g.nx2, i - o1 * g.nx1)];
    }
  }
  if (i < g.nc1 && j <= g.nc2 && k < g.nc3) {  // x2 faces
    int o1 = ghost_dir(i, g.is, g.ie), o2 = ghost_dir(j, g.js, g.je + 1), o3 = ghost_dir(k, g.ks, g.ke);
    if (o1 | o2 | o3) {
      int src = nb[(o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)];
      if (src >= 0)
        p.b2[(int64_t)b * g.nf2 + f2idx(g, k, j, i)] =
            p.b2[(int64_t)src * g.nf2 + f2idx(g, k - o3 * g.nx3, j - o2 * g.nx2, i - o1 * g.nx1)];
    }
  }
  if (i < g.nc1 && j < g.nc2 && k <= g.nc3) {  // x3 faces
    int o1 = ghost_dir(i, g.is, g.ie), o2 = ghost_dir(j, g.js, g.je), o3 = ghost_dir(k, g.ks, g.ke + 1);
    if (o1 | o2 | o3) {
      int src = nb[(o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)];
      if (src >= 0)
        p.b3[(int64_t)b * g.nf3 + f3idx(g, k, j, i)] =
            p.b3[(int64_t)src * g.nf3 + f3idx(g, k - o3 * g.nx3, j - o2 * g.nx2, i - o1 * g.nx1)];
    }
  }
}

// The same exchange for the mixed path's FP32 working arrays when the primitives of the
// interior are recovered inside the update (k_update_c2p): up to three cell-variable groups
// (W, bcc, cell-centred E) and the FP32 face-field copies, with the ownership rules above.
// cell[2] may be null (no cell-centred E: the single-pass stage recomputes it).
struct GhostPtrs32 {
  float* cell[3];  // [nb][ncomp[q]][cells]
  int ncomp[3];
  float* face[3];  // [nb][faces] per direction (nullptr: hydro)
  const int* nbr;
};

// Every value is loaded before any is stored (the source is always a neighbour's interior,
// never a ghost, so loads and stores never overlap), keeping all of a thread's loads in flight.
template <bool MHD>
__global__ void __launch_bounds__(256) k_ghost_f32(Geom g, GhostPtrs32 p) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ghost_shell_size(g)) return;
  int k, j, i;
  ghost_shell_pos(g, (int)t, k, j, i);
  const int b = blockIdx.y;
  const int* nb = p.nbr + (int64_t)b * 27;
  const int64_t nc = g.ncell;
  constexpr int NV = MHD ? 11 : 5;
  float v[NV];
  int64_t dst = -1;
  if (i < g.nc1 && j < g.nc2 && k < g.nc3) {
    int o1 = ghost_dir(i, g.is, g.ie), o2 = ghost_dir(j, g.js, g.je), o3 = ghost_dir(k, g.ks, g.ke);
    if (o1 | o2 | o3) {
      int src = nb[(o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)];
      if (src >= 0) {
        const int64_t s = cidx(g, k - o3 * g.nx3, j - o2 * g.nx2, i - o1 * g.nx1);
        const float* __restrict__ w = p.cell[0] + (int64_t)src * 5 * nc;
#pragma unroll
        for (int n = 0; n < 5; ++n) v[n] = __ldg(w + n * nc + s);
        if constexpr (MHD) {
          const float* __restrict__ bc = p.cell[1] + (int64_t)src * 3 * nc;
#pragma unroll
          for (int n = 0; n < 3; ++n) v[5 + n] = __ldg(bc + n * nc + s);
          if (p.cell[2]) {  // the cell-centred EMF (absent for the single-pass stage)
            const float* __restrict__ ce = p.cell[2] + (int64_t)src * 3 * nc;
#pragma unroll
            for (int n = 0; n < 3; ++n) v[8 + n] = __ldg(ce + n * nc + s);
          }
        }
        dst = cidx(g, k, j, i);
      }
    }
  }
  float fv[3];
  int64_t fd[3] = {-1, -1, -1};
  if constexpr (MHD) {
    if (i <= g.nc1 && j < g.nc2 && k < g.nc3) {
      int o1 = ghost_dir(i, g.is, g.ie + 1), o2 = ghost_dir(j, g.js, g.je), o3 = ghost_dir(k, g.ks, g.ke);
      int src = (o1 | o2 | o3) ? nb[(o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)] : -1;
      if (src >= 0) {
        fv[0] = __ldg(p.face[0] + (int64_t)src * g.nf1 +
                      f1idx(g, k - o3 * g.nx3, j - o2 * g.nx2, i - o1 * g.nx1));
        fd[0] = (int64_t)b * g.nf1 + f1idx(g, k, j, i);
      }
    }
    if (i < g.nc1 && j <= g.nc2 && k < g.nc3) {
      int o1 = ghost_dir(i, g.is, g.ie), o2 = ghost_dir(j, g.js, g.je + 1), o3 = ghost_dir(k, g.ks, g.ke);
      int src = (o1 | o2 | o3) ? nb[(o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)] : -1;
      if (src >= 0) {
        fv[1] = __ldg(p.face[1] + (int64_t)src * g.nf2 +
                      f2idx(g, k - o3 * g.nx3, j - o2 * g.nx2, i - o1 * g.nx1));
        fd[1] = (int64_t)b * g.nf2 + f2idx(g, k, j, i);
      }
    }
    if (i < g.nc1 && j < g.nc2 && k <= g.nc3) {
      int o1 = ghost_dir(i, g.is, g.ie), o2 = ghost_dir(j, g.js, g.je), o3 = ghost_dir(k, g.ks, g.ke + 1);
      int src = (o1 | o2 | o3) ? nb[(o3 + 1) * 9 + (o2 + 1) * 3 + (o1 + 1)] : -1;
      if (src >= 0) {
        fv[2] = __ldg(p.face[2] + (int64_t)src * g.nf3 +
                      f3idx(g, k - o3 * g.nx3, j - o2 * g.nx2, i - o1 * g.nx1));
        fd[2] = (int64_t)b * g.nf3 + f3idx(g, k, j, i);
      }
    }
  }
  if (dst >= 0) {
    float* __restrict__ w = p.cell[0] + (int64_t)b * 5 * nc;
#pragma unroll
    for (int n = 0; n < 5; ++n) w[n * nc + dst] = v[n];
    if constexpr (MHD) {
      float* __restrict__ bc = p.cell[1] + (int64_t)b * 3 * nc;
#pragma unroll
      for (int n = 0; n < 3; ++n) bc[n * nc + dst] = v[5 + n];
      if (p.cell[2]) {
        float* __restrict__ ce = p.cell[2] + (int64_t)b * 3 * nc;
#pragma unroll
        for (int n = 0; n < 3; ++n) ce[n * nc + dst] = v[8 + n];
      }
    }
  }
  if constexpr (MHD) {
#pragma unroll
    for (int d = 0; d < 3; ++d)
      if (fd[d] >= 0) p.face[d][fd[d]] = fv[d];
  }
}

}  // namespace athg

namespace athg {

// ---- outflow physical boundaries (uniform meshes) ---------------------------------------
// Reference bvals/cc/outflow_cc.cpp and bvals/fc/outflow_fc.cpp as BoundaryValues::
// ApplyPhysicalBoundaries (bvals/bvals.cpp:436-600) applies them after the same-level
// exchange and the primitive recovery: primitives and face fields are copied outward from
// the last interior cell (the boundary face itself for the normal field), x1 faces first,
// then x2 over the x1 ghosts, then x3 over both; then the cell-centred field and U(W) of
// the filled ghost cells. Copying from the index clamped to the interior along every
// physical side gives the same values as the three passes. A block side is physical where
// its face neighbour in the table is -1 (a uniform mesh with that axis not periodic).
struct OutflowPtrs {
  double *u, *w, *b1, *b2, *b3, *bcc;
  const int* nbr;
  int mhd;
  double igm1;  // 1 / (gamma - 1)
};

struct PhysSides {
  bool lo[3], hi[3];
};
__device__ __forceinline__ PhysSides phys_sides(const int* nb) {
  PhysSides s;
  s.lo[0] = nb[13 - 1] < 0; s.hi[0] = nb[13 + 1] < 0;
  s.lo[1] = nb[13 - 3] < 0; s.hi[1] = nb[13 + 3] < 0;
  s.lo[2] = nb[13 - 9] < 0; s.hi[2] = nb[13 + 9] < 0;
  return s;
}
__device__ __forceinline__ int clamp_side(int x, int s, int e, bool lo, bool hi) {
  return (lo && x < s) ? s : ((hi && x > e) ? e : x);
}

// pass 1: primitives and face fields of the physical ghost zones
__global__ void __launch_bounds__(256) k_outflow_copy(Geom g, OutflowPtrs p) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ghost_shell_size(g)) return;
  int k, j, i;
  ghost_shell_pos(g, (int)t, k, j, i);
  const int b = blockIdx.y;
  const PhysSides ps = phys_sides(p.nbr + (int64_t)b * 27);
  if (i < g.nc1 && j < g.nc2 && k < g.nc3) {
    const int si = clamp_side(i, g.is, g.ie, ps.lo[0], ps.hi[0]);
    const int sj = clamp_side(j, g.js, g.je, ps.lo[1], ps.hi[1]);
    const int sk = clamp_side(k, g.ks, g.ke, ps.lo[2], ps.hi[2]);
    if (si != i || sj != j || sk != k) {
      double* w = p.w + (int64_t)b * NHYD * g.ncell;
      const int64_t d = cidx(g, k, j, i), s = cidx(g, sk, sj, si);
#pragma unroll
      for (int n = 0; n < NHYD; ++n) w[n * g.ncell + d] = w[n * g.ncell + s];
    }
  }
  if (!p.mhd) return;
  if (i <= g.nc1 && j < g.nc2 && k < g.nc3) {  // x1 faces: the boundary face is is / ie+1
    const int si = clamp_side(i, g.is, g.ie + 1, ps.lo[0], ps.hi[0]);
    const int sj = clamp_side(j, g.js, g.je, ps.lo[1], ps.hi[1]);
    const int sk = clamp_side(k, g.ks, g.ke, ps.lo[2], ps.hi[2]);
    if (si != i || sj != j || sk != k) {
      double* b1 = p.b1 + (int64_t)b * g.nf1;
      b1[f1idx(g, k, j, i)] = b1[f1idx(g, sk, sj, si)];
    }
  }
  if (i < g.nc1 && j <= g.nc2 && k < g.nc3) {  // x2 faces
    const int si = clamp_side(i, g.is, g.ie, ps.lo[0], ps.hi[0]);
    const int sj = clamp_side(j, g.js, g.je + 1, ps.lo[1], ps.hi[1]);
    const int sk = clamp_side(k, g.ks, g.ke, ps.lo[2], ps.hi[2]);
    if (si != i || sj != j || sk != k) {
      double* b2 = p.b2 + (int64_t)b * g.nf2;
      b2[f2idx(g, k, j, i)] = b2[f2idx(g, sk, sj, si)];
    }
  }
  if (i < g.nc1 && j < g.nc2 && k <= g.nc3) {  // x3 faces
    const int si = clamp_side(i, g.is, g.ie, ps.lo[0], ps.hi[0]);
    const int sj = clamp_side(j, g.js, g.je, ps.lo[1], ps.hi[1]);
    const int sk = clamp_side(k, g.ks, g.ke + 1, ps.lo[2], ps.hi[2]);
    if (si != i || sj != j || sk != k) {
      double* b3 = p.b3 + (int64_t)b * g.nf3;
      b3[f3idx(g, k, j, i)] = b3[f3idx(g, sk, sj, si)];
    }
  }
}

// pass 2: cell-centred field (field/field.cpp:117-160, uniform weights) and U(W)
// (eos/adiabatic_mhd.cpp:99-136, eos/adiabatic_hydro.cpp:89-118) of the filled ghost cells
__global__ void __launch_bounds__(256) k_outflow_cons(Geom g, OutflowPtrs p) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ghost_shell_size(g)) return;
  int k, j, i;
  ghost_shell_pos(g, (int)t, k, j, i);
  if (!(i < g.nc1 && j < g.nc2 && k < g.nc3)) return;
  const int b = blockIdx.y;
  const PhysSides ps = phys_sides(p.nbr + (int64_t)b * 27);
  const int si = clamp_side(i, g.is, g.ie, ps.lo[0], ps.hi[0]);
  const int sj = clamp_side(j, g.js, g.je, ps.lo[1], ps.hi[1]);
  const int sk = clamp_side(k, g.ks, g.ke, ps.lo[2], ps.hi[2]);
  if (si == i && sj == j && sk == k) return;
  const int64_t nc = g.ncell, c = cidx(g, k, j, i);
  const double* w = p.w + (int64_t)b * NHYD * nc;
  double* u = p.u + (int64_t)b * NHYD * nc;
  const double d = w[c], vx = w[nc + c], vy = w[2 * nc + c], vz = w[3 * nc + c],
               pr = w[4 * nc + c];
  // rounded operation by operation (no contraction), as the reference's scalar FP64 code
  auto M = [](double a, double x) { return __dmul_rn(a, x); };
  auto A = [](double a, double x) { return __dadd_rn(a, x); };
  u[c] = d;
  u[nc + c] = M(vx, d);
  u[2 * nc + c] = M(vy, d);
  u[3 * nc + c] = M(vz, d);
  const double v2 = A(A(M(vx, vx), M(vy, vy)), M(vz, vz));
  if (p.mhd) {
    const double* b1 = p.b1 + (int64_t)b * g.nf1;
    const double* b2 = p.b2 + (int64_t)b * g.nf2;
    const double* b3 = p.b3 + (int64_t)b * g.nf3;
    double* bcc = p.bcc + (int64_t)b * 3 * nc;
    const double c1 = A(M(0.5, b1[f1idx(g, k, j, i)]), M(0.5, b1[f1idx(g, k, j, i + 1)]));
    const double c2 = A(M(0.5, b2[f2idx(g, k, j, i)]), M(0.5, b2[f2idx(g, k, j + 1, i)]));
    const double c3 = A(M(0.5, b3[f3idx(g, k, j, i)]), M(0.5, b3[f3idx(g, k + 1, j, i)]));
    bcc[c] = c1; bcc[nc + c] = c2; bcc[2 * nc + c] = c3;
    const double b2s = A(A(M(c1, c1), M(c2, c2)), M(c3, c3));
    u[4 * nc + c] = A(M(pr, p.igm1), M(0.5, A(M(d, v2), b2s)));
  } else {
    u[4 * nc + c] = A(M(pr, p.igm1), M(M(0.5, d), v2));
  }
}

}  // namespace athg

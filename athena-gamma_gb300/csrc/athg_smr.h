// athg_smr.h -- static mesh refinement (SMR) on the block pool: work lists and the
// per-element arithmetic shared by the CUDA kernels and the CPU check.
//
// The reference fills ghost zones across refinement levels with per-neighbour pack /
// unpack buffers, coarse buffers and prolongation (src/bvals/bvals_refine.cpp,
// src/bvals/cc/bvals_cc.cpp, src/bvals/fc/bvals_fc.cpp, src/mesh/mesh_refinement.cpp) and
// corrects fluxes and EMFs at level boundaries (src/bvals/cc/flux_correction_cc.cpp,
// src/bvals/fc/flux_correction_fc.cpp). Here the host replays those index ranges once
// per mesh (athg_smr_plan.cpp) and emits flat work lists; the device runs each list with
// one generic kernel. Where several of the reference's receives write the same element,
// the list keeps the last writer, so the result is that of the reference's receive order.
//
// Everything below is plain C++ usable on host and device; the arithmetic keeps the
// reference's operation order (FP64, no contraction) so results agree bit for bit.
#pragma once
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "athg_numeric.h"  // ATHG_HD

namespace athg {

// Index geometry of one block and of its coarse buffer (mesh/meshblock.cpp:59-94:
// ncc = nx/2 + 2 NGHOST, cis = NGHOST, cnghost = (NGHOST+1)/2 + 1).
struct SmrDims {
  int nx1, nx2, nx3, ng;
  int nc1, nc2, nc3;
  int ncc1, ncc2, ncc3;
  int is, ie, js, je, ks, ke;
  int cis, cie, cjs, cje, cks, cke;
  int cng;  // cnghost
  int64_t ncell, nf1, nf2, nf3, ne;   // fine arrays per block (cells, faces, edges)
  int64_t ccell, cf1, cf2, cf3;       // coarse arrays per block
  ATHG_HD int64_t c(int k, int j, int i) const { return ((int64_t)k * nc2 + j) * nc1 + i; }
  ATHG_HD int64_t f1(int k, int j, int i) const {
    return ((int64_t)k * nc2 + j) * (nc1 + 1) + i;
  }
  ATHG_HD int64_t f2(int k, int j, int i) const {
    return ((int64_t)k * (nc2 + 1) + j) * nc1 + i;
  }
  ATHG_HD int64_t f3(int k, int j, int i) const { return c(k, j, i); }
  ATHG_HD int64_t e(int k, int j, int i) const {
    return ((int64_t)k * (nc2 + 1) + j) * (nc1 + 1) + i;
  }
  ATHG_HD int64_t cc(int k, int j, int i) const { return ((int64_t)k * ncc2 + j) * ncc1 + i; }
  ATHG_HD int64_t cf1i(int k, int j, int i) const {
    return ((int64_t)k * ncc2 + j) * (ncc1 + 1) + i;
  }
  ATHG_HD int64_t cf2i(int k, int j, int i) const {
    return ((int64_t)k * (ncc2 + 1) + j) * ncc1 + i;
  }
  ATHG_HD int64_t cf3i(int k, int j, int i) const { return cc(k, j, i); }
};

inline SmrDims smr_dims(int nx1, int nx2, int nx3, int ng) {
  SmrDims d;
  d.nx1 = nx1; d.nx2 = nx2; d.nx3 = nx3; d.ng = ng;
  d.nc1 = nx1 + 2 * ng; d.nc2 = nx2 + 2 * ng; d.nc3 = nx3 + 2 * ng;
  d.ncc1 = nx1 / 2 + 2 * ng; d.ncc2 = nx2 / 2 + 2 * ng; d.ncc3 = nx3 / 2 + 2 * ng;
  d.is = ng; d.ie = ng + nx1 - 1; d.js = ng; d.je = ng + nx2 - 1; d.ks = ng; d.ke = ng + nx3 - 1;
  d.cis = ng; d.cie = ng + nx1 / 2 - 1; d.cjs = ng; d.cje = ng + nx2 / 2 - 1;
  d.cks = ng; d.cke = ng + nx3 / 2 - 1;
  d.cng = (ng + 1) / 2 + 1;
  d.ncell = (int64_t)d.nc1 * d.nc2 * d.nc3;
  d.nf1 = (int64_t)d.nc3 * d.nc2 * (d.nc1 + 1);
  d.nf2 = (int64_t)d.nc3 * (d.nc2 + 1) * d.nc1;
  d.nf3 = (int64_t)(d.nc3 + 1) * d.nc2 * d.nc1;
  d.ne = (int64_t)(d.nc3 + 1) * (d.nc2 + 1) * (d.nc1 + 1);
  d.ccell = (int64_t)d.ncc1 * d.ncc2 * d.ncc3;
  d.cf1 = (int64_t)d.ncc3 * d.ncc2 * (d.ncc1 + 1);
  d.cf2 = (int64_t)d.ncc3 * (d.ncc2 + 1) * d.ncc1;
  d.cf3 = (int64_t)(d.ncc3 + 1) * d.ncc2 * d.ncc1;
  return d;
}

// arrays an element transfer writes: the block's own cells/faces, or its coarse buffer
enum SmrArr { SA_U = 0, SA_B1 = 1, SA_B2 = 2, SA_B3 = 3, SA_CU = 4, SA_CB1 = 5, SA_CB2 = 6,
              SA_CB3 = 7 };
// how the value is made: a copy of the source element, or a restriction of the 8 fine
// cells / 4 fine faces whose lower corner is the source index
enum SmrOp { SO_COPY = 0, SO_RCC = 1, SO_RF1 = 2, SO_RF2 = 3, SO_RF3 = 4 };

// One element of a ghost fill. didx indexes the destination array's own grid (fine or
// coarse); sidx the source block's fine arrays (U for cells, B1..B3 for faces). Cell
// entries move all NHYDRO components.
struct SmrXfer {
  int32_t dblk, sblk, didx, sidx;
  int16_t darr, op;
};

// Coarse face flux <- area average of four fine face fluxes (flux_correction_cc.cpp:66-158)
struct SmrFlux {
  int32_t dblk, dir, sblk;
  int32_t didx, sidx;  // face indices (sidx: lower corner of the four fine faces)
};

// Corrected EMF of one block-boundary edge: v = (own ? E : 0); v += each addition in
// order; v *= mul[0]; v *= mul[1] (flux_correction_fc.cpp:623-1749)
struct SmrEmf {
  int32_t blk, comp, own, add0, add1, idx;
  double mul[2];
};
// One addition: the neighbour's edge value, or (step != 0) the length-weighted average of
// two fine edges idx and idx + step of edge length len
struct SmrEmfAdd {
  int32_t sblk, comp, idx, step;
  double len;
};

// A cell or face position in a block (coarse or fine indices, as the list says)
struct SmrPos {
  int32_t blk, k, j, i;
};

struct SmrPlan {
  std::vector<SmrXfer> xfer;   // sender restrictions and receives, final writer per element
  std::vector<SmrXfer> pre;    // restriction of same-level ghosts into the coarse buffers
  std::vector<SmrFlux> flux;
  std::vector<SmrEmf> emf;
  std::vector<SmrEmfAdd> emf_add;
  std::vector<SmrPos> c2p;     // coarse cells: coarse bcc and W(U) (bvals_refine.cpp:375-381)
  std::vector<SmrPos> pcc;     // coarse cells prolongated into fine W
  std::vector<SmrPos> psf[3];  // coarse faces of the shared-field prolongation
  std::vector<SmrPos> pint;    // coarse cells of the internal-field prolongation
  std::vector<SmrPos> pfine;   // fine cells: bcc and U(W) after prolongation
  int nlevels = 1;
};

// One block of a multi-level mesh: level relative to the root grid and logical location
struct SmrLoc {
  int level;
  int64_t lx[3];
};

// Builds every work list for blocks `loc` of a periodic mesh whose root grid has nrb[d]
// blocks per axis. mhd: include face fields and EMFs. Returns false with a message for a
// mesh it does not support (levels must differ by at most one between neighbours).
// dx: [block][3] cell widths (the fine edge lengths of the EMF restriction).
bool smr_plan(const SmrDims& d, const int nrb[3], const std::vector<SmrLoc>& loc,
              const double* dx, bool mhd, SmrPlan* plan, std::string* err);

// Levels of every block's 26 neighbours (BoundaryBase::nblevel; -1 where none), 27 per
// block, index (ox3+1)*9 + (ox2+1)*3 + (ox1+1), the centre being the block's own level.
bool smr_neighbor_levels(const int nrb[3], const std::vector<SmrLoc>& loc, std::vector<int>* lv,
                         std::string* err);

// Cell widths and cell centres of one block along one axis, fine (nx + 2 ng entries) and
// of its coarse buffer (nx/2 + 2 ng entries), as the reference's Coordinates constructor
// computes them for a uniform mesh (coordinates/coordinates.cpp:88-145, coarse_flag
// variant, coordinates/cartesian.cpp:27-30). mesh_nx: root cells along the axis, nrb:
// root blocks along it; xff (optional): the fine face positions (nx + 2 ng + 1 entries).
void smr_axis_coords(int mesh_nx, int nrb, double xmin, double xmax, int level, int64_t lx,
                     int nx, int ng, double* dx, double* xvf, double* xvc, double* xff);

// ---- arithmetic ---------------------------------------------------------------------
// Pointers to one block's arrays; cell arrays hold NHYDRO (or 3) components of ncell
// (or ccell) each.
struct SmrBlockPtrs {
  double *u, *w, *b1, *b2, *b3, *bcc;      // fine
  double *cu, *cw, *cb1, *cb2, *cb3, *cbcc;  // coarse buffer
  double dx[3];                              // fine cell widths
  const double* xvf[3];                      // fine cell centres (nc entries)
  const double* xvc[3];                      // coarse cell centres (ncc entries)
};

// RestrictCellCenteredValues, 3-D (mesh_refinement.cpp:106-141): fine lower corner c
ATHG_HD double smr_restrict_cc(const SmrDims& d, const double* f, int64_t c, double vol) {
  const int64_t sj = d.nc1, sk = (int64_t)d.nc1 * d.nc2;
  const double tvol = ((vol + vol) + (vol + vol)) + ((vol + vol) + (vol + vol));
  return (((f[c] * vol + f[c + sj] * vol) + (f[c + 1] * vol + f[c + sj + 1] * vol)) +
          ((f[c + sk] * vol + f[c + sk + sj] * vol) +
           (f[c + sk + 1] * vol + f[c + sk + sj + 1] * vol))) / tvol;
}

// RestrictFieldX1/X2/X3, 3-D (mesh_refinement.cpp:184-371)
template <typename F>
ATHG_HD double smr_restrict_f1(const SmrDims& d, const F* f, int64_t q, double a) {
  const int64_t sj = d.nc1 + 1, sk = (int64_t)(d.nc1 + 1) * d.nc2;
  const double tarea = a + a + a + a;
  return ((double)f[q] * a + (double)f[q + sj] * a + (double)f[q + sk] * a +
          (double)f[q + sk + sj] * a) / tarea;
}
template <typename F>
ATHG_HD double smr_restrict_f2(const SmrDims& d, const F* f, int64_t q, double a) {
  const int64_t sk = (int64_t)d.nc1 * (d.nc2 + 1);
  const double tarea = a + a + a + a;
  return ((double)f[q] * a + (double)f[q + 1] * a + (double)f[q + sk] * a +
          (double)f[q + sk + 1] * a) / tarea;
}
template <typename F>
ATHG_HD double smr_restrict_f3(const SmrDims& d, const F* f, int64_t q, double a) {
  const int64_t sj = d.nc1;
  const double tarea = a + a + a + a;
  return ((double)f[q] * a + (double)f[q + 1] * a + (double)f[q + sj] * a +
          (double)f[q + sj + 1] * a) / tarea;
}

// minmod-limited slope 0.5 (SIGN(m) + SIGN(p)) min(|m|, |p|) (mesh_refinement.cpp:428-440)
ATHG_HD double smr_sign(double x) { return (x < 0.0) ? -1.0 : 1.0; }
ATHG_HD double smr_minmod(double gm, double gp) {
  const double am = fabs(gm), ap = fabs(gp);
  return 0.5 * (smr_sign(gm) + smr_sign(gp)) * ((ap < am) ? ap : am);
}

// Offsets of a coarse cell's centre from its neighbours' and from its fine cells' centres
// along one axis (x?v of the coarse buffer and of the block, mesh_refinement.cpp:392-427)
struct SmrAxis {
  double dm, dp, dfm, dfp;
};
ATHG_HD SmrAxis smr_axis(const double* xc, const double* xf, int c, int f) {
  SmrAxis a;
  const double x0 = xc[c - 1], x1 = xc[c], x2 = xc[c + 1];
  a.dm = x1 - x0;
  a.dp = x2 - x1;
  a.dfm = x1 - xf[f];
  a.dfp = xf[f + 1] - x1;
  return a;
}

// ProlongateCellCenteredValues, 3-D (mesh_refinement.cpp:386-451): one component of
// coarse cell (k,j,i) into its eight fine cells
ATHG_HD void smr_prolong_cc(const SmrDims& d, const double* co, double* fi, int k, int j, int i,
                            const SmrAxis& a1, const SmrAxis& a2, const SmrAxis& a3) {
  const int fk = (k - d.cks) * 2 + d.ks, fj = (j - d.cjs) * 2 + d.js, fx = (i - d.cis) * 2 + d.is;
  const int64_t c = d.cc(k, j, i), sj = d.ncc1, sk = (int64_t)d.ncc1 * d.ncc2;
  const double v = co[c];
  const double g1 = smr_minmod((v - co[c - 1]) / a1.dm, (co[c + 1] - v) / a1.dp);
  const double g2 = smr_minmod((v - co[c - sj]) / a2.dm, (co[c + sj] - v) / a2.dp);
  const double g3 = smr_minmod((v - co[c - sk]) / a3.dm, (co[c + sk] - v) / a3.dp);
  const int64_t q = d.c(fk, fj, fx), tj = d.nc1, tk = (int64_t)d.nc1 * d.nc2;
  fi[q] = v - (g1 * a1.dfm + g2 * a2.dfm + g3 * a3.dfm);
  fi[q + 1] = v + (g1 * a1.dfp - g2 * a2.dfm - g3 * a3.dfm);
  fi[q + tj] = v - (g1 * a1.dfm - g2 * a2.dfp + g3 * a3.dfm);
  fi[q + tj + 1] = v + (g1 * a1.dfp + g2 * a2.dfp - g3 * a3.dfm);
  fi[q + tk] = v - (g1 * a1.dfm + g2 * a2.dfm - g3 * a3.dfp);
  fi[q + tk + 1] = v + (g1 * a1.dfp - g2 * a2.dfm + g3 * a3.dfp);
  fi[q + tk + tj] = v - (g1 * a1.dfm - g2 * a2.dfp - g3 * a3.dfp);
  fi[q + tk + tj + 1] = v + (g1 * a1.dfp + g2 * a2.dfp + g3 * a3.dfp);
}

// ProlongateSharedFieldX1/X2/X3, 3-D (mesh_refinement.cpp:541-826): the coarse face
// (k,j,i) into its four fine faces, slopes along the two transverse axes
ATHG_HD void smr_prolong_f1(const SmrDims& d, const double* co, double* fi, int k, int j, int i,
                            const SmrAxis& a2, const SmrAxis& a3) {
  const int fk = (k - d.cks) * 2 + d.ks, fj = (j - d.cjs) * 2 + d.js, fx = (i - d.cis) * 2 + d.is;
  const int64_t c = d.cf1i(k, j, i), sj = d.ncc1 + 1, sk = (int64_t)(d.ncc1 + 1) * d.ncc2;
  const double v = co[c];
  const double g2 = smr_minmod((v - co[c - sj]) / a2.dm, (co[c + sj] - v) / a2.dp);
  const double g3 = smr_minmod((v - co[c - sk]) / a3.dm, (co[c + sk] - v) / a3.dp);
  const int64_t q = d.f1(fk, fj, fx), tj = d.nc1 + 1, tk = (int64_t)(d.nc1 + 1) * d.nc2;
  fi[q] = v - g2 * a2.dfm - g3 * a3.dfm;
  fi[q + tj] = v + g2 * a2.dfp - g3 * a3.dfm;
  fi[q + tk] = v - g2 * a2.dfm + g3 * a3.dfp;
  fi[q + tk + tj] = v + g2 * a2.dfp + g3 * a3.dfp;
}
ATHG_HD void smr_prolong_f2(const SmrDims& d, const double* co, double* fi, int k, int j, int i,
                            const SmrAxis& a1, const SmrAxis& a3) {
  const int fk = (k - d.cks) * 2 + d.ks, fj = (j - d.cjs) * 2 + d.js, fx = (i - d.cis) * 2 + d.is;
  const int64_t c = d.cf2i(k, j, i), sk = (int64_t)d.ncc1 * (d.ncc2 + 1);
  const double v = co[c];
  const double g1 = smr_minmod((v - co[c - 1]) / a1.dm, (co[c + 1] - v) / a1.dp);
  const double g3 = smr_minmod((v - co[c - sk]) / a3.dm, (co[c + sk] - v) / a3.dp);
  const int64_t q = d.f2(fk, fj, fx), tk = (int64_t)d.nc1 * (d.nc2 + 1);
  fi[q] = v - g1 * a1.dfm - g3 * a3.dfm;
  fi[q + 1] = v + g1 * a1.dfp - g3 * a3.dfm;
  fi[q + tk] = v - g1 * a1.dfm + g3 * a3.dfp;
  fi[q + tk + 1] = v + g1 * a1.dfp + g3 * a3.dfp;
}
ATHG_HD void smr_prolong_f3(const SmrDims& d, const double* co, double* fi, int k, int j, int i,
                            const SmrAxis& a1, const SmrAxis& a2) {
  const int fk = (k - d.cks) * 2 + d.ks, fj = (j - d.cjs) * 2 + d.js, fx = (i - d.cis) * 2 + d.is;
  const int64_t c = d.cf3i(k, j, i), sj = d.ncc1;
  const double v = co[c];
  const double g1 = smr_minmod((v - co[c - 1]) / a1.dm, (co[c + 1] - v) / a1.dp);
  const double g2 = smr_minmod((v - co[c - sj]) / a2.dm, (co[c + sj] - v) / a2.dp);
  const int64_t q = d.f3(fk, fj, fx), tj = d.nc1;
  fi[q] = v - g1 * a1.dfm - g2 * a2.dfm;
  fi[q + 1] = v + g1 * a1.dfp - g2 * a2.dfm;
  fi[q + tj] = v - g1 * a1.dfm + g2 * a2.dfp;
  fi[q + tj + 1] = v + g1 * a1.dfp + g2 * a2.dfp;
}

// ProlongateInternalField, 3-D (mesh_refinement.cpp:831-944): the twelve fine faces inside
// coarse cell (k,j,i) from the fine faces on its surface (Toth & Roe 2002), uniform
// Cartesian areas a1 = dx2 dx3, a2 = dx1 dx3, a3 = dx1 dx2
ATHG_HD void smr_prolong_internal(const SmrDims& d, double* b1, double* b2, double* b3, int k,
                                  int j, int i, const double dx[3]) {
  const int fk = (k - d.cks) * 2 + d.ks, fj = (j - d.cjs) * 2 + d.js, fi = (i - d.cis) * 2 + d.is;
  const double a1 = dx[1] * dx[2], a2 = dx[0] * dx[2], a3 = dx[0] * dx[1];
  double Uxx = 0.0, Vyy = 0.0, Wzz = 0.0, Uxyz = 0.0, Vxyz = 0.0, Wxyz = 0.0;
  for (int jj = 0; jj < 2; jj++) {
    const int sj = 2 * jj - 1, fjj = fj + jj, fjp = fj + 2 * jj;
    for (int ii = 0; ii < 2; ii++) {
      const int si = 2 * ii - 1, fii = fi + ii, fip = fi + 2 * ii;
      const double x2lo = b2[d.f2(fk, fjp, fii)] * a2, x2hi = b2[d.f2(fk + 1, fjp, fii)] * a2;
      const double x3lo = b3[d.f3(fk, fjj, fii)] * a3, x3hi = b3[d.f3(fk + 2, fjj, fii)] * a3;
      const double x1lo = b1[d.f1(fk, fjj, fip)] * a1, x1hi = b1[d.f1(fk + 1, fjj, fip)] * a1;
      Uxx += si * (sj * (x2lo + x2hi) + (x3hi - x3lo));
      Vyy += sj * ((x3hi - x3lo) + si * (x1lo + x1hi));
      Wzz += si * (x1hi - x1lo) + sj * (x2hi - x2lo);
      Uxyz += si * sj * (x1hi - x1lo);
      Vxyz += si * sj * (x2hi - x2lo);
      Wxyz += si * sj * (x3hi - x3lo);
    }
  }
  const double s1 = (dx[0] + dx[0]) * (dx[0] + dx[0]);
  const double s2 = (dx[1] + dx[1]) * (dx[1] + dx[1]);
  const double s3 = (dx[2] + dx[2]) * (dx[2] + dx[2]);
  Uxx *= 0.125; Vyy *= 0.125; Wzz *= 0.125;
  Uxyz *= 0.125 / (s2 + s3);
  Vxyz *= 0.125 / (s1 + s3);
  Wxyz *= 0.125 / (s1 + s2);
  auto B1 = [&](int kk, int jj, int ii) -> double& { return b1[d.f1(kk, jj, ii)]; };
  auto B2 = [&](int kk, int jj, int ii) -> double& { return b2[d.f2(kk, jj, ii)]; };
  auto B3 = [&](int kk, int jj, int ii) -> double& { return b3[d.f3(kk, jj, ii)]; };
  B1(fk, fj, fi + 1) =
      (0.5 * (B1(fk, fj, fi) * a1 + B1(fk, fj, fi + 2) * a1) + Uxx - s3 * Vxyz - s2 * Wxyz) / a1;
  B1(fk, fj + 1, fi + 1) = (0.5 * (B1(fk, fj + 1, fi) * a1 + B1(fk, fj + 1, fi + 2) * a1) + Uxx -
                            s3 * Vxyz + s2 * Wxyz) / a1;
  B1(fk + 1, fj, fi + 1) = (0.5 * (B1(fk + 1, fj, fi) * a1 + B1(fk + 1, fj, fi + 2) * a1) + Uxx +
                            s3 * Vxyz - s2 * Wxyz) / a1;
  B1(fk + 1, fj + 1, fi + 1) = (0.5 * (B1(fk + 1, fj + 1, fi) * a1 +
                                       B1(fk + 1, fj + 1, fi + 2) * a1) + Uxx + s3 * Vxyz +
                                s2 * Wxyz) / a1;
  B2(fk, fj + 1, fi) =
      (0.5 * (B2(fk, fj, fi) * a2 + B2(fk, fj + 2, fi) * a2) + Vyy - s3 * Uxyz - s1 * Wxyz) / a2;
  B2(fk, fj + 1, fi + 1) = (0.5 * (B2(fk, fj, fi + 1) * a2 + B2(fk, fj + 2, fi + 1) * a2) + Vyy -
                            s3 * Uxyz + s1 * Wxyz) / a2;
  B2(fk + 1, fj + 1, fi) = (0.5 * (B2(fk + 1, fj, fi) * a2 + B2(fk + 1, fj + 2, fi) * a2) + Vyy +
                            s3 * Uxyz - s1 * Wxyz) / a2;
  B2(fk + 1, fj + 1, fi + 1) = (0.5 * (B2(fk + 1, fj, fi + 1) * a2 +
                                       B2(fk + 1, fj + 2, fi + 1) * a2) + Vyy + s3 * Uxyz +
                                s1 * Wxyz) / a2;
  B3(fk + 1, fj, fi) =
      (0.5 * (B3(fk + 2, fj, fi) * a3 + B3(fk, fj, fi) * a3) + Wzz - s2 * Uxyz - s1 * Vxyz) / a3;
  B3(fk + 1, fj, fi + 1) = (0.5 * (B3(fk + 2, fj, fi + 1) * a3 + B3(fk, fj, fi + 1) * a3) + Wzz -
                            s2 * Uxyz + s1 * Vxyz) / a3;
  B3(fk + 1, fj + 1, fi) = (0.5 * (B3(fk + 2, fj + 1, fi) * a3 + B3(fk, fj + 1, fi) * a3) + Wzz +
                            s2 * Uxyz - s1 * Vxyz) / a3;
  B3(fk + 1, fj + 1, fi + 1) = (0.5 * (B3(fk + 2, fj + 1, fi + 1) * a3 +
                                       B3(fk, fj + 1, fi + 1) * a3) + Wzz + s2 * Uxyz +
                                s1 * Vxyz) / a3;
}

// Cell-centred field of one cell from its faces, uniform weights 0.5
// (field/field.cpp:117-160); comp stride ns
ATHG_HD void smr_bcc(double* bcc, int64_t ns, int64_t c, const double* b1, int64_t q1,
                     const double* b2, int64_t q2, int64_t s2, const double* b3, int64_t q3,
                     int64_t s3) {
  bcc[c] = 0.5 * b1[q1] + 0.5 * b1[q1 + 1];
  bcc[ns + c] = 0.5 * b2[q2] + 0.5 * b2[q2 + s2];
  bcc[2 * ns + c] = 0.5 * b3[q3] + 0.5 * b3[q3 + s3];
}

// EquationOfState::ConservedToPrimitive of one cell (eos/adiabatic_mhd.cpp,
// eos/adiabatic_hydro.cpp; the arithmetic of the FP64 stage's k_c2p). bc: cell-centred
// field (MHD) or nullptr; u and w: component stride ns
ATHG_HD void smr_c2p(double* u, double* w, int64_t ns, int64_t c, const double* bc,
                     double gamma, double dfloor, double pfloor) {
  const double gm1 = gamma - 1.0;
  double pb = 0.0;
  if (bc) pb = 0.5 * (bc[c] * bc[c] + bc[ns + c] * bc[ns + c] + bc[2 * ns + c] * bc[2 * ns + c]);
  double ud = u[c];
  const double m1 = u[ns + c], m2 = u[2 * ns + c], m3 = u[3 * ns + c], ue = u[4 * ns + c];
  ud = (ud > dfloor) ? ud : dfloor;
  u[c] = ud;
  const double di = 1.0 / ud;
  const double e_k = 0.5 * di * (m1 * m1 + m2 * m2 + m3 * m3);
  double wp = bc ? gm1 * (ue - e_k - pb) : gm1 * (ue - e_k);
  if (!(wp > pfloor)) {
    u[4 * ns + c] = bc ? ((pfloor / gm1) + e_k + pb) : ((pfloor / gm1) + e_k);
    wp = pfloor;
  }
  w[c] = ud;
  w[ns + c] = m1 * di;
  w[2 * ns + c] = m2 * di;
  w[3 * ns + c] = m3 * di;
  w[4 * ns + c] = wp;
}

// EquationOfState::PrimitiveToConserved of one cell (eos/adiabatic_mhd.cpp:99-136,
// eos/adiabatic_hydro.cpp:89-118)
ATHG_HD void smr_p2c(const double* w, double* u, int64_t ns, int64_t c, const double* bc,
                     double igm1) {
  const double d = w[c], vx = w[ns + c], vy = w[2 * ns + c], vz = w[3 * ns + c],
               p = w[4 * ns + c];
  u[c] = d;
  u[ns + c] = vx * d;
  u[2 * ns + c] = vy * d;
  u[3 * ns + c] = vz * d;
  if (bc) {
    const double b1 = bc[c], b2 = bc[ns + c], b3 = bc[2 * ns + c];
    u[4 * ns + c] = p * igm1 + 0.5 * (d * (vx * vx + vy * vy + vz * vz) +
                                      (b1 * b1 + b2 * b2 + b3 * b3));
  } else {
    u[4 * ns + c] = p * igm1 + 0.5 * d * (vx * vx + vy * vy + vz * vz);
  }
}


// ---- one work-list entry --------------------------------------------------------------
// Base pointers of every block's arrays (FP64 path): cell arrays [nb][ncomp][cells],
// faces [nb][faces], fluxes [nb][nflx][faces_d], edges [nb][3][edges], widths [nb][3],
// cell centres [nb][3][ncmax] (fine) and [nb][3][nccmax] (coarse buffer).
struct SmrPool {
  double *u, *w, *b1, *b2, *b3, *bcc;
  double *cu, *cw, *cb1, *cb2, *cb3, *cbcc;
  double* flx[3];
  int nflx;
  double* edge;
  // mixed path: the face fluxes and edge EMFs are FP32 (flx / edge then unused); w and bcc
  // are FP64 scratch for the prolongated ghost cells
  float* flx32[3];
  float* edge32;
  const double *dx, *xvf, *xvc;
  int ncmax, nccmax;
  double gamma, dfloor, pfloor;
  int mhd;
};

ATHG_HD void smr_exec_xfer(const SmrDims& d, const SmrPool& P, const SmrXfer& x) {
  const double* dxs = P.dx + 3 * x.sblk;
  if (x.darr == SA_U || x.darr == SA_CU) {
    const int64_t ds = x.darr == SA_U ? d.ncell : d.ccell;
    double* dst = (x.darr == SA_U ? P.u : P.cu) + (int64_t)x.dblk * 5 * ds;
    const double* src = P.u + (int64_t)x.sblk * 5 * d.ncell;
    if (x.op == SO_COPY) {
      for (int n = 0; n < 5; ++n) dst[n * ds + x.didx] = src[n * d.ncell + x.sidx];
    } else {
      const double vol = dxs[0] * dxs[1] * dxs[2];
      for (int n = 0; n < 5; ++n)
        dst[n * ds + x.didx] = smr_restrict_cc(d, src + n * d.ncell, x.sidx, vol);
    }
    return;
  }
  const int f = (x.darr - 1) & 3;  // face component 0..2
  const bool coarse = x.darr >= SA_CB1;
  double* dst;
  const double* src;
  if (f == 0) {
    dst = coarse ? P.cb1 + (int64_t)x.dblk * d.cf1 : P.b1 + (int64_t)x.dblk * d.nf1;
    src = P.b1 + (int64_t)x.sblk * d.nf1;
  } else if (f == 1) {
    dst = coarse ? P.cb2 + (int64_t)x.dblk * d.cf2 : P.b2 + (int64_t)x.dblk * d.nf2;
    src = P.b2 + (int64_t)x.sblk * d.nf2;
  } else {
    dst = coarse ? P.cb3 + (int64_t)x.dblk * d.cf3 : P.b3 + (int64_t)x.dblk * d.nf3;
    src = P.b3 + (int64_t)x.sblk * d.nf3;
  }
  if (x.op == SO_COPY) dst[x.didx] = src[x.sidx];
  else if (x.op == SO_RF1) dst[x.didx] = smr_restrict_f1(d, src, x.sidx, dxs[1] * dxs[2]);
  else if (x.op == SO_RF2) dst[x.didx] = smr_restrict_f2(d, src, x.sidx, dxs[0] * dxs[2]);
  else dst[x.didx] = smr_restrict_f3(d, src, x.sidx, dxs[0] * dxs[1]);
}

// hydro flux components of a coarse face from the area-weighted fine fluxes
template <typename F>
ATHG_HD void smr_flux_typed(const SmrDims& d, F* base, int nflx, const double* dx,
                            const SmrFlux& f) {
  const int64_t nf = f.dir == 0 ? d.nf1 : (f.dir == 1 ? d.nf2 : d.nf3);
  const double* dxs = dx + 3 * f.sblk;
  F* dst = base + (int64_t)f.dblk * nflx * nf;
  const F* src = base + (int64_t)f.sblk * nflx * nf;
  for (int n = 0; n < 5; ++n) {
    double v;
    if (f.dir == 0) v = smr_restrict_f1(d, src + n * nf, f.sidx, dxs[1] * dxs[2]);
    else if (f.dir == 1) v = smr_restrict_f2(d, src + n * nf, f.sidx, dxs[0] * dxs[2]);
    else v = smr_restrict_f3(d, src + n * nf, f.sidx, dxs[0] * dxs[1]);
    dst[n * nf + f.didx] = (F)v;
  }
}
ATHG_HD void smr_exec_flux(const SmrDims& d, const SmrPool& P, const SmrFlux& f) {
  if (P.flx32[f.dir]) smr_flux_typed(d, P.flx32[f.dir], P.nflx, P.dx, f);
  else smr_flux_typed(d, P.flx[f.dir], P.nflx, P.dx, f);
}

// corrected value of one block-boundary edge (reads the uncorrected EMFs only)
template <typename F>
ATHG_HD double smr_emf_typed(const SmrDims& d, const F* edge, const SmrEmf& e,
                             const SmrEmfAdd* adds) {
  double v = e.own ? (double)edge[((int64_t)e.blk * 3 + e.comp) * d.ne + e.idx] : 0.0;
  for (int a = e.add0; a < e.add1; ++a) {
    const SmrEmfAdd& x = adds[a];
    const F* s = edge + ((int64_t)x.sblk * 3 + x.comp) * d.ne;
    if (x.step == 0) v += (double)s[x.idx];
    else v += ((double)s[x.idx] * x.len + (double)s[x.idx + x.step] * x.len) / (x.len + x.len);
  }
  v *= e.mul[0];
  v *= e.mul[1];
  return v;
}
// (the mixed path sums and scales the FP32 EMFs in FP64 and rounds once when storing)
ATHG_HD double smr_exec_emf(const SmrDims& d, const SmrPool& P, const SmrEmf& e,
                            const SmrEmfAdd* adds) {
  return P.edge32 ? smr_emf_typed(d, P.edge32, e, adds) : smr_emf_typed(d, P.edge, e, adds);
}

// coarse bcc and W(U) of one coarse-buffer cell
ATHG_HD void smr_exec_c2p(const SmrDims& d, const SmrPool& P, const SmrPos& p) {
  const int64_t c = d.cc(p.k, p.j, p.i);
  double* bc = nullptr;
  if (P.mhd) {
    bc = P.cbcc + (int64_t)p.blk * 3 * d.ccell;
    smr_bcc(bc, d.ccell, c, P.cb1 + (int64_t)p.blk * d.cf1, d.cf1i(p.k, p.j, p.i),
            P.cb2 + (int64_t)p.blk * d.cf2, d.cf2i(p.k, p.j, p.i), d.ncc1,
            P.cb3 + (int64_t)p.blk * d.cf3, d.cf3i(p.k, p.j, p.i), (int64_t)d.ncc1 * d.ncc2);
  }
  smr_c2p(P.cu + (int64_t)p.blk * 5 * d.ccell, P.cw + (int64_t)p.blk * 5 * d.ccell, d.ccell, c,
          bc, P.gamma, P.dfloor, P.pfloor);
}

// offsets along axis a (0: x1, 1: x2, 2: x3) at the coarse cell of position p. A shared
// face's index along its normal runs to the last coarse face, one past the last cell whose
// neighbours the coordinate rows hold, so face prolongation asks only for its two
// tangential axes.
ATHG_HD SmrAxis smr_axis_of(const SmrDims& d, const SmrPool& P, const SmrPos& p, int a) {
  const double* xf = P.xvf + ((int64_t)p.blk * 3 + a) * P.ncmax;
  const double* xc = P.xvc + ((int64_t)p.blk * 3 + a) * P.nccmax;
  if (a == 0) return smr_axis(xc, xf, p.i, (p.i - d.cis) * 2 + d.is);
  if (a == 1) return smr_axis(xc, xf, p.j, (p.j - d.cjs) * 2 + d.js);
  return smr_axis(xc, xf, p.k, (p.k - d.cks) * 2 + d.ks);
}
ATHG_HD void smr_axes(const SmrDims& d, const SmrPool& P, const SmrPos& p, SmrAxis ax[3]) {
  for (int a = 0; a < 3; ++a) ax[a] = smr_axis_of(d, P, p, a);
}

// prolongated primitives of one coarse cell
ATHG_HD void smr_exec_pcc(const SmrDims& d, const SmrPool& P, const SmrPos& p) {
  SmrAxis ax[3];
  smr_axes(d, P, p, ax);
  const double* cw = P.cw + (int64_t)p.blk * 5 * d.ccell;
  double* w = P.w + (int64_t)p.blk * 5 * d.ncell;
  for (int n = 0; n < 5; ++n)
    smr_prolong_cc(d, cw + n * d.ccell, w + n * d.ncell, p.k, p.j, p.i, ax[0], ax[1], ax[2]);
}

// prolongated shared faces of one coarse face of component f
ATHG_HD void smr_exec_psf(const SmrDims& d, const SmrPool& P, int f, const SmrPos& p) {
  if (f == 0)
    smr_prolong_f1(d, P.cb1 + (int64_t)p.blk * d.cf1, P.b1 + (int64_t)p.blk * d.nf1, p.k, p.j,
                   p.i, smr_axis_of(d, P, p, 1), smr_axis_of(d, P, p, 2));
  else if (f == 1)
    smr_prolong_f2(d, P.cb2 + (int64_t)p.blk * d.cf2, P.b2 + (int64_t)p.blk * d.nf2, p.k, p.j,
                   p.i, smr_axis_of(d, P, p, 0), smr_axis_of(d, P, p, 2));
  else
    smr_prolong_f3(d, P.cb3 + (int64_t)p.blk * d.cf3, P.b3 + (int64_t)p.blk * d.nf3, p.k, p.j,
                   p.i, smr_axis_of(d, P, p, 0), smr_axis_of(d, P, p, 1));
}

ATHG_HD void smr_exec_pint(const SmrDims& d, const SmrPool& P, const SmrPos& p) {
  smr_prolong_internal(d, P.b1 + (int64_t)p.blk * d.nf1, P.b2 + (int64_t)p.blk * d.nf2,
                       P.b3 + (int64_t)p.blk * d.nf3, p.k, p.j, p.i, P.dx + 3 * p.blk);
}

// bcc and U(W) of one prolongated fine cell
ATHG_HD void smr_exec_pfine(const SmrDims& d, const SmrPool& P, const SmrPos& p) {
  const int64_t c = d.c(p.k, p.j, p.i);
  double* bc = nullptr;
  if (P.mhd) {
    bc = P.bcc + (int64_t)p.blk * 3 * d.ncell;
    smr_bcc(bc, d.ncell, c, P.b1 + (int64_t)p.blk * d.nf1, d.f1(p.k, p.j, p.i),
            P.b2 + (int64_t)p.blk * d.nf2, d.f2(p.k, p.j, p.i), d.nc1,
            P.b3 + (int64_t)p.blk * d.nf3, d.f3(p.k, p.j, p.i), (int64_t)d.nc1 * d.nc2);
  }
  smr_p2c(P.w + (int64_t)p.blk * 5 * d.ncell, P.u + (int64_t)p.blk * 5 * d.ncell, d.ncell, c, bc,
          1.0 / (P.gamma - 1.0));
}

}  // namespace athg

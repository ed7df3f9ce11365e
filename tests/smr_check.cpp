// smr_check.cpp -- CPU run of the SMR work lists (test infrastructure).
//
// Builds the plan of athg_smr_plan.cpp for a multi-level block list, loads the blocks'
// interiors, and runs the ghost fill, the prolongation and W(U) over every block with the
// same per-entry functions the CUDA kernels use (athg_smr.h), on host arrays. The tests
// compare the result, ghost zones included, with the reference's state after
// Mesh::Initialize on the same mesh.
//
// usage: smr_check <in.bin> <out.bin>
//   in : int32 nx1 nx2 nx3 ng mesh_nx1 mesh_nx2 mesh_nx3 mhd nblocks;
//        float64 x1min x1max x2min x2max x3min x3max gamma dfloor pfloor;
//        per block int64 level lx1 lx2 lx3, then interior U[5][nx3][nx2][nx1] and with MHD
//        B1f[nx3][nx2][nx1+1] B2f[nx3][nx2+1][nx1] B3f[nx3+1][nx2][nx1]
//   out: per block (input order) U[5][nc3][nc2][nc1], W[5][...], B1f, B2f, B3f with ghosts;
//        then int64 sizes of the work lists (xfer, pre, flux, emf, c2p, pcc, pint, pfine)
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "athg_smr.h"

using namespace athg;

static void rd(FILE* f, void* p, size_t sz, size_t n) {
  if (fread(p, sz, n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}

int main(int argc, char** argv) {
  if (argc != 3) { fprintf(stderr, "usage: smr_check in out\n"); return 2; }
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 2;
  int32_t h[9];
  rd(f, h, 4, 9);
  double dd[9];
  rd(f, dd, 8, 9);
  const int nx[3] = {h[0], h[1], h[2]}, ng = h[3], mnx[3] = {h[4], h[5], h[6]};
  const bool mhd = h[7] != 0;
  const int nb = h[8];
  const SmrDims d = smr_dims(nx[0], nx[1], nx[2], ng);
  int nrb[3];
  for (int a = 0; a < 3; ++a) nrb[a] = mnx[a] / nx[a];
  std::vector<SmrLoc> loc(nb);
  std::vector<double> u((size_t)nb * 5 * d.ncell, 0.0), w(u.size(), 0.0);
  std::vector<double> b1((size_t)nb * d.nf1, 0.0), b2((size_t)nb * d.nf2, 0.0),
      b3((size_t)nb * d.nf3, 0.0), bcc((size_t)nb * 3 * d.ncell, 0.0);
  std::vector<double> cu((size_t)nb * 5 * d.ccell, 0.0), cw(cu.size(), 0.0),
      cb1((size_t)nb * d.cf1, 0.0), cb2((size_t)nb * d.cf2, 0.0), cb3((size_t)nb * d.cf3, 0.0),
      cbcc((size_t)nb * 3 * d.ccell, 0.0);
  const int ncmax = std::max(d.nc1, std::max(d.nc2, d.nc3));
  const int nccmax = std::max(d.ncc1, std::max(d.ncc2, d.ncc3));
  std::vector<double> dx((size_t)nb * 3), xvf((size_t)nb * 3 * ncmax), xvc((size_t)nb * 3 * nccmax);
  for (int b = 0; b < nb; ++b) {
    int64_t l[4];
    rd(f, l, 8, 4);
    loc[b].level = (int)l[0];
    for (int a = 0; a < 3; ++a) loc[b].lx[a] = l[1 + a];
    for (int a = 0; a < 3; ++a)
      smr_axis_coords(mnx[a], nrb[a], dd[2 * a], dd[2 * a + 1], loc[b].level, loc[b].lx[a], nx[a], ng,
                      &dx[3 * b + a], &xvf[((size_t)b * 3 + a) * ncmax],
                      &xvc[((size_t)b * 3 + a) * nccmax], nullptr);
    for (int n = 0; n < 5; ++n)
      for (int k = d.ks; k <= d.ke; ++k)
        for (int j = d.js; j <= d.je; ++j)
          for (int i = d.is; i <= d.ie; ++i) rd(f, &u[((size_t)b * 5 + n) * d.ncell + d.c(k, j, i)], 8, 1);
    if (mhd) {
      for (int k = d.ks; k <= d.ke; ++k)
        for (int j = d.js; j <= d.je; ++j)
          for (int i = d.is; i <= d.ie + 1; ++i) rd(f, &b1[(size_t)b * d.nf1 + d.f1(k, j, i)], 8, 1);
      for (int k = d.ks; k <= d.ke; ++k)
        for (int j = d.js; j <= d.je + 1; ++j)
          for (int i = d.is; i <= d.ie; ++i) rd(f, &b2[(size_t)b * d.nf2 + d.f2(k, j, i)], 8, 1);
      for (int k = d.ks; k <= d.ke + 1; ++k)
        for (int j = d.js; j <= d.je; ++j)
          for (int i = d.is; i <= d.ie; ++i) rd(f, &b3[(size_t)b * d.nf3 + d.f3(k, j, i)], 8, 1);
    }
  }
  fclose(f);
  SmrPlan plan;
  std::string err;
  if (!smr_plan(d, nrb, loc, dx.data(), mhd, &plan, &err)) {
    fprintf(stderr, "plan: %s\n", err.c_str());
    return 3;
  }
  SmrPool P{};
  P.u = u.data(); P.w = w.data(); P.b1 = b1.data(); P.b2 = b2.data(); P.b3 = b3.data();
  P.bcc = bcc.data();
  P.cu = cu.data(); P.cw = cw.data(); P.cb1 = cb1.data(); P.cb2 = cb2.data(); P.cb3 = cb3.data();
  P.cbcc = cbcc.data();
  P.flx[0] = P.flx[1] = P.flx[2] = nullptr; P.nflx = 0; P.edge = nullptr;
  P.dx = dx.data(); P.xvf = xvf.data(); P.xvc = xvc.data(); P.ncmax = ncmax; P.nccmax = nccmax;
  P.gamma = dd[6]; P.dfloor = dd[7]; P.pfloor = dd[8]; P.mhd = mhd ? 1 : 0;
  // Mesh::Initialize: ghost fill, prolongation, W(U) over every cell
  for (const SmrXfer& x : plan.xfer) smr_exec_xfer(d, P, x);
  for (const SmrXfer& x : plan.pre) smr_exec_xfer(d, P, x);
  for (const SmrPos& p : plan.c2p) smr_exec_c2p(d, P, p);
  for (const SmrPos& p : plan.pcc) smr_exec_pcc(d, P, p);
  if (mhd) {
    for (int c = 0; c < 3; ++c)
      for (const SmrPos& p : plan.psf[c]) smr_exec_psf(d, P, c, p);
    for (const SmrPos& p : plan.pint) smr_exec_pint(d, P, p);
  }
  for (const SmrPos& p : plan.pfine) smr_exec_pfine(d, P, p);
  for (int b = 0; b < nb; ++b)
    for (int k = 0; k < d.nc3; ++k)
      for (int j = 0; j < d.nc2; ++j)
        for (int i = 0; i < d.nc1; ++i) {
          SmrPos p{b, k, j, i};
          double* bc = nullptr;
          const int64_t c = d.c(k, j, i);
          if (mhd) {
            bc = P.bcc + (int64_t)b * 3 * d.ncell;
            smr_bcc(bc, d.ncell, c, P.b1 + (int64_t)b * d.nf1, d.f1(k, j, i), P.b2 + (int64_t)b * d.nf2,
                    d.f2(k, j, i), d.nc1, P.b3 + (int64_t)b * d.nf3, d.f3(k, j, i),
                    (int64_t)d.nc1 * d.nc2);
          }
          (void)p;
          smr_c2p(P.u + (int64_t)b * 5 * d.ncell, P.w + (int64_t)b * 5 * d.ncell, d.ncell, c, bc,
                  P.gamma, P.dfloor, P.pfloor);
        }
  FILE* o = fopen(argv[2], "wb");
  if (!o) return 2;
  for (int b = 0; b < nb; ++b) {
    fwrite(&u[(size_t)b * 5 * d.ncell], 8, 5 * d.ncell, o);
    fwrite(&w[(size_t)b * 5 * d.ncell], 8, 5 * d.ncell, o);
    if (mhd) {
      fwrite(&b1[(size_t)b * d.nf1], 8, d.nf1, o);
      fwrite(&b2[(size_t)b * d.nf2], 8, d.nf2, o);
      fwrite(&b3[(size_t)b * d.nf3], 8, d.nf3, o);
    }
  }
  int64_t sz[8] = {(int64_t)plan.xfer.size(), (int64_t)plan.pre.size(), (int64_t)plan.flux.size(),
                   (int64_t)plan.emf.size(), (int64_t)plan.c2p.size(), (int64_t)plan.pcc.size(),
                   (int64_t)plan.pint.size(), (int64_t)plan.pfine.size()};
  fwrite(sz, 8, 8, o);
  fclose(o);
  return 0;
}

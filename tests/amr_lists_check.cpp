// amr_lists_check.cpp -- CPU walk of every level-boundary work list through random adaptive
// refinement sequences (test infrastructure), built with AddressSanitizer and UBSan by
// tests/test_sanitized_host.py.
//
// Each sequence starts from a uniform root of blocks and applies random refine / derefine
// flags for several passes (amr_update_tree keeps 2:1 balance, amr_fill makes the new
// blocks' arrays). After every regrid the mesh is planned (smr_plan) and every list runs
// with the per-entry functions the CUDA kernels use (athg_smr.h) on host arrays allocated
// one array per device allocation and with exactly the sizes the device allocates
// (block pool arrays [nb][...], coarse buffers, fluxes [nb][nflx][faces], edges
// [nb][3][edges], widths and cell centres), so any index outside an allocation is
// reported by the sanitizer. In addition every entry's block indices and element indices
// are checked against one block's extent here, which also catches an index that stays
// inside the pool but leaves its block.
//
// usage: amr_lists_check <nx> <nghost> <mesh_nx> <max_level> <sequences> <passes> <mhd>
// prints one line per regrid and "checked <n> meshes" at the end; exits 1 on the first
// entry out of its block.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "athg_amr.h"

using namespace athg;

static uint64_t g_rng = 0x9e3779b97f4a7c15ull;
static double urand() {
  g_rng = g_rng * 6364136223846793005ull + 1442695040888963407ull;
  return (double)(g_rng >> 11) * (1.0 / 9007199254740992.0);
}

static int g_bad = 0;
static void bad(const char* what, long long a, long long b) {
  if (g_bad++ < 20) fprintf(stderr, "out of range: %s %lld (limit %lld)\n", what, a, b);
}
static void in_range(const char* what, long long v, long long lo, long long hi) {
  if (v < lo || v >= hi) bad(what, v, v < lo ? lo : hi);
}

struct Pool {
  std::vector<double> u, w, b1, b2, b3, bcc, cu, cw, cb1, cb2, cb3, cbcc, f[3], edge;
  std::vector<double> dx, xvf, xvc;
};

static void coords(const SmrDims& d, int mnx, int nx, const std::vector<SmrLoc>& L,
                   std::vector<double>* dx, std::vector<double>* xvf, std::vector<double>* xvc,
                   int* ncmax, int* nccmax) {
  *ncmax = d.nc1;
  *nccmax = nx / 2 + 2 * d.ng;
  dx->assign(L.size() * 3, 0.0);
  xvf->assign(L.size() * 3 * *ncmax, 0.0);
  xvc->assign(L.size() * 3 * *nccmax, 0.0);
  for (size_t b = 0; b < L.size(); ++b)
    for (int a = 0; a < 3; ++a)
      smr_axis_coords(mnx, mnx / nx, -1.0, 1.0, L[b].level, L[b].lx[a], nx, d.ng,
                      &(*dx)[3 * b + a], &(*xvf)[(b * 3 + a) * *ncmax],
                      &(*xvc)[(b * 3 + a) * *nccmax], nullptr);
}

// element checks per entry (a block's own extent; the sanitizer checks the allocations).
// A position's index along axis a, as a coarse (c) or fine (f) index, must lie in [lo, hi).
static void axis_range(const char* what, int v, int lo, int hi) { in_range(what, v, lo, hi); }
static int fine_of(int c, int cs, int s) { return (c - cs) * 2 + s; }

static void check_lists(const SmrDims& d, const SmrPlan& plan, int nb, bool mhd) {
  const int ncc[3] = {d.ncc1, d.ncc2, d.ncc3}, nc[3] = {d.nc1, d.nc2, d.nc3};
  const int cs[3] = {d.cis, d.cjs, d.cks}, fs[3] = {d.is, d.js, d.ks};
  auto pos = [](const SmrPos& p, int a) { return a == 0 ? p.i : (a == 1 ? p.j : p.k); };
  const int64_t fsz[3] = {d.nf1, d.nf2, d.nf3}, cfsz[3] = {d.cf1, d.cf2, d.cf3};
  // element transfers: destination inside the destination grid, the source's restriction
  // stencil (lower corner plus one cell or face along the restricted axes) inside the block
  auto xfer = [&](const SmrXfer& x, const char* nm) {
    in_range(nm, x.dblk, 0, nb);
    in_range(nm, x.sblk, 0, nb);
    const bool coarse = x.darr >= SA_CU;
    if (x.darr == SA_U || x.darr == SA_CU) {
      in_range("xfer cell didx", x.didx, 0, coarse ? d.ccell : d.ncell);
      const int64_t top = x.op == SO_COPY ? x.sidx
                                          : x.sidx + (int64_t)d.nc1 * d.nc2 + d.nc1 + 1;
      in_range("xfer cell sidx", x.sidx, 0, d.ncell);
      in_range("xfer cell stencil", top, 0, d.ncell);
      return;
    }
    const int f = (x.darr - 1) & 3;
    in_range("xfer face didx", x.didx, 0, coarse ? cfsz[f] : fsz[f]);
    in_range("xfer face sidx", x.sidx, 0, fsz[f]);
    int64_t top = x.sidx;
    if (x.op == SO_RF1) top += (int64_t)(d.nc1 + 1) * d.nc2 + (d.nc1 + 1);
    else if (x.op == SO_RF2) top += (int64_t)d.nc1 * (d.nc2 + 1) + 1;
    else if (x.op == SO_RF3) top += d.nc1 + 1;
    in_range("xfer face stencil", top, 0, fsz[f]);
  };
  for (const SmrXfer& x : plan.xfer) xfer(x, "xfer block");
  for (const SmrXfer& x : plan.pre) xfer(x, "pre block");
  for (const SmrPos& p : plan.c2p) {
    in_range("c2p block", p.blk, 0, nb);
    for (int a = 0; a < 3; ++a) axis_range("c2p", pos(p, a), 0, ncc[a]);
  }
  // prolongation of a coarse cell: neighbours on both sides, eight fine cells
  for (const SmrPos& p : plan.pcc) {
    in_range("pcc block", p.blk, 0, nb);
    for (int a = 0; a < 3; ++a) {
      axis_range("pcc coarse", pos(p, a), 1, ncc[a] - 1);
      axis_range("pcc fine", fine_of(pos(p, a), cs[a], fs[a]), 0, nc[a] - 1);
    }
  }
  // shared faces: the normal index runs over faces, the two tangential ones need both
  // neighbours and write two fine faces each
  for (int f = 0; f < 3; ++f)
    for (const SmrPos& p : plan.psf[f]) {
      in_range("psf block", p.blk, 0, nb);
      for (int a = 0; a < 3; ++a) {
        const int c = pos(p, a), fi = fine_of(c, cs[a], fs[a]);
        if (a == f) {
          axis_range("psf normal coarse", c, 0, ncc[a] + 1);
          axis_range("psf normal fine", fi, 0, nc[a] + 1);
        } else {
          axis_range("psf tangential coarse", c, 1, ncc[a] - 1);
          axis_range("psf tangential fine", fi, 0, nc[a] - 1);
        }
      }
    }
  // internal field: the fine faces of the coarse cell, normal index up to fine + 2
  for (const SmrPos& p : plan.pint) {
    in_range("pint block", p.blk, 0, nb);
    for (int a = 0; a < 3; ++a) {
      axis_range("pint coarse", pos(p, a), 0, ncc[a]);
      axis_range("pint fine", fine_of(pos(p, a), cs[a], fs[a]), 0, nc[a] - 1);
    }
  }
  for (const SmrPos& p : plan.pfine) {
    in_range("pfine block", p.blk, 0, nb);
    for (int a = 0; a < 3; ++a) axis_range("pfine", pos(p, a), 0, nc[a]);
  }
  for (const SmrFlux& f : plan.flux) {
    in_range("flux dblk", f.dblk, 0, nb);
    in_range("flux sblk", f.sblk, 0, nb);
    in_range("flux dir", f.dir, 0, 3);
    if (f.dir < 0 || f.dir > 2) continue;
    in_range("flux didx", f.didx, 0, fsz[f.dir]);
    int64_t top = f.sidx;
    if (f.dir == 0) top += (int64_t)(d.nc1 + 1) * d.nc2 + (d.nc1 + 1);
    else if (f.dir == 1) top += (int64_t)d.nc1 * (d.nc2 + 1) + 1;
    else top += d.nc1 + 1;
    in_range("flux sidx", f.sidx, 0, fsz[f.dir]);
    in_range("flux stencil", top, 0, fsz[f.dir]);
  }
  if (!mhd) return;
  for (const SmrEmf& e : plan.emf) {
    in_range("emf blk", e.blk, 0, nb);
    in_range("emf comp", e.comp, 0, 3);
    in_range("emf idx", e.idx, 0, d.ne);
    in_range("emf add0", e.add0, 0, (long long)plan.emf_add.size() + 1);
    in_range("emf add1", e.add1, e.add0, (long long)plan.emf_add.size() + 1);
  }
  for (const SmrEmfAdd& a : plan.emf_add) {
    in_range("emf_add sblk", a.sblk, 0, nb);
    in_range("emf_add comp", a.comp, 0, 3);
    in_range("emf_add idx", a.idx, 0, d.ne);
    in_range("emf_add idx+step", (long long)a.idx + a.step, 0, d.ne);
  }
}

static void run_lists(const SmrDims& d, const SmrPlan& plan, int nb, bool mhd, Pool& A,
                      int ncmax, int nccmax) {
  check_lists(d, plan, nb, mhd);
  SmrPool P{};
  P.u = A.u.data(); P.w = A.w.data(); P.b1 = mhd ? A.b1.data() : nullptr;
  P.b2 = mhd ? A.b2.data() : nullptr; P.b3 = mhd ? A.b3.data() : nullptr;
  P.bcc = mhd ? A.bcc.data() : nullptr;
  P.cu = A.cu.data(); P.cw = A.cw.data();
  P.cb1 = mhd ? A.cb1.data() : nullptr; P.cb2 = mhd ? A.cb2.data() : nullptr;
  P.cb3 = mhd ? A.cb3.data() : nullptr; P.cbcc = mhd ? A.cbcc.data() : nullptr;
  for (int f = 0; f < 3; ++f) P.flx[f] = A.f[f].data();
  P.nflx = mhd ? 8 : 5;
  P.edge = mhd ? A.edge.data() : nullptr;
  P.dx = A.dx.data(); P.xvf = A.xvf.data(); P.xvc = A.xvc.data();
  P.ncmax = ncmax; P.nccmax = nccmax;
  P.gamma = 5.0 / 3.0; P.dfloor = 1e-10; P.pfloor = 1e-10; P.mhd = mhd ? 1 : 0;
  // the order of a stage: ghost fill and prolongation, then flux and EMF corrections
  for (const SmrXfer& x : plan.xfer) smr_exec_xfer(d, P, x);
  for (const SmrXfer& x : plan.pre) smr_exec_xfer(d, P, x);
  for (const SmrPos& p : plan.c2p) smr_exec_c2p(d, P, p);
  for (const SmrPos& p : plan.pcc) smr_exec_pcc(d, P, p);
  if (mhd) {
    for (int f = 0; f < 3; ++f)
      for (const SmrPos& p : plan.psf[f]) smr_exec_psf(d, P, f, p);
    for (const SmrPos& p : plan.pint) smr_exec_pint(d, P, p);
  }
  for (const SmrPos& p : plan.pfine) smr_exec_pfine(d, P, p);
  for (const SmrFlux& f : plan.flux) smr_exec_flux(d, P, f);
  if (mhd) {
    std::vector<double> tmp(plan.emf.size());
    for (size_t q = 0; q < plan.emf.size(); ++q)
      tmp[q] = smr_exec_emf(d, P, plan.emf[q], plan.emf_add.data());
    for (size_t q = 0; q < plan.emf.size(); ++q) {
      const SmrEmf& e = plan.emf[q];
      A.edge[((size_t)e.blk * 3 + e.comp) * d.ne + e.idx] = tmp[q];
    }
  }
}

int main(int argc, char** argv) {
  if (argc != 8) {
    fprintf(stderr, "usage: amr_lists_check nx nghost mesh_nx max_level sequences passes mhd\n");
    return 2;
  }
  const int nx = atoi(argv[1]), ng = atoi(argv[2]), mnx = atoi(argv[3]);
  const int max_level = atoi(argv[4]), nseq = atoi(argv[5]), npass = atoi(argv[6]);
  const bool mhd = atoi(argv[7]) != 0;
  const SmrDims d = smr_dims(nx, nx, nx, ng);
  const int nr = mnx / nx;
  const int nrb[3] = {nr, nr, nr};
  long long checked = 0;
  for (int s = 0; s < nseq; ++s) {
    g_rng = 0x9e3779b97f4a7c15ull + 7919ull * (uint64_t)s;
    std::vector<SmrLoc> cur;
    for (int k = 0; k < nr; ++k)
      for (int j = 0; j < nr; ++j)
        for (int i = 0; i < nr; ++i) {
          SmrLoc l{};
          l.level = 0; l.lx[0] = i; l.lx[1] = j; l.lx[2] = k;
          cur.push_back(l);
        }
    AmrArrays A;
    const size_t nb0 = cur.size();
    A.u.assign(nb0 * 5 * d.ncell, 1.0);
    A.cu.assign(nb0 * 5 * d.ccell, 1.0);
    if (mhd) {
      A.b1.assign(nb0 * d.nf1, 0.1); A.b2.assign(nb0 * d.nf2, 0.2); A.b3.assign(nb0 * d.nf3, 0.3);
      A.cb1.assign(nb0 * d.cf1, 0.1); A.cb2.assign(nb0 * d.cf2, 0.2); A.cb3.assign(nb0 * d.cf3, 0.3);
    }
    for (size_t q = 0; q < A.u.size(); ++q) A.u[q] += 1e-3 * (double)(q % 97);
    std::vector<int> deref(cur.size(), 0);
    // refinement is likelier early in a sequence, derefinement later
    for (int pass = 0; pass < npass; ++pass) {
      const double pr = pass < npass / 2 ? 0.1 : 0.03, pd = pass < npass / 2 ? 0.05 : 0.3;
      // derefinement needs all eight siblings flagged: the decision is made per parent
      // (a hash of the parent's location and the pass), refinement per block
      std::vector<int> flags(cur.size(), 0);
      for (size_t b = 0; b < cur.size(); ++b) {
        const SmrLoc& l = cur[b];
        if (urand() < pr && l.level < max_level) {
          flags[b] = 1;
        } else if (l.level > 0) {
          uint64_t h = 0x243f6a8885a308d3ull ^ ((uint64_t)s << 40) ^ ((uint64_t)pass << 32) ^
                       ((uint64_t)l.level << 24);
          for (int a = 0; a < 3; ++a) h = (h ^ (uint64_t)(l.lx[a] >> 1)) * 0x100000001b3ull;
          h ^= h >> 29;
          if ((double)(h % 1000) < 1000.0 * pd) flags[b] = -1;
        }
      }
      std::vector<SmrLoc> nl;
      if (!amr_update_tree(nrb, cur, flags, &nl)) continue;
      std::vector<double> odx, oxf, oxc, ndx, nxf, nxc;
      int ncm, nccm;
      coords(d, mnx, nx, cur, &odx, &oxf, &oxc, &ncm, &nccm);
      coords(d, mnx, nx, nl, &ndx, &nxf, &nxc, &ncm, &nccm);
      AmrArrays nw;
      std::vector<int> nd;
      amr_fill(d, mhd, cur, A, odx, deref, nl, ndx, nxf, nxc, ncm, nccm, &nw, &nd);
      SmrPlan plan;
      std::string err;
      if (!smr_plan(d, nrb, nl, ndx.data(), mhd, &plan, &err)) {
        fprintf(stderr, "plan failed: %s\n", err.c_str());
        return 3;
      }
      const size_t nb = nl.size();
      // the device pool of this mesh, one vector per allocation, exact sizes
      Pool P;
      P.u = nw.u;
      P.w.assign(nb * 5 * d.ncell, 0.0);
      P.cu = nw.cu;
      P.cw.assign(nb * 5 * d.ccell, 0.0);
      const int nflx = mhd ? 8 : 5;
      P.f[0].assign(nb * nflx * d.nf1, 1e-3);
      P.f[1].assign(nb * nflx * d.nf2, 2e-3);
      P.f[2].assign(nb * nflx * d.nf3, 3e-3);
      if (mhd) {
        P.b1 = nw.b1; P.b2 = nw.b2; P.b3 = nw.b3;
        P.bcc.assign(nb * 3 * d.ncell, 0.0);
        P.cb1 = nw.cb1; P.cb2 = nw.cb2; P.cb3 = nw.cb3;
        P.cbcc.assign(nb * 3 * d.ccell, 0.0);
        P.edge.assign(nb * 3 * d.ne, 1e-4);
      }
      P.dx = ndx; P.xvf = nxf; P.xvc = nxc;
      run_lists(d, plan, (int)nb, mhd, P, ncm, nccm);
      if (g_bad) {
        fprintf(stderr, "sequence %d pass %d: %d entries out of range\n", s, pass, g_bad);
        return 1;
      }
      int lv[8] = {0};
      for (const SmrLoc& l : nl) lv[l.level < 8 ? l.level : 7]++;
      printf("seq %d pass %d: %zu -> %zu blocks (levels %d %d %d), lists %zu %zu %zu %zu %zu %zu\n",
             s, pass, cur.size(), nl.size(), lv[0], lv[1], lv[2], plan.xfer.size(),
             plan.pcc.size(), plan.pint.size(), plan.pfine.size(), plan.flux.size(),
             plan.emf.size());
      ++checked;
      cur = nl;
      A = nw;
      deref = nd;
    }
  }
  printf("checked %lld meshes\n", checked);
  return 0;
}

// amr_fill_check.cpp -- CPU run of the adaptive-refinement host path (test infrastructure),
// built with AddressSanitizer by tests/test_sanitized_host.py: a 32^3 root of 8^3 blocks
// with two ghost layers and a refined centre is refined to three levels
// (FillSameRankCoarseToFineAMR), refined again at the root level, then derefined
// (FillSameRankFineToCoarseAMR), through amr_update_tree and amr_fill.
#include <cstdio>
#include <vector>
#include "athg_amr.h"
using namespace athg;
static const int NB = 8, NG = 2, MNX = 32;
static void coords(const SmrDims& d, const std::vector<SmrLoc>& L, std::vector<double>* dx,
                   std::vector<double>* xvf, std::vector<double>* xvc, int* ncmax, int* nccmax) {
  *ncmax = d.nc1; *nccmax = NB / 2 + 2 * NG;
  dx->assign(L.size() * 3, 0.0); xvf->assign(L.size() * 3 * *ncmax, 0.0);
  xvc->assign(L.size() * 3 * *nccmax, 0.0);
  for (size_t b = 0; b < L.size(); ++b)
    for (int a = 0; a < 3; ++a)
      smr_axis_coords(MNX, MNX / NB, -1.0, 1.0, L[b].level, L[b].lx[a], NB, NG, &(*dx)[3 * b + a],
                      &(*xvf)[(b * 3 + a) * *ncmax], &(*xvc)[(b * 3 + a) * *nccmax], nullptr);
}
static AmrArrays arrays(const SmrDims& d, size_t nb) {
  AmrArrays A;
  A.u.assign(nb * 5 * d.ncell, 1.0); A.cu.assign(nb * 5 * d.ccell, 1.0);
  A.b1.assign(nb * d.nf1, 0.1); A.b2.assign(nb * d.nf2, 0.2); A.b3.assign(nb * d.nf3, 0.3);
  A.cb1.assign(nb * d.cf1, 0.1); A.cb2.assign(nb * d.cf2, 0.2); A.cb3.assign(nb * d.cf3, 0.3);
  for (size_t q = 0; q < A.u.size(); ++q) A.u[q] += 1e-3 * (double)(q % 97);
  return A;
}
int main() {
  const SmrDims d = smr_dims(NB, NB, NB, NG);
  const int nrb[3] = {MNX / NB, MNX / NB, MNX / NB};
  std::vector<SmrLoc> L;
  for (int k = 0; k < 4; ++k) for (int j = 0; j < 4; ++j) for (int i = 0; i < 4; ++i) {
    const bool in = i >= 1 && i <= 2 && j >= 1 && j <= 2 && k >= 1 && k <= 2;
    if (!in) { SmrLoc l{}; l.level = 0; l.lx[0] = i; l.lx[1] = j; l.lx[2] = k; L.push_back(l); continue; }
    for (int m = 0; m < 8; ++m) { SmrLoc l{}; l.level = 1; l.lx[0] = 2 * i + (m & 1);
      l.lx[1] = 2 * j + ((m >> 1) & 1); l.lx[2] = 2 * k + (m >> 2); L.push_back(l); }
  }
  std::vector<SmrLoc> cur = L;
  AmrArrays A = arrays(d, cur.size());
  std::vector<int> deref(cur.size(), 0);
  for (int pass = 0; pass < 3; ++pass) {
    std::vector<int> flags(cur.size(), 0);
    for (size_t b = 0; b < cur.size(); ++b) {
      const SmrLoc& l = cur[b];
      auto mid = [&](int a) { return l.lx[a] >= 3 && l.lx[a] <= 4; };
      if (pass == 0 && l.level == 1 && mid(0) && mid(1) && mid(2)) flags[b] = 1;
      if (pass == 1 && l.level == 0 && l.lx[0] == 3 && l.lx[1] == 3 && l.lx[2] == 3) flags[b] = 1;
      if (pass == 2 && l.level == 2) flags[b] = -1;
    }
    std::vector<SmrLoc> nl;
    const bool changed = amr_update_tree(nrb, cur, flags, &nl);
    std::vector<double> odx, ox, oc, ndx, nxf, nxc; int ncm, nccm;
    coords(d, cur, &odx, &ox, &oc, &ncm, &nccm);
    coords(d, nl, &ndx, &nxf, &nxc, &ncm, &nccm);
    AmrArrays nw; std::vector<int> nd;
    amr_fill(d, true, cur, A, odx, deref, nl, ndx, nxf, nxc, ncm, nccm, &nw, &nd);
    int lv[3] = {0, 0, 0};
    for (const SmrLoc& l : nl) lv[l.level]++;
    printf("pass %d changed %d: %zu -> %zu blocks (levels %d %d %d)\n", pass, (int)changed,
           cur.size(), nl.size(), lv[0], lv[1], lv[2]);
    cur = nl; A = nw; deref = nd;
  }
  return 0;
}

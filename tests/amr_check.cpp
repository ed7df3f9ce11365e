// amr_check.cpp -- CPU run of the adaptive-refinement host logic (test infrastructure).
//
// Reads from stdin
//   tree  nrb1 nrb2 nrb3 n   then n lines "level lx1 lx2 lx3 flag"
//   flag  maxeps threshold deref_fraction level max_level deref_threshold deref_count
//         then 27 neighbour levels
// and prints, for "tree": the gid order of the input leaves ("order g0 g1 ..."), whether
// amr_update_tree changed the tree ("changed 0|1") and the new leaves, one per line; for
// "flag": the flag of amr_flag and the updated derefinement counter.
#include <cstdio>
#include <iostream>
#include <string>
#include <vector>

#include "athg_amr.h"

using namespace athg;

int main() {
  std::string mode;
  std::cin >> mode;
  if (mode == "tree") {
    int nrb[3], n;
    std::cin >> nrb[0] >> nrb[1] >> nrb[2] >> n;
    std::vector<SmrLoc> leaves(n);
    std::vector<int> flags(n);
    for (int q = 0; q < n; ++q) {
      long long lx[3];
      std::cin >> leaves[q].level >> lx[0] >> lx[1] >> lx[2] >> flags[q];
      for (int d = 0; d < 3; ++d) leaves[q].lx[d] = lx[d];
    }
    if (!std::cin) { std::fprintf(stderr, "bad input\n"); return 2; }
    std::vector<int> order = amr_tree_order(nrb, leaves);
    std::printf("order");
    for (int g : order) std::printf(" %d", g);
    std::printf("\n");
    std::vector<SmrLoc> out;
    const bool changed = amr_update_tree(nrb, leaves, flags, &out);
    std::printf("changed %d\n", changed ? 1 : 0);
    for (const SmrLoc& l : out)
      std::printf("%d %lld %lld %lld\n", l.level, (long long)l.lx[0], (long long)l.lx[1],
                  (long long)l.lx[2]);
    return 0;
  }
  if (mode == "flag") {
    double maxeps, thr, frac;
    int level, max_level, dthr, dcount, nbl[27];
    std::cin >> maxeps >> thr >> frac >> level >> max_level >> dthr >> dcount;
    for (int q = 0; q < 27; ++q) std::cin >> nbl[q];
    if (!std::cin) { std::fprintf(stderr, "bad input\n"); return 2; }
    const int f = amr_flag(maxeps, thr, frac, level, max_level, nbl, dthr, &dcount);
    std::printf("%d %d\n", f, dcount);
    return 0;
  }
  std::fprintf(stderr, "unknown mode\n");
  return 2;
}

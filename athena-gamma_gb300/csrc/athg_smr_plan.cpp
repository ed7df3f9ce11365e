// athg_smr_plan.cpp -- host side of static mesh refinement: neighbour tables in the
// reference's order and the flat work lists the device runs (see athg_smr.h).
//
// Each list is produced by replaying, per block, the index ranges of the reference's
// boundary routines for a 3-D Cartesian mesh with periodic boundaries:
//   neighbours  BoundaryBase::SearchAndSetNeighbors        bvals/bvals_base.cpp:299-720
//   ghost fill  Load/SetBoundaryBuffer* (cells, faces)     bvals/cc/bvals_cc.cpp:170-470,
//                                                          bvals/fc/bvals_fc.cpp:344-976
//   prolong     BoundaryValues::ProlongateBoundaries       bvals/bvals_refine.cpp:93-570
//   fluxes      CellCenteredBoundaryVariable flux corr.    bvals/cc/flux_correction_cc.cpp
//   EMFs        FaceCenteredBoundaryVariable flux corr.    bvals/fc/flux_correction_fc.cpp
//   edge counts CountFineEdges                             bvals/fc/bvals_fc.cpp:1129-1197
// Elements written more than once by the reference keep their last writer.
#include <algorithm>
#include <cstdint>
#include <map>
#include <set>
#include <string>
#include <tuple>
#include <vector>

#include "athg_smr.h"

namespace athg {
namespace {

constexpr int NHYD = 5;

using Key = std::tuple<int, int64_t, int64_t, int64_t>;

// Neighbour entry (NeighborBlock): direction, connection type (1 face, 2 edge, 3 corner),
// fine-child indices fi1/fi2 of a finer neighbour, its level and block id
struct Nb {
  int ox[3];
  int type;
  int fi[2];
  int level;
  int id;
  int eid;
};

struct BlockNb {
  std::vector<Nb> nb;
  int nblevel[3][3][3];
  int myox[3];
  bool edge_flag[12];
  int nedge_fine[12];
  int lv(int o1, int o2, int o3) const { return nblevel[o3 + 1][o2 + 1][o1 + 1]; }
};

struct Tree {
  int nrb[3];
  std::map<Key, int> leaf;
  std::set<Key> inner;  // refined nodes
  int64_t wrap(int d, int level, int64_t x) const {
    const int64_t n = (int64_t)nrb[d] << level;
    return ((x % n) + n) % n;
  }
  int find(int level, int64_t x, int64_t y, int64_t z) const {
    auto it = leaf.find(Key(level, x, y, z));
    return it == leaf.end() ? -1 : it->second;
  }
  bool refined(int level, int64_t x, int64_t y, int64_t z) const {
    return inner.count(Key(level, x, y, z)) != 0;
  }
};

int edge_id(const int ox[3]) {
  if (ox[2] == 0) return ((ox[0] + 1) >> 1) | ((ox[1] + 1) & 2);
  if (ox[1] == 0) return 4 + (((ox[0] + 1) >> 1) | ((ox[2] + 1) & 2));
  return 8 + (((ox[1] + 1) >> 1) | ((ox[2] + 1) & 2));
}

// Tree::FindNeighbor + the three cases of SearchAndSetNeighbors for direction ox.
// kind: 0 same level (id), -1 coarser (id), +1 finer (node location in nx, level).
struct Found {
  int kind;
  int id;
  int64_t nx[3];
};

bool find_neighbor(const Tree& t, const SmrLoc& me, const int ox[3], Found* f, std::string* err) {
  int64_t x[3];
  for (int d = 0; d < 3; ++d) x[d] = t.wrap(d, me.level, me.lx[d] + ox[d]);
  int id = t.find(me.level, x[0], x[1], x[2]);
  if (id >= 0) { f->kind = 0; f->id = id; return true; }
  if (t.refined(me.level, x[0], x[1], x[2])) {
    f->kind = 1; f->id = -1;
    for (int d = 0; d < 3; ++d) f->nx[d] = x[d];
    return true;
  }
  if (me.level > 0) {
    id = t.find(me.level - 1, x[0] >> 1, x[1] >> 1, x[2] >> 1);
    if (id >= 0) { f->kind = -1; f->id = id; return true; }
  }
  *err = "mesh is not 2:1 balanced (a neighbour is more than one level coarser)";
  return false;
}

// child (m0,m1,m2) of the refined node at `level`, location nx: must be a leaf
int child_leaf(const Tree& t, int level, const int64_t nx[3], int m0, int m1, int m2,
               std::string* err) {
  int id = t.find(level + 1, 2 * nx[0] + m0, 2 * nx[1] + m1, 2 * nx[2] + m2);
  if (id < 0) *err = "mesh is not 2:1 balanced (a neighbour is more than one level finer)";
  return id;
}

// SearchAndSetNeighbors (3-D, multilevel): faces x1, x2, x3 (each -1 then +1), edges
// x1x2, x1x3, x2x3, corners, with the reference's loop order and finer-leaf order
bool search_neighbors(const Tree& t, const std::vector<SmrLoc>& loc, int b, BlockNb* out,
                      std::string* err) {
  const SmrLoc& me = loc[b];
  BlockNb& B = *out;
  B.nb.clear();
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 3; ++j)
      for (int i = 0; i < 3; ++i) B.nblevel[k][j][i] = -1;
  B.nblevel[1][1][1] = me.level;
  for (int d = 0; d < 3; ++d) B.myox[d] = ((me.lx[d] & 1) == 1) ? 1 : -1;
  auto add = [&](const int ox[3], int type, int f1, int f2, int level, int id) {
    Nb n;
    for (int d = 0; d < 3; ++d) n.ox[d] = ox[d];
    n.type = type; n.fi[0] = f1; n.fi[1] = f2; n.level = level; n.id = id;
    n.eid = (type == 2) ? edge_id(ox) : -1;
    B.nb.push_back(n);
  };
  // faces
  for (int d = 0; d < 3; ++d) {
    for (int n = -1; n <= 1; n += 2) {
      int ox[3] = {0, 0, 0};
      ox[d] = n;
      Found f;
      if (!find_neighbor(t, me, ox, &f, err)) return false;
      if (f.kind == 1) {
        B.nblevel[ox[2] + 1][ox[1] + 1][ox[0] + 1] = me.level + 1;
        const int fface = 1 - (n + 1) / 2;
        for (int f2 = 0; f2 < 2; ++f2)
          for (int f1 = 0; f1 < 2; ++f1) {
            int m[3];
            if (d == 0) { m[0] = fface; m[1] = f1; m[2] = f2; }
            else if (d == 1) { m[0] = f1; m[1] = fface; m[2] = f2; }
            else { m[0] = f1; m[1] = f2; m[2] = fface; }
            int id = child_leaf(t, me.level, f.nx, m[0], m[1], m[2], err);
            if (id < 0) return false;
            add(ox, 1, f1, f2, me.level + 1, id);
          }
      } else {
        const int lvl = loc[f.id].level;
        B.nblevel[ox[2] + 1][ox[1] + 1][ox[0] + 1] = lvl;
        add(ox, 1, 0, 0, lvl, f.id);
      }
    }
  }
  // edges: (a, b) = the two axes of the edge, loops over ox[b] (outer) then ox[a]
  const int eaxes[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int e = 0; e < 3; ++e) {
    const int a = eaxes[e][0], c = eaxes[e][1];
    for (int m = -1; m <= 1; m += 2)
      for (int n = -1; n <= 1; n += 2) {
        int ox[3] = {0, 0, 0};
        ox[a] = n; ox[c] = m;
        Found f;
        if (!find_neighbor(t, me, ox, &f, err)) return false;
        if (f.kind == 1) {
          B.nblevel[ox[2] + 1][ox[1] + 1][ox[0] + 1] = me.level + 1;
          const int ff1 = 1 - (n + 1) / 2, ff2 = 1 - (m + 1) / 2;
          for (int f1 = 0; f1 < 2; ++f1) {
            int mm[3];
            mm[a] = ff1; mm[c] = ff2; mm[3 - a - c] = f1;
            int id = child_leaf(t, me.level, f.nx, mm[0], mm[1], mm[2], err);
            if (id < 0) return false;
            add(ox, 2, f1, 0, me.level + 1, id);
          }
        } else {
          const int lvl = loc[f.id].level;
          B.nblevel[ox[2] + 1][ox[1] + 1][ox[0] + 1] = lvl;
          if (lvl >= me.level || (B.myox[a] == n && B.myox[c] == m)) add(ox, 2, 0, 0, lvl, f.id);
        }
      }
  }
  // corners
  for (int l = -1; l <= 1; l += 2)
    for (int m = -1; m <= 1; m += 2)
      for (int n = -1; n <= 1; n += 2) {
        int ox[3] = {n, m, l};
        Found f;
        if (!find_neighbor(t, me, ox, &f, err)) return false;
        int id = f.id, lvl;
        if (f.kind == 1) {
          id = child_leaf(t, me.level, f.nx, 1 - (n + 1) / 2, 1 - (m + 1) / 2, 1 - (l + 1) / 2,
                          err);
          if (id < 0) return false;
          lvl = me.level + 1;
        } else {
          lvl = loc[id].level;
        }
        B.nblevel[l + 1][m + 1][n + 1] = lvl;
        if (lvl >= me.level || (B.myox[0] == n && B.myox[1] == m && B.myox[2] == l))
          add(ox, 3, 0, 0, lvl, id);
      }
  // CountFineEdges: finest level among the four blocks around each edge, and how many
  // of them are at it
  int eid = 0;
  for (int e = 0; e < 3; ++e) {
    const int a = eaxes[e][0], c = eaxes[e][1];
    for (int m = -1; m <= 1; m += 2)
      for (int n = -1; n <= 1; n += 2) {
        const int na0 = std::max(n - 1, -1), na1 = std::min(n + 1, 1);
        const int nc0 = std::max(m - 1, -1), nc1 = std::min(m + 1, 1);
        int nf = 0, fl = me.level;
        for (int q = nc0; q <= nc1; ++q)
          for (int p = na0; p <= na1; ++p) {
            int o[3] = {0, 0, 0};
            o[a] = p; o[c] = q;
            const int lv = B.lv(o[0], o[1], o[2]);
            if (lv > fl) { fl++; nf = 0; }
            if (lv == fl) nf++;
          }
        B.edge_flag[eid] = (fl == me.level);
        B.nedge_fine[eid++] = nf;
      }
  }
  return true;
}


// ---- ghost fill ------------------------------------------------------------------------
struct Box {
  int s[3], e[3];  // per axis (0 = i, 1 = j, 2 = k), inclusive
};

// Dense "last writer" slots of one block's eight destination arrays
struct Slots {
  const SmrDims* d;
  std::vector<SmrXfer> v[8];
  std::vector<char> set[8];
  std::vector<int32_t> touched[8];
  void init(const SmrDims& dd) {
    d = &dd;
    const int64_t n[8] = {dd.ncell, dd.nf1, dd.nf2, dd.nf3, dd.ccell, dd.cf1, dd.cf2, dd.cf3};
    for (int a = 0; a < 8; ++a) { v[a].resize(n[a]); set[a].assign(n[a], 0); }
  }
  void put(int arr, int64_t didx, int op, int sblk, int64_t sidx, int dblk) {
    SmrXfer& x = v[arr][didx];
    x.dblk = dblk; x.sblk = sblk; x.didx = (int32_t)didx; x.sidx = (int32_t)sidx;
    x.darr = (int16_t)arr; x.op = (int16_t)op;
    if (!set[arr][didx]) { set[arr][didx] = 1; touched[arr].push_back((int32_t)didx); }
  }
  void flush(std::vector<SmrXfer>* out) {
    for (int a = 0; a < 8; ++a) {
      std::sort(touched[a].begin(), touched[a].end());
      for (int32_t i : touched[a]) { out->push_back(v[a][i]); set[a][i] = 0; }
      touched[a].clear();
    }
  }
};

// index of (k,j,i) in array kind arr (0..3 fine, 4..7 coarse)
int64_t aidx(const SmrDims& d, int arr, int k, int j, int i) {
  switch (arr) {
    case SA_U: return d.c(k, j, i);
    case SA_B1: return d.f1(k, j, i);
    case SA_B2: return d.f2(k, j, i);
    case SA_B3: return d.f3(k, j, i);
    case SA_CU: return d.cc(k, j, i);
    case SA_CB1: return d.cf1i(k, j, i);
    case SA_CB2: return d.cf2i(k, j, i);
    default: return d.cf3i(k, j, i);
  }
}

// for every element of dst box (k outer, i inner): dst position and the matching source
// position (same offset inside the source box)
template <typename F>
void each(const Box& db, const Box& sb, F f) {
  for (int k = db.s[2]; k <= db.e[2]; ++k)
    for (int j = db.s[1]; j <= db.e[1]; ++j)
      for (int i = db.s[0]; i <= db.e[0]; ++i)
        f(k, j, i, sb.s[2] + (k - db.s[2]), sb.s[1] + (j - db.s[1]), sb.s[0] + (i - db.s[0]));
}

struct Ranges {
  int S[3], E[3], CS[3], CE[3], NX[3], ng, cng;
  explicit Ranges(const SmrDims& d) {
    S[0] = d.is; S[1] = d.js; S[2] = d.ks; E[0] = d.ie; E[1] = d.je; E[2] = d.ke;
    CS[0] = d.cis; CS[1] = d.cjs; CS[2] = d.cks; CE[0] = d.cie; CE[1] = d.cje; CE[2] = d.cke;
    NX[0] = d.nx1; NX[1] = d.nx2; NX[2] = d.nx3;
    ng = d.ng; cng = d.cng;
  }
  // normal: -1 for cells, else the face component's normal axis
  // same-level receive (SetBoundarySameLevel, cells bvals_cc.cpp:283-310, faces
  // bvals_fc.cpp:583-688)
  Box same_recv(const int ox[3], int normal, bool face_type) const {
    Box b;
    for (int a = 0; a < 3; ++a) {
      if (a != normal) {
        if (ox[a] == 0) { b.s[a] = S[a]; b.e[a] = E[a]; }
        else if (ox[a] > 0) { b.s[a] = E[a] + 1; b.e[a] = E[a] + ng; }
        else { b.s[a] = S[a] - ng; b.e[a] = S[a] - 1; }
      } else {
        if (ox[a] == 0) { b.s[a] = S[a]; b.e[a] = E[a] + 1; }
        else if (ox[a] > 0) { b.s[a] = E[a] + 2; b.e[a] = E[a] + ng + 1; }
        else { b.s[a] = S[a] - ng; b.e[a] = S[a] - 1; }
        if (!face_type) {
          if (ox[a] > 0) b.s[a]--;
          else if (ox[a] < 0) b.e[a]++;
        }
      }
    }
    return b;
  }
  // into the coarse buffer from a coarser neighbour (SetBoundaryFromCoarser,
  // bvals_cc.cpp:344-395, bvals_fc.cpp:690-811); lx: the receiving block's location
  Box coarser_recv(const int ox[3], int normal, const int64_t lx[3]) const {
    Box b;
    for (int a = 0; a < 3; ++a) {
      const int fc = (a == normal) ? 1 : 0;
      if (ox[a] == 0) {
        b.s[a] = CS[a]; b.e[a] = CE[a] + fc;
        if ((lx[a] & 1) == 0) b.e[a] += cng;
        else b.s[a] -= cng;
      } else if (ox[a] > 0) {
        b.s[a] = CE[a] + 1; b.e[a] = CE[a] + cng + fc;
      } else {
        b.s[a] = CS[a] - cng; b.e[a] = CS[a] - 1 + fc;
      }
    }
    return b;
  }
  // what a coarser block sends to a finer one (LoadBoundaryBufferToFiner,
  // bvals_cc.cpp:210-250, bvals_fc.cpp:476-581); o: direction of the fine block seen from
  // the coarse one, flx: the fine block's location (its child offsets pick the half)
  Box to_finer(const int o[3], int normal, const int64_t flx[3]) const {
    Box b;
    const int cn = cng - 1;
    for (int a = 0; a < 3; ++a) {
      const int fc = (a == normal) ? 1 : 0;
      if (o[a] == 0) {
        b.s[a] = S[a]; b.e[a] = E[a] + fc;
        if ((flx[a] & 1) == 1) b.s[a] += NX[a] / 2 - cng;
        else b.e[a] -= NX[a] / 2 - cng;
      } else if (o[a] > 0) {
        b.s[a] = fc ? E[a] + 1 - cng : E[a] - cn; b.e[a] = E[a] + fc;
      } else {
        b.s[a] = S[a]; b.e[a] = fc ? S[a] + cng : S[a] + cn;
      }
    }
    return b;
  }
  // into a coarser block's ghosts from a finer neighbour (SetBoundaryFromFiner,
  // bvals_cc.cpp:403-470, bvals_fc.cpp:813-976); flx: the finer block's location
  Box finer_recv(const int ox[3], int normal, bool face_type, const int64_t flx[3]) const {
    Box b;
    for (int a = 0; a < 3; ++a) {
      const int fc = (a == normal) ? 1 : 0;
      if (ox[a] == 0) {
        b.s[a] = S[a]; b.e[a] = E[a] + fc;
        if ((flx[a] & 1) == 1) b.s[a] += NX[a] / 2;
        else b.e[a] -= NX[a] / 2;
      } else if (ox[a] > 0) {
        b.s[a] = E[a] + 1 + fc; b.e[a] = E[a] + ng + fc;
      } else {
        b.s[a] = S[a] - ng; b.e[a] = S[a] - 1;
      }
      if (fc && !face_type) {
        if (ox[a] > 0) b.s[a]--;
        else if (ox[a] < 0) b.e[a]++;
      }
    }
    return b;
  }
  // what a finer block restricts and sends to a coarser one, in its coarse-buffer
  // indices (LoadBoundaryBufferToCoarser, bvals_cc.cpp:183-208, bvals_fc.cpp:403-474);
  // o: direction of the coarse block seen from the fine one
  Box to_coarser(const int o[3], int normal, bool face_type) const {
    Box b;
    for (int a = 0; a < 3; ++a) {
      const int fc = (a == normal) ? 1 : 0;
      if (o[a] == 0) { b.s[a] = CS[a]; b.e[a] = CE[a] + fc; }
      else if (o[a] > 0) { b.s[a] = CE[a] - ng + 1; b.e[a] = CE[a]; }
      else { b.s[a] = CS[a] + fc; b.e[a] = CS[a] + ng - 1 + fc; }
      if (fc && !face_type) {
        if (o[a] > 0) b.e[a]++;
        else if (o[a] < 0) b.s[a]--;
      }
    }
    return b;
  }
  // fine lower corner of coarse index c along axis a
  int fine_of(int a, int c) const { return (c - CS[a]) * 2 + S[a]; }
};

const int kFaceArr[3] = {SA_B1, SA_B2, SA_B3};
const int kCoarseFaceArr[3] = {SA_CB1, SA_CB2, SA_CB3};
const int kRestrictFace[3] = {SO_RF1, SO_RF2, SO_RF3};

void ghost_fill(const SmrDims& d, const Ranges& R, const std::vector<SmrLoc>& loc,
                const std::vector<BlockNb>& nbs, int b, bool mhd, Slots* sl) {
  const SmrLoc& me = loc[b];
  const BlockNb& B = nbs[b];
  // sends to coarser blocks restrict this block's interior into its own coarse buffer
  for (const Nb& n : B.nb) {
    if (n.level >= me.level) continue;
    const bool face = n.type == 1;
    Box cb = R.to_coarser(n.ox, -1, face);
    each(cb, cb, [&](int k, int j, int i, int, int, int) {
      sl->put(SA_CU, d.cc(k, j, i), SO_RCC, b, d.c(R.fine_of(2, k), R.fine_of(1, j), R.fine_of(0, i)), b);
    });
    if (!mhd) continue;
    for (int nrm = 0; nrm < 3; ++nrm) {
      Box fb = R.to_coarser(n.ox, nrm, face);
      each(fb, fb, [&](int k, int j, int i, int, int, int) {
        sl->put(kCoarseFaceArr[nrm], aidx(d, kCoarseFaceArr[nrm], k, j, i), kRestrictFace[nrm], b,
                aidx(d, kFaceArr[nrm], R.fine_of(2, k), R.fine_of(1, j), R.fine_of(0, i)), b);
      });
    }
  }
  // receives, in neighbour order
  for (const Nb& n : B.nb) {
    const bool face = n.type == 1;
    int o[3] = {-n.ox[0], -n.ox[1], -n.ox[2]};
    for (int nrm = -1; nrm < 3; ++nrm) {
      if (nrm >= 0 && !mhd) break;
      const int farr = nrm < 0 ? SA_U : kFaceArr[nrm];
      if (n.level == me.level) {
        Box db = R.same_recv(n.ox, nrm, face);
        each(db, db, [&](int k, int j, int i, int, int, int) {
          sl->put(farr, aidx(d, farr, k, j, i), SO_COPY, n.id,
                  aidx(d, farr, k - n.ox[2] * d.nx3, j - n.ox[1] * d.nx2, i - n.ox[0] * d.nx1), b);
        });
      } else if (n.level < me.level) {
        const int carr = nrm < 0 ? SA_CU : kCoarseFaceArr[nrm];
        Box db = R.coarser_recv(n.ox, nrm, me.lx);
        Box sb = R.to_finer(o, nrm, me.lx);
        each(db, sb, [&](int k, int j, int i, int sk, int sj, int si) {
          sl->put(carr, aidx(d, carr, k, j, i), SO_COPY, n.id, aidx(d, farr, sk, sj, si), b);
        });
      } else {
        const int64_t* flx = loc[n.id].lx;
        Box db = R.finer_recv(n.ox, nrm, face, flx);
        Box sb = R.to_coarser(o, nrm, face);
        const int op = nrm < 0 ? SO_RCC : kRestrictFace[nrm];
        each(db, sb, [&](int k, int j, int i, int sk, int sj, int si) {
          sl->put(farr, aidx(d, farr, k, j, i), op, n.id,
                  aidx(d, farr, R.fine_of(2, sk), R.fine_of(1, sj), R.fine_of(0, si)), b);
        });
      }
    }
  }
}

// Dense set of positions of one block (dedup of the prolongation lists)
struct PosSet {
  std::vector<char> f;
  std::vector<int64_t> t;
  void init(int64_t n) { f.assign(n, 0); }
  void add(int64_t i) { if (!f[i]) { f[i] = 1; t.push_back(i); } }
  template <typename G>
  void flush(int blk, std::vector<SmrPos>* out, G dec) {
    std::sort(t.begin(), t.end());
    for (int64_t i : t) {
      SmrPos p; p.blk = blk; dec(i, &p.k, &p.j, &p.i);
      out->push_back(p);
      f[i] = 0;
    }
    t.clear();
  }
};

// ProlongateBoundaries (bvals_refine.cpp:93-228) for every coarser neighbour of block b:
// restriction of same-level ghosts (RestrictGhostCellsOnSameLevel :234-329), the coarse
// cells converted to primitives (ApplyPhysicalBoundariesOnCoarseLevel :375-381), the
// prolongated cells and faces (ProlongateGhostCells :471-565)
void prolong_lists(const SmrDims& d, const Ranges& R, const std::vector<SmrLoc>& loc,
                   const std::vector<BlockNb>& nbs, int b, bool mhd, Slots* pre,
                   PosSet* c2p, PosSet* pcc, PosSet psf[3], PosSet* pint, PosSet* pfine) {
  const SmrLoc& me = loc[b];
  const BlockNb& B = nbs[b];
  const int L = me.level;
  for (const Nb& n : B.nb) {
    if (n.level >= L) continue;
    const int* ox = n.ox;
    // step 1: same-level ghost cells around the prolongation region into the coarse buffer
    int lo[3], hi[3];
    for (int a = 0; a < 3; ++a) { lo[a] = std::max(ox[a] - 1, -1); hi[a] = std::min(ox[a] + 1, 1); }
    for (int nk = lo[2]; nk <= hi[2]; ++nk)
      for (int nj = lo[1]; nj <= hi[1]; ++nj)
        for (int ni = lo[0]; ni <= hi[0]; ++ni) {
          const int nn[3] = {ni, nj, nk};
          if (std::abs(ni) + std::abs(nj) + std::abs(nk) == 0) continue;
          if (B.nblevel[nk + 1][nj + 1][ni + 1] != L) continue;
          Box r;
          for (int a = 0; a < 3; ++a) {
            if (nn[a] == 0) {
              r.s[a] = R.CS[a]; r.e[a] = R.CE[a];
              if (ox[a] == 1) r.s[a] = R.CE[a];
              else if (ox[a] == -1) r.e[a] = R.CS[a];
            } else if (nn[a] == 1) {
              r.s[a] = r.e[a] = R.CE[a] + 1;
            } else {
              r.s[a] = r.e[a] = R.CS[a] - 1;
            }
          }
          each(r, r, [&](int k, int j, int i, int, int, int) {
            pre->put(SA_CU, d.cc(k, j, i), SO_RCC, b,
                     d.c(R.fine_of(2, k), R.fine_of(1, j), R.fine_of(0, i)), b);
          });
          if (!mhd) continue;
          for (int nrm = 0; nrm < 3; ++nrm) {
            Box fb = r;
            int rs = r.s[nrm], re = r.e[nrm] + 1;
            // neighbour across the lower / upper side of this region along nrm
            int dl[3] = {nn[0] + 1, nn[1] + 1, nn[2] + 1}, du[3] = {nn[0] + 1, nn[1] + 1, nn[2] + 1};
            dl[nrm] -= 1; du[nrm] += 1;
            if (rs == R.CS[nrm] && B.nblevel[dl[2]][dl[1]][dl[0]] < L) rs++;
            if (re == R.CE[nrm] + 1 && B.nblevel[du[2]][du[1]][du[0]] < L) re--;
            fb.s[nrm] = rs; fb.e[nrm] = re;
            const int ca = kCoarseFaceArr[nrm];
            each(fb, fb, [&](int k, int j, int i, int, int, int) {
              pre->put(ca, aidx(d, ca, k, j, i), kRestrictFace[nrm], b,
                       aidx(d, kFaceArr[nrm], R.fine_of(2, k), R.fine_of(1, j), R.fine_of(0, i)), b);
            });
          }
        }
    // the region of coarse ghost cells to prolongate
    const int cn = R.cng - 1;
    Box g;
    for (int a = 0; a < 3; ++a) {
      if (ox[a] == 0) {
        g.s[a] = R.CS[a]; g.e[a] = R.CE[a];
        if ((me.lx[a] & 1) == 0) g.e[a] += cn;
        else g.s[a] -= cn;
      } else if (ox[a] > 0) {
        g.s[a] = R.CE[a] + 1; g.e[a] = R.CE[a] + cn;
      } else {
        g.s[a] = R.CS[a] - cn; g.e[a] = R.CS[a] - 1;
      }
    }
    // step 2: W(U) (and bcc) of the coarse buffer over the region and one cell around it
    Box g1 = g;
    for (int a = 0; a < 3; ++a) { g1.s[a]--; g1.e[a]++; }
    each(g1, g1, [&](int k, int j, int i, int, int, int) { c2p->add(d.cc(k, j, i)); });
    // step 3: cells, shared faces, internal faces
    each(g, g, [&](int k, int j, int i, int, int, int) {
      pcc->add(d.cc(k, j, i));
      if (mhd) pint->add(d.cc(k, j, i));
    });
    if (mhd) {
      for (int nrm = 0; nrm < 3; ++nrm) {
        Box fb = g;
        fb.e[nrm] += 1;
        int dl[3] = {ox[0] + 1, ox[1] + 1, ox[2] + 1}, du[3] = {ox[0] + 1, ox[1] + 1, ox[2] + 1};
        dl[nrm] -= 1; du[nrm] += 1;
        if (ox[nrm] >= 0 && B.nblevel[dl[2]][dl[1]][dl[0]] >= L) fb.s[nrm]++;
        if (ox[nrm] <= 0 && B.nblevel[du[2]][du[1]][du[0]] >= L) fb.e[nrm]--;
        const int ca = kCoarseFaceArr[nrm];
        each(fb, fb, [&](int k, int j, int i, int, int, int) { psf[nrm].add(aidx(d, ca, k, j, i)); });
      }
    }
    // step 4: fine cells of the region: bcc and U(W)
    Box fb;
    for (int a = 0; a < 3; ++a) { fb.s[a] = R.fine_of(a, g.s[a]); fb.e[a] = R.fine_of(a, g.e[a]) + 1; }
    each(fb, fb, [&](int k, int j, int i, int, int, int) { pfine->add(d.c(k, j, i)); });
  }
}

// ---- flux and EMF correction -----------------------------------------------------------
// axis strides of the edge array
int64_t edge_stride(const SmrDims& d, int a) {
  return a == 0 ? 1 : (a == 1 ? (int64_t)(d.nc1 + 1) : (int64_t)(d.nc1 + 1) * (d.nc2 + 1));
}
int64_t face_index(const SmrDims& d, int dir, const int x[3]) {
  return dir == 0 ? d.f1(x[2], x[1], x[0]) : (dir == 1 ? d.f2(x[2], x[1], x[0]) : d.f3(x[2], x[1], x[0]));
}

// Flux correction of block b (SetFluxBoundaryFromFiner, flux_correction_cc.cpp:206-258):
// the coarse face fluxes under each finer face neighbour, from its restricted fluxes
// (LoadFluxBoundaryBufferToCoarser :66-158)
void flux_list(const SmrDims& d, const Ranges& R, const std::vector<SmrLoc>& loc,
               const std::vector<BlockNb>& nbs, int b, std::vector<SmrFlux>* out) {
  const int L = loc[b].level;
  for (const Nb& n : nbs[b].nb) {
    if (n.type != 1) break;
    if (n.level != L + 1) continue;
    int a = 0;
    while (n.ox[a] == 0) ++a;
    const int64_t* flx = loc[n.id].lx;
    int lo[3], hi[3];
    for (int t = 0; t < 3; ++t) {
      if (t == a) {
        lo[t] = hi[t] = (n.ox[a] < 0) ? R.S[a] : R.E[a] + 1;
      } else if ((flx[t] & 1) == 0) {
        lo[t] = R.S[t]; hi[t] = R.S[t] + R.NX[t] / 2 - 1;
      } else {
        lo[t] = R.S[t] + R.NX[t] / 2; hi[t] = R.E[t];
      }
    }
    const int fface = (n.ox[a] > 0) ? R.S[a] : R.E[a] + 1;  // the fine block's face
    for (int k = lo[2]; k <= hi[2]; ++k)
      for (int j = lo[1]; j <= hi[1]; ++j)
        for (int i = lo[0]; i <= hi[0]; ++i) {
          const int x[3] = {i, j, k};
          int fx[3];
          for (int t = 0; t < 3; ++t) fx[t] = (t == a) ? fface : R.S[t] + 2 * (x[t] - lo[t]);
          SmrFlux f;
          f.dblk = b; f.dir = a; f.sblk = n.id;
          f.didx = (int32_t)face_index(d, a, x);
          f.sidx = (int32_t)face_index(d, a, fx);
          out->push_back(f);
        }
  }
}

struct EmfState {
  int own = 1;
  std::vector<SmrEmfAdd> adds;
  double mul[2] = {1.0, 1.0};
  int nmul = 0;
};

// EMF correction of block b (ReceiveFluxCorrection, flux_correction_fc.cpp:1610-1749):
// same-level sums, clearing of edges that touch finer blocks, restricted finer EMFs,
// then the averages
void emf_list(const SmrDims& d, const Ranges& R, const std::vector<SmrLoc>& loc,
              const std::vector<BlockNb>& nbs, int b, const double* dx, std::vector<SmrEmf>* out,
              std::vector<SmrEmfAdd>* adds) {
  const int L = loc[b].level;
  const BlockNb& B = nbs[b];
  std::map<std::pair<int, int64_t>, EmfState> st;
  auto at = [&](int comp, int k, int j, int i) -> EmfState& {
    return st[std::make_pair(comp, d.e(k, j, i))];
  };
  // visit the edges of component t on the face of block b across normal a at face index
  // fidx: along t over [t0, t1] (cells), along the other transverse axis u over [u0, u1]
  auto face_edges = [&](int a, int t, int fidx, int t0, int t1, int u0, int u1, auto fn) {
    const int u = 3 - a - t;
    for (int y = u0; y <= u1; ++y)
      for (int x = t0; x <= t1; ++x) {
        int p[3];
        p[a] = fidx; p[t] = x; p[u] = y;
        fn(p);
      }
  };
  auto face_pos = [&](int a, int side) { return side < 0 ? R.S[a] : R.E[a] + 1; };
  // 1. same-level face neighbours and same-level edge neighbours of flagged edges
  for (const Nb& n : B.nb) {
    if (n.type == 3) break;
    if (n.level != L) continue;
    if (n.type == 2 && !B.edge_flag[n.eid]) continue;
    auto addsrc = [&](int comp, const int p[3]) {
      SmrEmfAdd x;
      x.sblk = n.id; x.comp = comp; x.step = 0; x.len = 0.0;
      x.idx = (int32_t)d.e(p[2] - n.ox[2] * d.nx3, p[1] - n.ox[1] * d.nx2, p[0] - n.ox[0] * d.nx1);
      at(comp, p[2], p[1], p[0]).adds.push_back(x);
    };
    if (n.type == 1) {
      int a = 0;
      while (n.ox[a] == 0) ++a;
      for (int t = 0; t < 3; ++t) {
        if (t == a) continue;
        const int u = 3 - a - t;
        face_edges(a, t, face_pos(a, n.ox[a]), R.S[t], R.E[t], R.S[u], R.E[u] + 1,
                   [&](const int p[3]) { addsrc(t, p); });
      }
    } else {
      int t = 0;
      while (n.ox[t] != 0) ++t;
      for (int x = R.S[t]; x <= R.E[t]; ++x) {
        int p[3];
        for (int q = 0; q < 3; ++q) p[q] = (q == t) ? x : face_pos(q, n.ox[q]);
        addsrc(t, p);
      }
    }
  }
  // 2. ClearCoarseFluxBoundary (:1214-1351)
  for (int f = 0; f < 6; ++f) {
    const int a = f / 2, side = (f & 1) ? 1 : -1;
    int o[3] = {0, 0, 0};
    o[a] = side;
    if (B.lv(o[0], o[1], o[2]) <= L) continue;
    for (int t = 0; t < 3; ++t) {
      if (t == a) continue;
      const int u = 3 - a - t;
      face_edges(a, t, face_pos(a, side), R.S[t], R.E[t], R.S[u] + 1, R.E[u],
                 [&](const int p[3]) { EmfState& s = at(t, p[2], p[1], p[0]); s.own = 0; s.adds.clear(); });
    }
  }
  const int eaxes[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int eid = 0; eid < 12; ++eid) {
    if (B.edge_flag[eid]) continue;
    const int a = eaxes[eid / 4][0], c = eaxes[eid / 4][1], t = 3 - a - c;
    const int pa = (eid & 1) ? R.E[a] + 1 : R.S[a], pc = (eid & 2) ? R.E[c] + 1 : R.S[c];
    for (int x = R.S[t]; x <= R.E[t]; ++x) {
      int p[3];
      p[a] = pa; p[c] = pc; p[t] = x;
      EmfState& s = at(t, p[2], p[1], p[0]);
      s.own = 0;
      s.adds.clear();
    }
  }
  // 3. restricted EMFs of finer face and edge neighbours
  for (const Nb& n : B.nb) {
    if (n.type == 3) break;
    if (n.level != L + 1) continue;
    const int64_t* flx = loc[n.id].lx;
    int lo[3], hi[3];
    for (int t = 0; t < 3; ++t) {
      if ((flx[t] & 1) == 0) { lo[t] = R.S[t]; hi[t] = R.S[t] + R.NX[t] / 2 - 1; }
      else { lo[t] = R.S[t] + R.NX[t] / 2; hi[t] = R.E[t]; }
    }
    auto addfine = [&](int t, const int p[3]) {
      // the two fine edges along t under coarse edge p, on the fine block's surface
      int fp[3];
      for (int q = 0; q < 3; ++q) {
        if (n.ox[q] != 0) fp[q] = (n.ox[q] > 0) ? R.S[q] : R.E[q] + 1;
        else fp[q] = R.S[q] + 2 * (p[q] - lo[q]);
      }
      SmrEmfAdd x;
      x.sblk = n.id; x.comp = t;
      x.idx = (int32_t)d.e(fp[2], fp[1], fp[0]);
      x.step = (int32_t)edge_stride(d, t);
      x.len = dx[3 * n.id + t];
      at(t, p[2], p[1], p[0]).adds.push_back(x);
    };
    if (n.type == 1) {
      int a = 0;
      while (n.ox[a] == 0) ++a;
      for (int t = 0; t < 3; ++t) {
        if (t == a) continue;
        const int u = 3 - a - t;
        face_edges(a, t, face_pos(a, n.ox[a]), lo[t], hi[t], lo[u], hi[u] + 1,
                   [&](const int p[3]) { addfine(t, p); });
      }
    } else {
      int t = 0;
      while (n.ox[t] != 0) ++t;
      for (int x = lo[t]; x <= hi[t]; ++x) {
        int p[3];
        for (int q = 0; q < 3; ++q) p[q] = (q == t) ? x : face_pos(q, n.ox[q]);
        addfine(t, p);
      }
    }
  }
  // 4. AverageFluxBoundary (:1355-1543)
  auto mul = [&](EmfState& s, double m) { if (s.nmul < 2) s.mul[s.nmul++] = m; };
  for (int f = 0; f < 6; ++f) {
    const int a = f / 2, side = (f & 1) ? 1 : -1;
    int o[3] = {0, 0, 0};
    o[a] = side;
    const int nl = B.lv(o[0], o[1], o[2]);
    for (int t = 0; t < 3; ++t) {
      if (t == a) continue;
      const int u = 3 - a - t;
      if (nl == L) {
        face_edges(a, t, face_pos(a, side), R.S[t], R.E[t], R.S[u] + 1, R.E[u],
                   [&](const int p[3]) { mul(at(t, p[2], p[1], p[0]), 0.5); });
      } else if (nl > L) {
        const int mid = R.S[u] + R.NX[u] / 2;
        face_edges(a, t, face_pos(a, side), R.S[t], R.E[t], mid, mid,
                   [&](const int p[3]) { mul(at(t, p[2], p[1], p[0]), 0.5); });
      }
    }
  }
  for (int eid = 0; eid < 12; ++eid) {
    if (B.nedge_fine[eid] == 1) continue;
    const double div = 1.0 / static_cast<double>(B.nedge_fine[eid]);
    const int a = eaxes[eid / 4][0], c = eaxes[eid / 4][1], t = 3 - a - c;
    const int pa = (eid & 1) ? R.E[a] + 1 : R.S[a], pc = (eid & 2) ? R.E[c] + 1 : R.S[c];
    for (int x = R.S[t]; x <= R.E[t]; ++x) {
      int p[3];
      p[a] = pa; p[c] = pc; p[t] = x;
      mul(at(t, p[2], p[1], p[0]), div);
    }
  }
  for (auto& kv : st) {
    EmfState& s = kv.second;
    if (s.own && s.adds.empty() && s.nmul == 0) continue;
    SmrEmf e;
    e.blk = b; e.comp = kv.first.first; e.idx = (int32_t)kv.first.second; e.own = s.own;
    e.add0 = (int32_t)adds->size();
    for (const SmrEmfAdd& x : s.adds) adds->push_back(x);
    e.add1 = (int32_t)adds->size();
    e.mul[0] = s.mul[0]; e.mul[1] = s.mul[1];
    out->push_back(e);
  }
}

}  // namespace

namespace {
// ComputeMeshGeneratorX(index, nrange, true) and UniformMeshGeneratorX1
// (mesh/mesh.hpp:389-470)
double gen_rx(int64_t index, int64_t nrange) {
  const int64_t noffset = index - nrange / 2;
  const int64_t noffset_ceil = index - (nrange + 1) / 2;
  return static_cast<double>(noffset + noffset_ceil) / (2.0 * nrange);
}
double gen_x(double rx, double xmin, double xmax) {
  return 0.5 * (xmin + xmax) + (rx * xmax - rx * xmin);
}
}  // namespace

void smr_axis_coords(int mesh_nx, int nrb, double xmin, double xmax, int level, int64_t lx,
                     int nx, int ng, double* dx, double* xvf, double* xvc, double* xff) {
  const int64_t nroot = (int64_t)mesh_nx << level, nrbl = (int64_t)nrb << level;
  const int nc = nx + 2 * ng, ncc = nx / 2 + 2 * ng;
  std::vector<double> xf(nc + 1), cf(ncc + 1);
  // block_size (mesh/mesh.cpp:1675-1690): exact mesh bounds at the edges
  const double bmin = (lx == 0) ? xmin : gen_x(gen_rx(lx, nrbl), xmin, xmax);
  const double bmax = (lx == nrbl - 1) ? xmax : gen_x(gen_rx(lx + 1, nrbl), xmin, xmax);
  for (int t = 0; t <= nc; ++t) xf[t] = gen_x(gen_rx((t - ng) + lx * nx, nroot), xmin, xmax);
  xf[ng] = bmin;
  xf[ng + nx] = bmax;
  for (int t = 0; t <= ncc; ++t)
    cf[t] = gen_x(gen_rx((int64_t)(t - ng) * 2 + lx * nx, nroot), xmin, xmax);
  cf[ng] = bmin;
  cf[ng + nx / 2] = bmax;
  for (int t = 0; t < nc; ++t) xvf[t] = 0.5 * (xf[t + 1] + xf[t]);
  if (xff)
    for (int t = 0; t <= nc; ++t) xff[t] = xf[t];
  for (int t = 0; t < ncc; ++t) xvc[t] = 0.5 * (cf[t + 1] + cf[t]);
  *dx = (bmax - bmin) / nx;
}

bool smr_neighbor_levels(const int nrb[3], const std::vector<SmrLoc>& loc, std::vector<int>* lv,
                         std::string* err) {
  Tree t;
  for (int a = 0; a < 3; ++a) t.nrb[a] = nrb[a];
  for (size_t b = 0; b < loc.size(); ++b) {
    const SmrLoc& l = loc[b];
    t.leaf[Key(l.level, l.lx[0], l.lx[1], l.lx[2])] = (int)b;
    for (int q = l.level - 1; q >= 0; --q) {
      const int sh = l.level - q;
      t.inner.insert(Key(q, l.lx[0] >> sh, l.lx[1] >> sh, l.lx[2] >> sh));
    }
  }
  lv->assign(27 * loc.size(), -1);
  BlockNb B;
  for (size_t b = 0; b < loc.size(); ++b) {
    if (!search_neighbors(t, loc, (int)b, &B, err)) return false;
    for (int k = 0; k < 3; ++k)
      for (int j = 0; j < 3; ++j)
        for (int i = 0; i < 3; ++i) (*lv)[27 * b + (k * 3 + j) * 3 + i] = B.nblevel[k][j][i];
  }
  return true;
}

bool smr_plan(const SmrDims& d, const int nrb[3], const std::vector<SmrLoc>& loc,
              const double* dx, bool mhd, SmrPlan* plan, std::string* err) {
  if (d.nx1 % 2 || d.nx2 % 2 || d.nx3 % 2 || d.ng % 2) {
    *err = "mesh refinement needs even block sizes and an even number of ghost cells";
    return false;
  }
  if (d.nx1 < 2 * d.ng || d.nx2 < 2 * d.ng || d.nx3 < 2 * d.ng) {
    *err = "mesh refinement needs blocks of at least 2*nghost cells per axis";
    return false;
  }
  Tree t;
  for (int a = 0; a < 3; ++a) t.nrb[a] = nrb[a];
  int maxl = 0;
  for (size_t b = 0; b < loc.size(); ++b) {
    const SmrLoc& l = loc[b];
    Key k(l.level, l.lx[0], l.lx[1], l.lx[2]);
    if (t.leaf.count(k)) { *err = "duplicate block location"; return false; }
    t.leaf[k] = (int)b;
    maxl = std::max(maxl, l.level);
    for (int lv = l.level - 1; lv >= 0; --lv) {
      const int sh = l.level - lv;
      t.inner.insert(Key(lv, l.lx[0] >> sh, l.lx[1] >> sh, l.lx[2] >> sh));
    }
  }
  for (const auto& kv : t.leaf)
    if (t.inner.count(kv.first)) { *err = "a block overlaps a refined block"; return false; }
  const int nb = (int)loc.size();
  std::vector<BlockNb> nbs(nb);
  for (int b = 0; b < nb; ++b)
    if (!search_neighbors(t, loc, b, &nbs[b], err)) return false;
  Ranges R(d);
  *plan = SmrPlan();
  plan->nlevels = maxl + 1;
  Slots xs, ps;
  xs.init(d);
  ps.init(d);
  PosSet c2p, pcc, psf[3], pint, pfine;
  c2p.init(d.ccell); pcc.init(d.ccell); pint.init(d.ccell); pfine.init(d.ncell);
  psf[0].init(d.cf1); psf[1].init(d.cf2); psf[2].init(d.cf3);
  auto dec_c = [&](int64_t q, int* k, int* j, int* i) {
    *i = (int)(q % d.ncc1); *j = (int)((q / d.ncc1) % d.ncc2); *k = (int)(q / ((int64_t)d.ncc1 * d.ncc2));
  };
  auto dec_f = [&](int64_t q, int* k, int* j, int* i) {
    *i = (int)(q % d.nc1); *j = (int)((q / d.nc1) % d.nc2); *k = (int)(q / ((int64_t)d.nc1 * d.nc2));
  };
  auto dec_cf1 = [&](int64_t q, int* k, int* j, int* i) {
    *i = (int)(q % (d.ncc1 + 1)); *j = (int)((q / (d.ncc1 + 1)) % d.ncc2);
    *k = (int)(q / ((int64_t)(d.ncc1 + 1) * d.ncc2));
  };
  auto dec_cf2 = [&](int64_t q, int* k, int* j, int* i) {
    *i = (int)(q % d.ncc1); *j = (int)((q / d.ncc1) % (d.ncc2 + 1));
    *k = (int)(q / ((int64_t)d.ncc1 * (d.ncc2 + 1)));
  };
  for (int b = 0; b < nb; ++b) {
    ghost_fill(d, R, loc, nbs, b, mhd, &xs);
    xs.flush(&plan->xfer);
    prolong_lists(d, R, loc, nbs, b, mhd, &ps, &c2p, &pcc, psf, &pint, &pfine);
    ps.flush(&plan->pre);
    c2p.flush(b, &plan->c2p, dec_c);
    pcc.flush(b, &plan->pcc, dec_c);
    pint.flush(b, &plan->pint, dec_c);
    pfine.flush(b, &plan->pfine, dec_f);
    psf[0].flush(b, &plan->psf[0], dec_cf1);
    psf[1].flush(b, &plan->psf[1], dec_cf2);
    psf[2].flush(b, &plan->psf[2], dec_c);
    flux_list(d, R, loc, nbs, b, &plan->flux);
    if (mhd) emf_list(d, R, loc, nbs, b, dx, &plan->emf, &plan->emf_add);
  }
  return true;
}

}  // namespace athg

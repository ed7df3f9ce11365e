// athg_amr.cpp -- adaptive mesh refinement, host side (see athg_amr.h).
#include "athg_amr.h"

#include <algorithm>
#include <map>
#include <set>
#include <tuple>

namespace athg {

namespace {

using Key = std::tuple<int, int64_t, int64_t, int64_t>;

Key key_of(const SmrLoc& l) { return Key(l.level, l.lx[0], l.lx[1], l.lx[2]); }

SmrLoc loc_of(const Key& k) {
  SmrLoc l;
  l.level = std::get<0>(k);
  l.lx[0] = std::get<1>(k); l.lx[1] = std::get<2>(k); l.lx[2] = std::get<3>(k);
  return l;
}

// The block tree as sets of leaves and refined nodes (levels relative to the root grid)
struct Tree {
  int nrb[3];
  std::set<Key> leaves, inner;

  int64_t wrap(int d, int level, int64_t x) const {
    const int64_t n = (int64_t)nrb[d] << level;
    return ((x % n) + n) % n;
  }

  // MeshBlockTree::AddMeshBlock: walk down from the root, refining leaves on the way
  void add_block(int L, const int64_t x[3]) {
    for (int lv = 0; lv < L; ++lv) {
      const int sh = L - lv;
      Key a(lv, x[0] >> sh, x[1] >> sh, x[2] >> sh);
      if (leaves.count(a)) refine(a);
    }
  }

  // MeshBlockTree::Refine: eight children, then every neighbour of the node at its own
  // level must exist (2:1 balance)
  void refine(const Key& k) {
    if (!leaves.count(k)) return;  // already refined
    leaves.erase(k);
    inner.insert(k);
    const int L = std::get<0>(k);
    const int64_t x[3] = {std::get<1>(k), std::get<2>(k), std::get<3>(k)};
    for (int c = 0; c < 8; ++c)
      leaves.insert(Key(L + 1, 2 * x[0] + (c & 1), 2 * x[1] + ((c >> 1) & 1), 2 * x[2] + (c >> 2)));
    for (int oz = -1; oz <= 1; ++oz)
      for (int oy = -1; oy <= 1; ++oy)
        for (int ox = -1; ox <= 1; ++ox) {
          if (ox == 0 && oy == 0 && oz == 0) continue;
          const int64_t n[3] = {wrap(0, L, x[0] + ox), wrap(1, L, x[1] + oy), wrap(2, L, x[2] + oz)};
          add_block(L, n);
        }
  }

  // MeshBlockTree::Derefine: not if a neighbour's children next to this node are refined
  void derefine(const Key& k) {
    if (!inner.count(k)) return;
    const int L = std::get<0>(k);
    const int64_t x[3] = {std::get<1>(k), std::get<2>(k), std::get<3>(k)};
    for (int oz = -1; oz <= 1; ++oz)
      for (int oy = -1; oy <= 1; ++oy)
        for (int ox = -1; ox <= 1; ++ox) {
          const int o[3] = {ox, oy, oz};
          const int64_t n[3] = {wrap(0, L, x[0] + ox), wrap(1, L, x[1] + oy), wrap(2, L, x[2] + oz)};
          if (!inner.count(Key(L, n[0], n[1], n[2]))) continue;
          int lo[3], hi[3];
          for (int d = 0; d < 3; ++d) {
            if (o[d] == -1) lo[d] = hi[d] = 1;
            else if (o[d] == 1) lo[d] = hi[d] = 0;
            else { lo[d] = 0; hi[d] = 1; }
          }
          for (int lk = lo[2]; lk <= hi[2]; ++lk)
            for (int lj = lo[1]; lj <= hi[1]; ++lj)
              for (int li = lo[0]; li <= hi[0]; ++li)
                if (inner.count(Key(L + 1, 2 * n[0] + li, 2 * n[1] + lj, 2 * n[2] + lk))) return;
        }
    remove_children(k);
    inner.erase(k);
    leaves.insert(k);
  }

  void remove_children(const Key& k) {
    const int L = std::get<0>(k);
    const int64_t x[3] = {std::get<1>(k), std::get<2>(k), std::get<3>(k)};
    for (int c = 0; c < 8; ++c) {
      Key ch(L + 1, 2 * x[0] + (c & 1), 2 * x[1] + ((c >> 1) & 1), 2 * x[2] + (c >> 2));
      if (inner.count(ch)) {
        remove_children(ch);
        inner.erase(ch);
      }
      leaves.erase(ch);
    }
  }
};

}  // namespace

int amr_flag(double maxeps, double threshold, double deref_fraction, int level, int max_level,
             const int* nblevel27, int deref_threshold, int* deref_count) {
  int ret = 0;
  if (maxeps > threshold) ret = 1;
  else if (maxeps < deref_fraction * threshold) ret = -1;
  const int aret = std::max(-1, ret);
  int flag = 0;
  if (aret >= 0) *deref_count = 0;
  if (aret > 0) {
    flag = (level == max_level) ? 0 : 1;
  } else if (aret < 0) {
    if (level == 0) {
      *deref_count = 0;
    } else {
      ++*deref_count;
      int ec = 0;
      for (int q = 0; q < 27; ++q)
        if (nblevel27[q] > level) ++ec;
      if (ec == 0 && *deref_count >= deref_threshold) flag = -1;
    }
  }
  return flag;
}

std::vector<int> amr_tree_order(const int nrb[3], const std::vector<SmrLoc>& leaves) {
  const int nbmax = std::max(nrb[0], std::max(nrb[1], nrb[2]));
  int rl = 0;
  while ((1 << rl) < nbmax) ++rl;
  int depth = 0;
  for (const SmrLoc& b : leaves) depth = std::max(depth, rl + b.level);
  std::vector<std::pair<uint64_t, int>> keys(leaves.size());
  for (size_t q = 0; q < leaves.size(); ++q) {
    const SmrLoc& b = leaves[q];
    const int sh = depth - (rl + b.level);
    const uint64_t x = (uint64_t)b.lx[0] << sh, y = (uint64_t)b.lx[1] << sh,
                   z = (uint64_t)b.lx[2] << sh;
    uint64_t key = 0;
    for (int bit = depth - 1; bit >= 0; --bit)
      key = (key << 3) | (((z >> bit) & 1) << 2) | (((y >> bit) & 1) << 1) | ((x >> bit) & 1);
    keys[q] = std::make_pair(key, (int)q);
  }
  std::sort(keys.begin(), keys.end());
  std::vector<int> order(leaves.size());
  for (size_t q = 0; q < keys.size(); ++q) order[q] = keys[q].second;
  return order;
}

bool amr_update_tree(const int nrb[3], const std::vector<SmrLoc>& leaves,
                     const std::vector<int>& flags, std::vector<SmrLoc>* out) {
  const std::vector<int> order = amr_tree_order(nrb, leaves);
  int tnref = 0, tnderef = 0;
  for (int f : flags) {
    if (f == 1) ++tnref;
    if (f == -1) ++tnderef;
  }
  *out = leaves;
  if (tnref == 0 && tnderef < 8) return false;
  std::vector<SmrLoc> lref, lderef, clderef;
  for (int g : order) {
    if (flags[g] == 1) lref.push_back(leaves[g]);
    if (flags[g] == -1 && tnderef >= 8) lderef.push_back(leaves[g]);
  }
  // parents whose eight children are all flagged, found as eight consecutive entries of
  // the gid-ordered list starting at the child with even indices
  for (size_t n = 0; n < lderef.size(); ++n) {
    const SmrLoc& a = lderef[n];
    if ((a.lx[0] & 1) || (a.lx[1] & 1) || (a.lx[2] & 1)) continue;
    size_t r = n;
    int rr = 0;
    for (int k = 0; k <= 1; ++k)
      for (int j = 0; j <= 1; ++j)
        for (int i = 0; i <= 1; ++i) {
          if (r < lderef.size()) {
            const SmrLoc& b = lderef[r];
            if (a.lx[0] + i == b.lx[0] && a.lx[1] + j == b.lx[1] && a.lx[2] + k == b.lx[2] &&
                a.level == b.level)
              ++rr;
            ++r;
          }
        }
    if (rr == 8) {
      SmrLoc p;
      p.level = a.level - 1;
      for (int d = 0; d < 3; ++d) p.lx[d] = a.lx[d] >> 1;
      clderef.push_back(p);
    }
  }
  // the reference sorts all but the last candidate, finest first
  if (clderef.size() > 1)
    std::sort(clderef.begin(), clderef.end() - 1,
              [](const SmrLoc& l, const SmrLoc& r) { return l.level > r.level; });
  Tree t;
  for (int d = 0; d < 3; ++d) t.nrb[d] = nrb[d];
  for (const SmrLoc& l : leaves) {
    t.leaves.insert(key_of(l));
    for (int lv = l.level - 1; lv >= 0; --lv) {
      const int sh = l.level - lv;
      t.inner.insert(Key(lv, l.lx[0] >> sh, l.lx[1] >> sh, l.lx[2] >> sh));
    }
  }
  for (const SmrLoc& l : lref) t.refine(key_of(l));
  for (const SmrLoc& l : clderef) t.derefine(key_of(l));
  out->clear();
  for (const Key& k : t.leaves) out->push_back(loc_of(k));
  std::sort(out->begin(), out->end(), [](const SmrLoc& p, const SmrLoc& q) {
    return std::make_tuple(p.level, p.lx[2], p.lx[1], p.lx[0]) <
           std::make_tuple(q.level, q.lx[2], q.lx[1], q.lx[0]);
  });
  std::set<Key> before;
  for (const SmrLoc& l : leaves) before.insert(key_of(l));
  return before != t.leaves;
}

void amr_fill(const SmrDims& d, bool mhd, const std::vector<SmrLoc>& old_loc,
              const AmrArrays& old, const std::vector<double>& old_dx,
              const std::vector<int>& old_deref, const std::vector<SmrLoc>& new_loc,
              const std::vector<double>& new_dx, const std::vector<double>& new_xvf,
              const std::vector<double>& new_xvc, int ncmax, int nccmax, AmrArrays* nw,
              std::vector<int>* new_deref) {
  const size_t nb = new_loc.size();
  const int64_t NC = 5 * d.ncell, CC = 5 * d.ccell;
  nw->u.assign(nb * NC, 0.0);
  nw->cu.assign(nb * CC, 0.0);
  if (mhd) {
    nw->b1.assign(nb * d.nf1, 0.0); nw->b2.assign(nb * d.nf2, 0.0); nw->b3.assign(nb * d.nf3, 0.0);
    nw->cb1.assign(nb * d.cf1, 0.0); nw->cb2.assign(nb * d.cf2, 0.0); nw->cb3.assign(nb * d.cf3, 0.0);
  }
  new_deref->assign(nb, 0);
  std::map<Key, int> old_of;
  for (size_t q = 0; q < old_loc.size(); ++q) old_of[key_of(old_loc[q])] = (int)q;
  auto copy_block = [](const std::vector<double>& src, std::vector<double>* dst, int64_t n,
                       int from, int to) {
    std::copy(src.begin() + from * n, src.begin() + (from + 1) * n, dst->begin() + to * n);
  };
  for (size_t q = 0; q < nb; ++q) {
    const SmrLoc& nl = new_loc[q];
    auto same = old_of.find(key_of(nl));
    if (same != old_of.end()) {  // the block stays: its arrays and counter move along
      const int o = same->second;
      copy_block(old.u, &nw->u, NC, o, (int)q);
      copy_block(old.cu, &nw->cu, CC, o, (int)q);
      if (mhd) {
        copy_block(old.b1, &nw->b1, d.nf1, o, (int)q); copy_block(old.b2, &nw->b2, d.nf2, o, (int)q);
        copy_block(old.b3, &nw->b3, d.nf3, o, (int)q);
        copy_block(old.cb1, &nw->cb1, d.cf1, o, (int)q); copy_block(old.cb2, &nw->cb2, d.cf2, o, (int)q);
        copy_block(old.cb3, &nw->cb3, d.cf3, o, (int)q);
      }
      (*new_deref)[q] = old_deref[o];
      continue;
    }
    double* u = &nw->u[q * NC];
    double* cu = &nw->cu[q * CC];
    double* b1 = mhd ? &nw->b1[q * d.nf1] : nullptr;
    double* b2 = mhd ? &nw->b2[q * d.nf2] : nullptr;
    double* b3 = mhd ? &nw->b3[q * d.nf3] : nullptr;
    double* cb1 = mhd ? &nw->cb1[q * d.cf1] : nullptr;
    double* cb2 = mhd ? &nw->cb2[q * d.cf2] : nullptr;
    double* cb3 = mhd ? &nw->cb3[q * d.cf3] : nullptr;
    Key parent(nl.level - 1, nl.lx[0] >> 1, nl.lx[1] >> 1, nl.lx[2] >> 1);
    auto par = nl.level > 0 ? old_of.find(parent) : old_of.end();
    if (par != old_of.end()) {
      // FillSameRankCoarseToFineAMR: the parent's cells around this octant (one cell of
      // margin) into the coarse buffer, then prolongation of U and of the face field
      const int o = par->second;
      const double* ou = &old.u[o * NC];
      const int il = d.cis - 1, iu = d.cie + 1, jl = d.cjs - 1, ju = d.cje + 1, kl = d.cks - 1,
                ku = d.cke + 1;
      const int ci0 = (int)(nl.lx[0] & 1) * d.nx1 / 2 + d.is - 1;
      const int cj0 = (int)(nl.lx[1] & 1) * d.nx2 / 2 + d.js - 1;
      const int ck0 = (int)(nl.lx[2] & 1) * d.nx3 / 2 + d.ks - 1;
      for (int nv = 0; nv < 5; ++nv)
        for (int k = kl; k <= ku; ++k)
          for (int j = jl; j <= ju; ++j)
            for (int i = il; i <= iu; ++i)
              cu[nv * d.ccell + d.cc(k, j, i)] =
                  ou[nv * d.ncell + d.c(ck0 + k - kl, cj0 + j - jl, ci0 + i - il)];
      const double* xf = &new_xvf[q * 3 * ncmax];
      const double* xc = &new_xvc[q * 3 * nccmax];
      for (int nv = 0; nv < 5; ++nv)
        for (int k = d.cks; k <= d.cke; ++k)
          for (int j = d.cjs; j <= d.cje; ++j)
            for (int i = d.cis; i <= d.cie; ++i) {
              const SmrAxis a1 = smr_axis(xc, xf, i, (i - d.cis) * 2 + d.is);
              const SmrAxis a2 = smr_axis(xc + nccmax, xf + ncmax, j, (j - d.cjs) * 2 + d.js);
              const SmrAxis a3 = smr_axis(xc + 2 * nccmax, xf + 2 * ncmax, k, (k - d.cks) * 2 + d.ks);
              smr_prolong_cc(d, cu + nv * d.ccell, u + nv * d.ncell, k, j, i, a1, a2, a3);
            }
      if (mhd) {
        const double* o1 = &old.b1[o * d.nf1];
        const double* o2 = &old.b2[o * d.nf2];
        const double* o3 = &old.b3[o * d.nf3];
        for (int k = kl; k <= ku; ++k)
          for (int j = jl; j <= ju; ++j)
            for (int i = il; i <= iu + 1; ++i)
              cb1[d.cf1i(k, j, i)] = o1[d.f1(ck0 + k - kl, cj0 + j - jl, ci0 + i - il)];
        for (int k = kl; k <= ku; ++k)
          for (int j = jl; j <= ju + 1; ++j)
            for (int i = il; i <= iu; ++i)
              cb2[d.cf2i(k, j, i)] = o2[d.f2(ck0 + k - kl, cj0 + j - jl, ci0 + i - il)];
        for (int k = kl; k <= ku + 1; ++k)
          for (int j = jl; j <= ju; ++j)
            for (int i = il; i <= iu; ++i)
              cb3[d.cf3i(k, j, i)] = o3[d.f3(ck0 + k - kl, cj0 + j - jl, ci0 + i - il)];
        auto ax = [&](int a, int c, int cs, int fs) {
          return smr_axis(xc + a * nccmax, xf + a * ncmax, c, (c - cs) * 2 + fs);
        };
        for (int k = d.cks; k <= d.cke; ++k)
          for (int j = d.cjs; j <= d.cje; ++j)
            for (int i = d.cis; i <= d.cie + 1; ++i)
              smr_prolong_f1(d, cb1, b1, k, j, i, ax(1, j, d.cjs, d.js), ax(2, k, d.cks, d.ks));
        for (int k = d.cks; k <= d.cke; ++k)
          for (int j = d.cjs; j <= d.cje + 1; ++j)
            for (int i = d.cis; i <= d.cie; ++i)
              smr_prolong_f2(d, cb2, b2, k, j, i, ax(0, i, d.cis, d.is), ax(2, k, d.cks, d.ks));
        for (int k = d.cks; k <= d.cke + 1; ++k)
          for (int j = d.cjs; j <= d.cje; ++j)
            for (int i = d.cis; i <= d.cie; ++i)
              smr_prolong_f3(d, cb3, b3, k, j, i, ax(0, i, d.cis, d.is), ax(1, j, d.cjs, d.js));
        for (int k = d.cks; k <= d.cke; ++k)
          for (int j = d.cjs; j <= d.cje; ++j)
            for (int i = d.cis; i <= d.cie; ++i)
              smr_prolong_internal(d, b1, b2, b3, k, j, i, &new_dx[3 * q]);
      }
      continue;
    }
    // FillSameRankFineToCoarseAMR: each of the eight old children, in tree order,
    // restricted into its octant
    for (int m = 0; m < 8; ++m) {
      const int mx = m & 1, my = (m >> 1) & 1, mz = m >> 2;
      Key ck(nl.level + 1, 2 * nl.lx[0] + mx, 2 * nl.lx[1] + my, 2 * nl.lx[2] + mz);
      auto ch = old_of.find(ck);
      if (ch == old_of.end()) continue;
      const int o = ch->second;
      const double* cdx = &old_dx[3 * o];
      const double vol = cdx[0] * cdx[1] * cdx[2];
      const int il = d.is + mx * d.nx1 / 2, jl = d.js + my * d.nx2 / 2, kl = d.ks + mz * d.nx3 / 2;
      const double* ou = &old.u[o * NC];
      auto fc = [&](int c, int a) {
        const int cs = a == 0 ? d.cis : (a == 1 ? d.cjs : d.cks);
        const int fs = a == 0 ? d.is : (a == 1 ? d.js : d.ks);
        return (c - cs) * 2 + fs;
      };
      for (int nv = 0; nv < 5; ++nv)
        for (int k = d.cks; k <= d.cke; ++k)
          for (int j = d.cjs; j <= d.cje; ++j)
            for (int i = d.cis; i <= d.cie; ++i)
              u[nv * d.ncell + d.c(kl + k - d.cks, jl + j - d.cjs, il + i - d.cis)] =
                  smr_restrict_cc(d, ou + nv * d.ncell, d.c(fc(k, 2), fc(j, 1), fc(i, 0)), vol);
      if (mhd) {
        const double* o1 = &old.b1[o * d.nf1];
        const double* o2 = &old.b2[o * d.nf2];
        const double* o3 = &old.b3[o * d.nf3];
        for (int k = d.cks; k <= d.cke; ++k)
          for (int j = d.cjs; j <= d.cje; ++j)
            for (int i = d.cis; i <= d.cie + 1; ++i)
              b1[d.f1(kl + k - d.cks, jl + j - d.cjs, il + i - d.cis)] =
                  smr_restrict_f1(d, o1, d.f1(fc(k, 2), fc(j, 1), fc(i, 0)), cdx[1] * cdx[2]);
        for (int k = d.cks; k <= d.cke; ++k)
          for (int j = d.cjs; j <= d.cje + 1; ++j)
            for (int i = d.cis; i <= d.cie; ++i)
              b2[d.f2(kl + k - d.cks, jl + j - d.cjs, il + i - d.cis)] =
                  smr_restrict_f2(d, o2, d.f2(fc(k, 2), fc(j, 1), fc(i, 0)), cdx[0] * cdx[2]);
        for (int k = d.cks; k <= d.cke + 1; ++k)
          for (int j = d.cjs; j <= d.cje; ++j)
            for (int i = d.cis; i <= d.cie; ++i)
              b3[d.f3(kl + k - d.cks, jl + j - d.cjs, il + i - d.cis)] =
                  smr_restrict_f3(d, o3, d.f3(fc(k, 2), fc(j, 1), fc(i, 0)), cdx[0] * cdx[1]);
      }
    }
  }
}

}  // namespace athg

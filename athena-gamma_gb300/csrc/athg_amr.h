// athg_amr.h -- adaptive mesh refinement on the host side: refinement flags, the block-tree
// update and the data of new blocks, with the reference's rules and arithmetic.
//
//   flags         MeshRefinement::CheckRefinementCondition   mesh/mesh_refinement.cpp:1003-1062
//   tree update   Mesh::UpdateMeshBlockTree                  mesh/amr_loadbalance.cpp:178-317
//                 MeshBlockTree::Refine / Derefine           mesh/meshblock_tree.cpp:166-308
//   new blocks    Mesh::FillSameRankCoarseToFineAMR,         mesh/amr_loadbalance.cpp:805-976
//                 FillSameRankFineToCoarseAMR
// Blocks that keep their place keep their arrays (and coarse buffers and derefinement
// counters), as the reference reuses their MeshBlock objects.
#pragma once
#include <vector>

#include "athg_smr.h"

namespace athg {

// Refine flag (+1 refine, -1 derefine, 0 keep) of one block from its criterion value
// maxeps (refine above threshold, derefine below deref_fraction * threshold, as the
// reference's blast RefinementCondition); updates the block's derefinement counter.
// level/max_level relative to the root grid; nblevel27: smr_neighbor_levels of the block.
int amr_flag(double maxeps, double threshold, double deref_fraction, int level, int max_level,
             const int* nblevel27, int deref_threshold, int* deref_count);

// gid order of the reference's block tree: order[g] = index into `leaves`
std::vector<int> amr_tree_order(const int nrb[3], const std::vector<SmrLoc>& leaves);

// UpdateMeshBlockTree for flags aligned with `leaves`; returns whether the tree changed and
// the new leaves sorted by level, then lx3, lx2, lx1
bool amr_update_tree(const int nrb[3], const std::vector<SmrLoc>& leaves,
                     const std::vector<int>& flags, std::vector<SmrLoc>* out);

// Every block's whole arrays (FP64), block after block
struct AmrArrays {
  std::vector<double> u, b1, b2, b3;       // fine arrays with ghosts
  std::vector<double> cu, cb1, cb2, cb3;   // coarse buffers
};

// Arrays of the new blocks: kept blocks copy theirs, new fine blocks are prolongated from
// their old parent (conserved variables and face fields), new coarse blocks restricted
// from their eight old children. dx: [block][3]; xvf/xvc: cell centres of the new blocks
// ([block][3][ncmax], [block][3][nccmax]). New blocks start with zero counters.
void amr_fill(const SmrDims& d, bool mhd, const std::vector<SmrLoc>& old_loc,
              const AmrArrays& old, const std::vector<double>& old_dx,
              const std::vector<int>& old_deref, const std::vector<SmrLoc>& new_loc,
              const std::vector<double>& new_dx, const std::vector<double>& new_xvf,
              const std::vector<double>& new_xvc, int ncmax, int nccmax, AmrArrays* nw,
              std::vector<int>* new_deref);

}  // namespace athg

// athg_df.h -- host interface of the double-float flux sweeps and corner EMFs
// (athg_df.cu, precision ATHG_DFLOAT).
#pragma once
#include <cuda_runtime.h>

#include "athg_stage.cuh"

namespace athg {

// whether the double-float path has this reconstruction and Riemann solver (donor cell or
// PLM; HLLC or HLLE for hydro, HLLD or HLLE for MHD)
bool df_supported(int mhd, int solver, int xorder);
// Hydro::CalculateFluxes over every block: W and bcc split once into pairs (wp: scratch of
// (mhd ? 8 : 5) * ncell * nb pairs), then the three sweeps into the FP64 flux arrays
// fast: wp already holds the pairs (k_c2p_df), and the hydro fluxes are stored as pairs
// for df_update
void df_fluxes(const Geom& g, const StagePtrs<double>& p, bool mhd, int solver, int order,
               const Phys& ph, float2* wp, bool fast, cudaStream_t st);
// Field::ComputeCornerE over every block into the FP64 edge arrays; cce: scratch of
// 3 * ncell * nb pairs (the cell-centred EMF). Reads the face EMFs and CT weights that
// df_fluxes stores as double-float pairs in flux components 5..7 (no other kernel reads
// those components on this path).
// fast: the cell-centred EMF from the pairs wp, the edge EMFs stored as pairs for df_update
void df_corner_emf(const Geom& g, const StagePtrs<double>& p, float2* cce, const float2* wp,
                   bool fast, cudaStream_t st);
// The fast variant's update (register averaging, flux divergence, CT), primitive recovery
// (also leaving the pairs in wp) and CFL time step: inputs and outputs of k_update, k_c2p
// and k_block_dt, arithmetic in double-float.
void df_update(const Geom& g, const StagePtrs<double>& p, bool mhd, const StageW& sw,
               cudaStream_t st);
void df_c2p(const Geom& g, const StagePtrs<double>& p, bool mhd, const Phys& ph, float2* wp,
            cudaStream_t st);
void df_block_dt(const Geom& g, const StagePtrs<double>& p, bool mhd, const Phys& ph,
                 const float2* wp, unsigned long long* dtmin, cudaStream_t st);

}  // namespace athg

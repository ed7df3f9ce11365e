// athg_launch.cuh -- host-side launch sequences for one precision (T = double: plain
// FP64 path, T = float: mixed path). Instantiated once per precision in
// kernels_f64.cu (built without FMA contraction, so the FP64 path reproduces the
// reference's arithmetic bit for bit) and kernels_f32.cu.
#pragma once
#include <algorithm>
#include "athg_stage.cuh"

namespace athg {

inline Box make_box(int il, int iu, int jl, int ju, int kl, int ku) {
  return box_make(il, iu, jl, ju, kl, ku);
}
inline dim3 box_grid(const Box& b, int nblocks, int tpb) {
  return dim3((unsigned)((b.ni * b.nj + tpb - 1) / tpb), (unsigned)b.nk, (unsigned)nblocks);
}

// Launch shape of the flux sweeps, picked per context by the autotuner in athg_api.cu:
// threads per block of the x1 sweep and of the marching sweeps, and the faces per segment of
// a marching pencil (0: whole pencil).
struct FluxTune {
  int x1_tpb = 128;
  int march_tpb = 128;
  int seg = 16;
};

template <typename T>
struct Launcher {
  // Hydro::CalculateFluxes over every block: three directional sweeps.
  static void fluxes(const Geom& g, const StagePtrs<T>& p, bool mhd, int solver, int order,
                     const Phys& ph, const FluxTune& tune, cudaStream_t st);
  // Field::ComputeCornerE over every block.
  static void corner_emf(const Geom& g, const StagePtrs<T>& p, cudaStream_t st);
  // IntegrateHydro + IntegrateField (register average, flux divergence, CT).
  static void update(const Geom& g, const StagePtrs<T>& p, bool mhd, const StageW& sw,
                     cudaStream_t st);
  // EquationOfState::ConservedToPrimitive over interior and ghost cells.
  static void c2p(const Geom& g, const StagePtrs<T>& p, bool mhd, const Phys& ph,
                  cudaStream_t st);
  // Mixed VL2: update + interior primitive recovery from `sb.in` into `sb.out`
  // (k_update_c2p; no-op for the FP64 path, which never takes this route). phi2: the
  // potential as FP32 pairs [nb][cells] for the self-gravity source, or nullptr.
  static void update_c2p(const Geom& g, const StagePtrs<T>& p, bool mhd, const StageW& sw,
                         const Phys& ph, const StateBufs& sb, unsigned long long* dtmin,
                         const float2* phi2, cudaStream_t st);
  // HydroSourceTerms::SelfGravity over every block (phi: [nb][cells] potential).
  static void self_gravity(const Geom& g, const StagePtrs<T>& p, bool mhd, const StageW& sw,
                           const double* phi, cudaStream_t st);
  // Hydro::NewBlockTimeStep over every block, reduced to one minimum.
  static void block_dt(const Geom& g, const StagePtrs<T>& p, bool mhd, const Phys& ph,
                       unsigned long long* dtmin, cudaStream_t st);
};

#ifdef ATHG_LAUNCH_IMPL
// the mixed MHD HLLD sweeps (donor cell, PLM) on 64^3 blocks with two ghost layers take the
// fixed-size kernels (compile-time strides, BlockDims<68>)
template <typename T, int ORDER>
static bool fixed68(const Geom& g, bool mhd, int solver) {
  return kMixed<T> && ORDER <= 2 && mhd && solver == HLLD && g.nc1 == 68 && g.nc2 == 68 &&
         g.nc3 == 68;
}

template <typename T, int DIR, int ORDER>
static void flux_dir(const Geom& g, const StagePtrs<T>& p, bool mhd, int solver,
                     const Phys& ph, const FluxTune& tune, cudaStream_t st) {
  int il = g.is, iu = g.ie, jl = g.js, ju = g.je, kl = g.ks, ku = g.ke;
  if (DIR == 0) {
    iu = g.ie + 1;
    if (mhd) { jl = g.js - 1; ju = g.je + 1; kl = g.ks - 1; ku = g.ke + 1; }
  } else if (DIR == 1) {
    ju = g.je + 1; il = g.is - 1; iu = g.ie + 1;
    if (mhd) { kl = g.ks - 1; ku = g.ke + 1; }
  } else {
    ku = g.ke + 1;
    if (mhd) { il = g.is - 1; iu = g.ie + 1; jl = g.js - 1; ju = g.je + 1; }
  }
  if constexpr (DIR != 0) {
    // marching sweeps: pencils over (i, k) for DIR=1 and (i, j) for DIR=2
    Box pb = DIR == 1 ? make_box(il, iu, kl, ku, 0, 0) : make_box(il, iu, jl, ju, 0, 0);
    const int fs = DIR == 1 ? jl : kl, fe = DIR == 1 ? ju : ku;
    // pencils split into segments of ~tune.seg faces
    const unsigned nseg = tune.seg > 0 ? (unsigned)std::max(1, (fe - fs + 1) / tune.seg) : 1u;
    const int tpb = tune.march_tpb;
    dim3 grid((unsigned)((pb.ni * pb.nj + tpb - 1) / tpb), nseg, (unsigned)g.nb);
    if (fixed68<T, ORDER>(g, mhd, solver)) {
      k_flux_march<T, DIR, ORDER, HLLD, true, 68><<<grid, tpb, 0, st>>>(g, p, pb, ph, fs, fe);
    } else if (mhd) {
      if (solver == HLLD)
        k_flux_march<T, DIR, ORDER, HLLD, true><<<grid, tpb, 0, st>>>(g, p, pb, ph, fs, fe);
      else if (solver == LHLLD)
        k_flux_march<T, DIR, ORDER, LHLLD, true><<<grid, tpb, 0, st>>>(g, p, pb, ph, fs, fe);
      else
        k_flux_march<T, DIR, ORDER, HLLE, true><<<grid, tpb, 0, st>>>(g, p, pb, ph, fs, fe);
    } else {
      if (solver == HLLC)
        k_flux_march<T, DIR, ORDER, HLLC, false><<<grid, tpb, 0, st>>>(g, p, pb, ph, fs, fe);
      else if (solver == LHLLC)
        k_flux_march<T, DIR, ORDER, LHLLC, false><<<grid, tpb, 0, st>>>(g, p, pb, ph, fs, fe);
      else
        k_flux_march<T, DIR, ORDER, HLLE, false><<<grid, tpb, 0, st>>>(g, p, pb, ph, fs, fe);
    }
  } else {
  Box b = make_box(il, iu, jl, ju, kl, ku);
  if constexpr (ORDER == 3) {
    // PPM: each cell reconstructed once per sweep (k_flux_x1_ppm), when a block's rows fit
    // the default 48 KB of shared memory
    const int nw = mhd ? 7 : 5, cells = b.ni + 1;
    const int rows = std::max(1, 256 / cells);
    const size_t smem = 2 * (size_t)rows * nw * cells * sizeof(T);
    if (smem <= 48 * 1024) {
      const int tpb = std::min(256, ((rows * cells + 31) / 32) * 32);
      dim3 grid((unsigned)((b.nj * b.nk + rows - 1) / rows), 1, (unsigned)g.nb);
      if (mhd) {
        if (solver == HLLD) k_flux_x1_ppm<T, HLLD, true><<<grid, tpb, smem, st>>>(g, p, b, ph, rows);
        else if (solver == LHLLD) k_flux_x1_ppm<T, LHLLD, true><<<grid, tpb, smem, st>>>(g, p, b, ph, rows);
        else k_flux_x1_ppm<T, HLLE, true><<<grid, tpb, smem, st>>>(g, p, b, ph, rows);
      } else {
        if (solver == HLLC) k_flux_x1_ppm<T, HLLC, false><<<grid, tpb, smem, st>>>(g, p, b, ph, rows);
        else if (solver == LHLLC) k_flux_x1_ppm<T, LHLLC, false><<<grid, tpb, smem, st>>>(g, p, b, ph, rows);
        else k_flux_x1_ppm<T, HLLE, false><<<grid, tpb, smem, st>>>(g, p, b, ph, rows);
      }
      return;
    }
  }
  const int tpb = tune.x1_tpb;
  dim3 grid = box_grid(b, g.nb, tpb);
  if (fixed68<T, ORDER>(g, mhd, solver)) {
    k_flux<T, DIR, ORDER, HLLD, true, 68><<<grid, tpb, 0, st>>>(g, p, b, ph);
  } else if (mhd) {
    if (solver == HLLD) k_flux<T, DIR, ORDER, HLLD, true><<<grid, tpb, 0, st>>>(g, p, b, ph);
    else if (solver == LHLLD) k_flux<T, DIR, ORDER, LHLLD, true><<<grid, tpb, 0, st>>>(g, p, b, ph);
    else k_flux<T, DIR, ORDER, HLLE, true><<<grid, tpb, 0, st>>>(g, p, b, ph);
  } else {
    if (solver == HLLC) k_flux<T, DIR, ORDER, HLLC, false><<<grid, tpb, 0, st>>>(g, p, b, ph);
    else if (solver == LHLLC) k_flux<T, DIR, ORDER, LHLLC, false><<<grid, tpb, 0, st>>>(g, p, b, ph);
    else k_flux<T, DIR, ORDER, HLLE, false><<<grid, tpb, 0, st>>>(g, p, b, ph);
  }
  }
}

template <typename T>
void Launcher<T>::fluxes(const Geom& g, const StagePtrs<T>& p, bool mhd, int solver,
                         int order, const Phys& ph, const FluxTune& tune, cudaStream_t st) {
  if (order == 1) {
    flux_dir<T, 0, 1>(g, p, mhd, solver, ph, tune, st);
    flux_dir<T, 1, 1>(g, p, mhd, solver, ph, tune, st);
    flux_dir<T, 2, 1>(g, p, mhd, solver, ph, tune, st);
  } else if (order == 3) {
    flux_dir<T, 0, 3>(g, p, mhd, solver, ph, tune, st);
    flux_dir<T, 1, 3>(g, p, mhd, solver, ph, tune, st);
    flux_dir<T, 2, 3>(g, p, mhd, solver, ph, tune, st);
  } else {
    flux_dir<T, 0, 2>(g, p, mhd, solver, ph, tune, st);
    flux_dir<T, 1, 2>(g, p, mhd, solver, ph, tune, st);
    flux_dir<T, 2, 2>(g, p, mhd, solver, ph, tune, st);
  }
}

template <typename T>
void Launcher<T>::corner_emf(const Geom& g, const StagePtrs<T>& p, cudaStream_t st) {
  Box b = make_box(g.is, g.ie + 1, g.js, g.je + 1, g.ks, g.ke + 1);
  // 64^3 blocks with two ghost layers (68^3 cells) take the fixed-size instantiation
  if (kMixed<T> && g.nc1 == 68 && g.nc2 == 68 && g.nc3 == 68)
    k_corner_emf<T, 68><<<box_grid(b, g.nb, 128), 128, 0, st>>>(g, p, b);
  else
    k_corner_emf<T, 0><<<box_grid(b, g.nb, 128), 128, 0, st>>>(g, p, b);
}

template <typename T>
void Launcher<T>::update(const Geom& g, const StagePtrs<T>& p, bool mhd, const StageW& sw,
                         cudaStream_t st) {
  Box b = mhd ? make_box(g.is, g.ie + 1, g.js, g.je + 1, g.ks, g.ke + 1)
              : make_box(g.is, g.ie, g.js, g.je, g.ks, g.ke);
  if (mhd) k_update<T, true><<<box_grid(b, g.nb, 128), 128, 0, st>>>(g, p, b, sw);
  else k_update<T, false><<<box_grid(b, g.nb, 128), 128, 0, st>>>(g, p, b, sw);
}

template <typename T>
void Launcher<T>::update_c2p(const Geom& g, const StagePtrs<T>& p, bool mhd, const StageW& sw,
                             const Phys& ph, const StateBufs& sb, unsigned long long* dtmin,
                             const float2* phi2, cudaStream_t st) {
  if constexpr (kMixed<T>) {
    Box b = make_box(g.is, g.ie, g.js, g.je, g.ks, g.ke);
    const dim3 gr = box_grid(b, g.nb, 128);
    // MHD on 64^3 blocks with two ghost layers (68^3 cells): the fixed-size instantiation
    // (compile-time strides; on a GB300 at 256^3 1.096 and 1.156 ms per launch without and
    // with the time step, against 1.226 and 1.281 ms for the general one)
    const bool fixed68 = mhd && g.nc1 == 68 && g.nc2 == 68 && g.nc3 == 68;
#define ATHG_UC2P(M, D, S, N) \
  k_update_c2p<M, D, S, N><<<gr, 128, 0, st>>>(g, p, b, sw, ph, sb, dtmin, phi2)
    if (fixed68) {
      if (phi2) { if (dtmin) ATHG_UC2P(true, true, true, 68); else ATHG_UC2P(true, false, true, 68); }
      else { if (dtmin) ATHG_UC2P(true, true, false, 68); else ATHG_UC2P(true, false, false, 68); }
    } else if (phi2) {
      if (mhd) { if (dtmin) ATHG_UC2P(true, true, true, 0); else ATHG_UC2P(true, false, true, 0); }
      else { if (dtmin) ATHG_UC2P(false, true, true, 0); else ATHG_UC2P(false, false, true, 0); }
    } else {
      if (mhd) { if (dtmin) ATHG_UC2P(true, true, false, 0); else ATHG_UC2P(true, false, false, 0); }
      else { if (dtmin) ATHG_UC2P(false, true, false, 0); else ATHG_UC2P(false, false, false, 0); }
    }
#undef ATHG_UC2P
  }
}

template <typename T>
void Launcher<T>::self_gravity(const Geom& g, const StagePtrs<T>& p, bool mhd, const StageW& sw,
                               const double* phi, cudaStream_t st) {
  Box b = make_box(g.is, g.ie, g.js, g.je, g.ks, g.ke);
  if (mhd) k_self_gravity<T, true><<<box_grid(b, g.nb, 128), 128, 0, st>>>(g, p, b, sw, phi);
  else k_self_gravity<T, false><<<box_grid(b, g.nb, 128), 128, 0, st>>>(g, p, b, sw, phi);
}

template <typename T>
void Launcher<T>::c2p(const Geom& g, const StagePtrs<T>& p, bool mhd, const Phys& ph,
                      cudaStream_t st) {
  Box b = make_box(0, g.nc1 - 1, 0, g.nc2 - 1, 0, g.nc3 - 1);
  if (mhd) k_c2p<T, true><<<box_grid(b, g.nb, 256), 256, 0, st>>>(g, p, b, ph);
  else k_c2p<T, false><<<box_grid(b, g.nb, 256), 256, 0, st>>>(g, p, b, ph);
}

template <typename T>
void Launcher<T>::block_dt(const Geom& g, const StagePtrs<T>& p, bool mhd, const Phys& ph,
                           unsigned long long* dtmin, cudaStream_t st) {
  Box b = make_box(g.is, g.ie, g.js, g.je, g.ks, g.ke);
  if (mhd) k_block_dt<T, true><<<box_grid(b, g.nb, 256), 256, 0, st>>>(g, p, b, ph, dtmin);
  else k_block_dt<T, false><<<box_grid(b, g.nb, 256), 256, 0, st>>>(g, p, b, ph, dtmin);
}
#endif  // ATHG_LAUNCH_IMPL

extern template struct Launcher<double>;
extern template struct Launcher<float>;

}  // namespace athg

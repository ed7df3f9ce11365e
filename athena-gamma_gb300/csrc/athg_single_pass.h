// athg_single_pass.h -- host interface of the single-pass mixed VL2 MHD stage kernel
// (athg_single_pass.cu).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "athg_stage.cuh"

namespace athg {

// bits of the device error word (read back by the synchronising entry points)
constexpr unsigned int kErrTmaTimeout = 1u;  // a TMA load did not complete within its limit
constexpr unsigned int kErrTimeStep = 2u;    // the new time step is not a positive finite number
constexpr unsigned int kErrNonFinite = 4u;   // a non-finite density or pressure was produced

// the column of cells one thread block owns (i x j), marched along k
constexpr int SP_TILE_I = 32;
constexpr int SP_TILE_J = 8;

// TMA descriptors (CUtensorMap, 128 bytes each) of the FP32 W and bcc arrays a stage reads
struct SinglePassMaps {
  alignas(64) unsigned char w[128];
  alignas(64) unsigned char bcc[128];
};

// Whether the single-pass kernel covers this mesh: two ghost layers, block sizes that are
// multiples of the tile, nseg k-segments dividing nx3.
bool single_pass_fits(const Geom& g, int nseg);
size_t single_pass_smem();
// Raises the kernels' dynamic shared-memory limit to what they use (once, outside any
// stream capture); returns the CUDA error.
int single_pass_setup();
// Encodes the tensor maps of the W [nb][5][cells] and bcc [nb][3][cells] arrays.
int single_pass_maps(const float* w, const float* bcc, const Geom& g, SinglePassMaps* out,
                     std::string* err);
// One stage: reads W/bcc through `maps` (the arrays in p.w / p.bcc) and p.bf, the FP64 state
// from sb.u_in / sb.b_in; writes the new state to sb.u_out / sb.b_out and its W, bcc and
// FP32 face copies to w_out, bcc_out, bf_out (interior; ghosts are exchanged afterwards).
// order 1 (donor cell) or 2 (PLM); solver HLLD or HLLE; dtmin non-null on the last stage
// (CFL time step folded in); err: device error word (bit 0: a TMA load timed out).
// Returns the CUDA error of the launch.
int single_pass_launch(const SinglePassMaps& maps, const Geom& g, const StagePtrs<float>& p,
                       float* w_out, float* bcc_out, float* const bf_out[3], const StateBufs& sb,
                       const StageW& sw, const Phys& ph, unsigned long long* dtmin,
                       unsigned int* err, int order, int solver, int nseg, cudaStream_t st);

}  // namespace athg

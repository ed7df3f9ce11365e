// athg_internal.h -- what the hydro context needs from the multigrid solver when the two
// are coupled for self-gravity (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>

struct athg_mg;

namespace athg {

// Finest FP64 level of the solver: solution and source arrays of (n+2)^3 doubles with one
// ghost layer, index ((k*(n+2) + j)*(n+2) + i).
int mg_finest(athg_mg* m, double** u, double** src, int* n);

// Run the solver's work on `st` (nullptr: back to its own stream).
int mg_bind_stream(athg_mg* m, cudaStream_t st);

// Whether a solve issues no host synchronisation (fixed V-cycle count, no multipole
// boundary), so that it can be captured into a CUDA graph.
bool mg_solve_capturable(const athg_mg* m);

// MGGravityDriver::Solve after LoadSource: the solve of the configured mode, the final
// average subtraction and boundary fill. With want_norm false and a fixed V-cycle count
// it enqueues work only (no host synchronisation).
int mg_solve(athg_mg* m, bool want_norm, int* iterations, double* defect_norm);

}  // namespace athg

// ---- static mesh refinement (athg_smr.cu) ----------------------------------------------
#include <string>
#include <vector>

#include "athg_smr.h"

namespace athg {

// The work lists of a multi-level mesh on the device, with the coarse buffers and the
// per-block widths and cell centres they use
struct SmrDevice {
  SmrDims d;
  int nb = 0, nlevels = 1, ncmax = 0, nccmax = 0, mhd = 0;
  SmrXfer *xfer = nullptr, *pre = nullptr;
  int64_t nxfer = 0, npre = 0;
  SmrFlux* flux = nullptr;
  int64_t nflux = 0;
  SmrEmf* emf = nullptr;
  SmrEmfAdd* emf_add = nullptr;
  double* emf_tmp = nullptr;
  int64_t nemf = 0;
  SmrPos *c2p = nullptr, *pcc = nullptr, *pint = nullptr, *pfine = nullptr;
  SmrPos* psf[3] = {nullptr, nullptr, nullptr};
  int64_t nc2p = 0, npcc = 0, npint = 0, npfine = 0, npsf[3] = {0, 0, 0};
  double *cu = nullptr, *cw = nullptr, *cb1 = nullptr, *cb2 = nullptr, *cb3 = nullptr,
         *cbcc = nullptr;
  double *dx = nullptr, *xvf = nullptr, *xvc = nullptr;
};

// Plans the mesh (smr_plan) and copies lists, widths and cell centres to the device;
// coarse buffers start at zero. dx: [nb][3]; xvf: [nb][3][ncmax]; xvc: [nb][3][nccmax].
int smr_create(SmrDevice** out, const SmrDims& d, const int nrb[3],
               const std::vector<SmrLoc>& loc, const std::vector<double>& dx,
               const std::vector<double>& xvf, const std::vector<double>& xvc, bool mhd,
               cudaStream_t st, std::string* err);
void smr_destroy(SmrDevice* s);
// pool view with the device plan's own arrays filled in
SmrPool smr_pool(const SmrDevice* s);
// Ghost fill across levels, prolongation and U(W) of the prolongated cells
// (send/receive of U and B plus ProlongateBoundaries); returns the kernels launched
int smr_fill(const SmrDevice* s, const SmrPool& P, cudaStream_t st);
// Flux correction (coarse faces under finer neighbours); returns the kernels launched
int smr_correct_flux(const SmrDevice* s, const SmrPool& P, cudaStream_t st);
// EMF correction of every block-boundary edge; returns the kernels launched
int smr_correct_emf(const SmrDevice* s, const SmrPool& P, cudaStream_t st);
// Blast refinement criterion (max |grad p| / p per block) of FP64 primitives w into
// maxbits[nb] (bit patterns of non-negative doubles); returns the kernels launched
int amr_criterion(const SmrDims& d, int nb, const double* w, unsigned long long* maxbits,
                  cudaStream_t st);

}  // namespace athg

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

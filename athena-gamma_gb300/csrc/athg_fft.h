// athg_fft.h -- the FFT-based parts of the reference over the whole uniform periodic mesh,
// on cuFFT (not part of the C ABI; the hydro context in athg_api.cu owns both objects):
//
//   turbulence driving   TurbulenceDriver (fft/turbulence.cpp:42-542) with the FFT block of
//                        FFTDriver / FFTBlock (fft/fft_driver.cpp:30-172,
//                        fft/athena_fft.cpp:27-216) for one rank: one FFT over the mesh
//   FFT self-gravity     FFTGravityDriver::Solve + FFTGravity::ApplyKernel
//                        (gravity/fft_gravity.cpp:34-148)
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "athena_gb300.h"
#include "athg_device.cuh"

namespace athg {

// The whole mesh as the FFT sees it: cells per axis and domain lengths (x?max - x?min)
struct FftMesh {
  int n[3];
  double len[3];
};

struct FftGravity;
struct Turb;

// Plans (D2Z / Z2D) and work arrays; four_pi_G / (cells of the mesh) is the normalisation
// of the result (FFTGravityDriver ctor, SetNormFactor).
int fftgrav_create(const FftMesh& m, double four_pi_G, FftGravity** out, std::string* err);
void fftgrav_destroy(FftGravity* f);
// rho of every block (u, interior) -> phi of every block with one ghost layer (periodic
// wrap, as the gravity boundary exchange fills it). boff: each block's cell offset in the
// mesh (3 ints per block, device). phi2 (or nullptr): the same potential as FP32 pairs.
int fftgrav_solve(FftGravity* f, const Geom& g, int nb, const double* u, const int* boff,
                  double* phi, float2* phi2, cudaStream_t st, std::string* err);

// Driver state at Mesh construction: `time` is the mesh time then (tdrive starts there).
// Returns 0, 1 for an invalid configuration, -1 for a CUDA or cuFFT failure.
int turb_create(const FftMesh& m, const athg_turb_config& cfg, double time, Turb** out,
                std::string* err);
void turb_destroy(Turb* t);
int turb_flag(const Turb* t);
// TurbulenceDriver::Driving at mesh time `time` with time step `dt`: the perturbation of
// the momenta and energy of every block's interior (u, FP64), or nothing when an
// impulsive driver is not due. Host random numbers, device spectrum transform and sums.
int turb_drive(Turb* t, const Geom& g, int nb, double* u, const int* boff, double time,
               double dt, cudaStream_t st, std::string* err);

}  // namespace athg

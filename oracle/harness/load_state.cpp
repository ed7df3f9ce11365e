//! \file load_state.cpp
//! \brief Harness problem generator compiled INTO the reference solver (test
//!        infrastructure, never part of the product).
//!
//! It lets the unmodified reference run from an arbitrary seeded state and report
//! the state it reaches, so the CPU restatement and the CUDA path can be compared
//! with the reference on identical inputs.
//!
//! Input  (<problem> state_in):  raw little-endian float64, uniform single-level mesh,
//!   interior cells only, i fastest:
//!     U   [NHYDRO][NX3][NX2][NX1]
//!     B1f [NX3][NX2][NX1+1], B2f [NX3][NX2+1][NX1], B3f [NX3+1][NX2][NX1]   (MHD only)
//! Output (<problem> state_out): three float64 (time, dt, ncycle) followed by the
//!   same arrays at the end of the run, and, with self-gravity, phi [NX3][NX2][NX1].
//!
//! Hook names/signatures are the reference's (src/pgen/default_pgen.cpp:42-107).
//! Self-gravity runs take <problem> four_pi_G and use the reference's MG driver (or its
//! FFT driver when built with SELF_GRAVITY_ENABLED = 1). <problem> turb_flag (default 0)
//! turns on the reference's turbulence driver with the <turbulence> block, as its own
//! turb problem generator does (pgen/turb.cpp).

#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "athena.hpp"
#include "athena_arrays.hpp"
#include "coordinates/coordinates.hpp"
#include "field/field.hpp"
#include "gravity/gravity.hpp"
#include "hydro/hydro.hpp"
#include "mesh/mesh.hpp"
#include "parameter_input.hpp"

namespace {
std::string g_in, g_out;
int NX1, NX2, NX3;

inline std::size_t idx3(int k, int j, int i, int n2, int n1) {
  return (static_cast<std::size_t>(k)*n2 + j)*n1 + i;
}
}  // namespace

void Mesh::InitUserMeshData(ParameterInput *pin) {
  g_in = pin->GetString("problem", "state_in");
  g_out = pin->GetOrAddString("problem", "state_out", "state_out.bin");
  NX1 = mesh_size.nx1; NX2 = mesh_size.nx2; NX3 = mesh_size.nx3;
  if (SELF_GRAVITY_ENABLED) {
    SetFourPiG(pin->GetReal("problem", "four_pi_G"));
  }
  turb_flag = pin->GetOrAddInteger("problem", "turb_flag", 0);
}

void MeshBlock::ProblemGenerator(ParameterInput *pin) {
  const std::size_t ncell = static_cast<std::size_t>(NX1)*NX2*NX3;
  std::size_t total = NHYDRO*ncell;
  if (MAGNETIC_FIELDS_ENABLED)
    total += static_cast<std::size_t>(NX3)*NX2*(NX1+1) + static_cast<std::size_t>(NX3)*(NX2+1)*NX1
             + static_cast<std::size_t>(NX3+1)*NX2*NX1;
  std::vector<double> buf(total);
  FILE *f = std::fopen(g_in.c_str(), "rb");
  if (f == nullptr) throw std::runtime_error("load_state: cannot open state_in");
  if (std::fread(buf.data(), sizeof(double), total, f) != total) {
    std::fclose(f);
    throw std::runtime_error("load_state: short read");
  }
  std::fclose(f);
  const int oi = static_cast<int>(loc.lx1)*block_size.nx1;
  const int oj = static_cast<int>(loc.lx2)*block_size.nx2;
  const int ok = static_cast<int>(loc.lx3)*block_size.nx3;
  for (int n = 0; n < NHYDRO; ++n)
    for (int k = ks; k <= ke; ++k)
      for (int j = js; j <= je; ++j)
        for (int i = is; i <= ie; ++i)
          phydro->u(n, k, j, i) = buf[n*ncell + idx3(k-ks+ok, j-js+oj, i-is+oi, NX2, NX1)];
  if (MAGNETIC_FIELDS_ENABLED) {
    const double *b1 = buf.data() + NHYDRO*ncell;
    const double *b2 = b1 + static_cast<std::size_t>(NX3)*NX2*(NX1+1);
    const double *b3 = b2 + static_cast<std::size_t>(NX3)*(NX2+1)*NX1;
    for (int k = ks; k <= ke; ++k)
      for (int j = js; j <= je; ++j)
        for (int i = is; i <= ie+1; ++i)
          pfield->b.x1f(k, j, i) = b1[idx3(k-ks+ok, j-js+oj, i-is+oi, NX2, NX1+1)];
    for (int k = ks; k <= ke; ++k)
      for (int j = js; j <= je+1; ++j)
        for (int i = is; i <= ie; ++i)
          pfield->b.x2f(k, j, i) = b2[idx3(k-ks+ok, j-js+oj, i-is+oi, NX2+1, NX1)];
    for (int k = ks; k <= ke+1; ++k)
      for (int j = js; j <= je; ++j)
        for (int i = is; i <= ie; ++i)
          pfield->b.x3f(k, j, i) = b3[idx3(k-ks+ok, j-js+oj, i-is+oi, NX2, NX1)];
  }
}

void Mesh::UserWorkAfterLoop(ParameterInput *pin) {
  const std::size_t ncell = static_cast<std::size_t>(NX1)*NX2*NX3;
  std::vector<double> u(NHYDRO*ncell), b1, b2, b3, phi;
  if (MAGNETIC_FIELDS_ENABLED) {
    b1.resize(static_cast<std::size_t>(NX3)*NX2*(NX1+1));
    b2.resize(static_cast<std::size_t>(NX3)*(NX2+1)*NX1);
    b3.resize(static_cast<std::size_t>(NX3+1)*NX2*NX1);
  }
  if (SELF_GRAVITY_ENABLED) phi.resize(ncell);
  for (int b = 0; b < nblocal; ++b) {
    MeshBlock *pmb = my_blocks(b);
    const int is = pmb->is, ie = pmb->ie, js = pmb->js, je = pmb->je,
              ks = pmb->ks, ke = pmb->ke;
    const int oi = static_cast<int>(pmb->loc.lx1)*pmb->block_size.nx1;
    const int oj = static_cast<int>(pmb->loc.lx2)*pmb->block_size.nx2;
    const int ok = static_cast<int>(pmb->loc.lx3)*pmb->block_size.nx3;
    for (int n = 0; n < NHYDRO; ++n)
      for (int k = ks; k <= ke; ++k)
        for (int j = js; j <= je; ++j)
          for (int i = is; i <= ie; ++i)
            u[n*ncell + idx3(k-ks+ok, j-js+oj, i-is+oi, NX2, NX1)] = pmb->phydro->u(n, k, j, i);
    if (MAGNETIC_FIELDS_ENABLED) {
      for (int k = ks; k <= ke; ++k)
        for (int j = js; j <= je; ++j)
          for (int i = is; i <= ie+1; ++i)
            b1[idx3(k-ks+ok, j-js+oj, i-is+oi, NX2, NX1+1)] = pmb->pfield->b.x1f(k, j, i);
      for (int k = ks; k <= ke; ++k)
        for (int j = js; j <= je+1; ++j)
          for (int i = is; i <= ie; ++i)
            b2[idx3(k-ks+ok, j-js+oj, i-is+oi, NX2+1, NX1)] = pmb->pfield->b.x2f(k, j, i);
      for (int k = ks; k <= ke+1; ++k)
        for (int j = js; j <= je; ++j)
          for (int i = is; i <= ie; ++i)
            b3[idx3(k-ks+ok, j-js+oj, i-is+oi, NX2, NX1)] = pmb->pfield->b.x3f(k, j, i);
    }
    if (SELF_GRAVITY_ENABLED) {
      for (int k = ks; k <= ke; ++k)
        for (int j = js; j <= je; ++j)
          for (int i = is; i <= ie; ++i)
            phi[idx3(k-ks+ok, j-js+oj, i-is+oi, NX2, NX1)] = pmb->pgrav->phi(k, j, i);
    }
  }
  FILE *f = std::fopen(g_out.c_str(), "wb");
  if (f == nullptr) throw std::runtime_error("load_state: cannot open state_out");
  double hdr[3] = {time, dt, static_cast<double>(ncycle)};
  std::fwrite(hdr, sizeof(double), 3, f);
  std::fwrite(u.data(), sizeof(double), u.size(), f);
  if (MAGNETIC_FIELDS_ENABLED) {
    std::fwrite(b1.data(), sizeof(double), b1.size(), f);
    std::fwrite(b2.data(), sizeof(double), b2.size(), f);
    std::fwrite(b3.data(), sizeof(double), b3.size(), f);
  }
  if (SELF_GRAVITY_ENABLED) std::fwrite(phi.data(), sizeof(double), phi.size(), f);
  std::fclose(f);
}

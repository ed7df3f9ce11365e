//! \file shim_driver.cpp
//! \brief Harness problem generator compiled INTO the reference with gb300_shim.cpp (test
//!        infrastructure, never part of the product): the reference's own Orszag-Tang
//!        initial state is built by this file's ProblemGenerator as pgen/orszag_tang.cpp
//!        does (3-D, z-invariant, vector potential), then Mesh::UserWorkAfterLoop hands the
//!        mesh to the GB300 stage through the shim: setup, `<problem> gb300_cycles` VL2
//!        cycles of two stages each, download. Without a GPU the first call into the
//!        library fails and the shim raises the reference's ATHENA_ERROR, which the
//!        reference's main catches: the run ends cleanly with the library's message.

#include <cmath>
#include <exception>
#include <iostream>

#include "athena.hpp"
#include "athena_arrays.hpp"
#include "coordinates/coordinates.hpp"
#include "eos/eos.hpp"
#include "field/field.hpp"
#include "hydro/hydro.hpp"
#include "mesh/mesh.hpp"
#include "parameter_input.hpp"

void GB300Setup(Mesh* pm, ParameterInput* pin);
void GB300Stage(int stage);
void GB300EndCycle(Mesh* pm);
void GB300Download(Mesh* pm);
void GB300Finalize();

void MeshBlock::ProblemGenerator(ParameterInput* pin) {
  const Real gm1 = peos->GetGamma() - 1.0;
  const Real B0 = 1.0 / std::sqrt(4.0 * PI);
  const Real d0 = 25.0 / (36.0 * PI), p0 = 5.0 / (12.0 * PI);
  AthenaArray<Real> az;
  az.NewAthenaArray(ncells2, ncells1);
  for (int j = js; j <= je + 1; ++j)
    for (int i = is; i <= ie + 1; ++i)
      az(j, i) = B0 / (4.0 * PI) * (std::cos(4.0 * PI * pcoord->x1f(i)) -
                                    2.0 * std::cos(2.0 * PI * pcoord->x2f(j)));
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie; ++i) {
        phydro->u(IDN, k, j, i) = d0;
        phydro->u(IM1, k, j, i) = d0 * std::sin(2.0 * PI * pcoord->x2v(j));
        phydro->u(IM2, k, j, i) = -d0 * std::sin(2.0 * PI * pcoord->x1v(i));
        phydro->u(IM3, k, j, i) = 0.0;
      }
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie + 1; ++i)
        pfield->b.x1f(k, j, i) = (az(j + 1, i) - az(j, i)) / pcoord->dx2f(j);
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je + 1; ++j)
      for (int i = is; i <= ie; ++i)
        pfield->b.x2f(k, j, i) = (az(j, i) - az(j, i + 1)) / pcoord->dx1f(i);
  for (int k = ks; k <= ke + 1; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie; ++i) pfield->b.x3f(k, j, i) = 0.0;
  for (int k = ks; k <= ke; ++k)
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie; ++i) {
        const Real bx = 0.5 * (pfield->b.x1f(k, j, i) + pfield->b.x1f(k, j, i + 1));
        const Real by = 0.5 * (pfield->b.x2f(k, j, i) + pfield->b.x2f(k, j + 1, i));
        const Real m1 = phydro->u(IM1, k, j, i), m2 = phydro->u(IM2, k, j, i);
        phydro->u(IEN, k, j, i) = p0 / gm1 + 0.5 * (m1 * m1 + m2 * m2) / d0 +
                                  0.5 * (bx * bx + by * by);
      }
}

// (the reference's main catches errors of its main loop only; this hook runs after it,
// so the error of the shim is reported here)
void Mesh::UserWorkAfterLoop(ParameterInput* pin) {
  const int n = pin->GetOrAddInteger("problem", "gb300_cycles", 2);
  try {
    GB300Setup(this, pin);
    for (int c = 0; c < n; ++c) {
      GB300Stage(1);
      GB300Stage(2);
      GB300EndCycle(this);
    }
    GB300Download(this);
    std::cout << "gb300 shim: " << n << " cycles, time " << time << std::endl;
  } catch (std::exception& e) {
    std::cout << e.what();
  }
  GB300Finalize();
}

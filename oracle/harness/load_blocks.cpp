//! \file load_blocks.cpp
//! \brief Harness problem generator compiled INTO the reference solver (test
//!        infrastructure, never part of the product) for multi-level (SMR) meshes.
//!
//! Every MeshBlock takes its interior state from a file keyed by its logical location, so
//! the unmodified reference can run a refined mesh from an arbitrary seeded state and
//! report what it reaches, ghost zones included.
//!
//! Input  (<problem> state_in), little-endian:
//!   int64 nblocks; then per block: int64 level (relative to the root grid), lx1, lx2, lx3,
//!   float64 U[NHYDRO][nx3][nx2][nx1], and with MHD B1f[nx3][nx2][nx1+1],
//!   B2f[nx3][nx2+1][nx1], B3f[nx3+1][nx2][nx1] (interior cells and faces only).
//! Output (<problem> state_out): float64 time, dt, ncycle; int64 nblocks; then per block
//!   (in the mesh's own order) int64 level, lx1, lx2, lx3 followed by, when
//!   <problem> ghosts = true, the whole arrays including ghost zones:
//!   U[NHYDRO][nc3][nc2][nc1], W[NHYDRO][...], B1f[nc3][nc2][nc1+1], B2f[nc3][nc2+1][nc1],
//!   B3f[nc3+1][nc2][nc1]; otherwise the interior arrays in the input layout.
//!
//! Hook names/signatures are the reference's (src/pgen/default_pgen.cpp:42-107).

#include <cstdint>
#include <cstdio>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "athena.hpp"
#include "athena_arrays.hpp"
#include "field/field.hpp"
#include "hydro/hydro.hpp"
#include "mesh/mesh.hpp"
#include "parameter_input.hpp"

namespace {
std::string g_out;
bool g_ghosts = false;
int g_root_level = 0;
using Key = std::tuple<std::int64_t, std::int64_t, std::int64_t, std::int64_t>;
std::map<Key, std::vector<double>> g_blocks;

std::size_t interior_count(int n1, int n2, int n3) {
  std::size_t c = static_cast<std::size_t>(NHYDRO)*n1*n2*n3;
  if (MAGNETIC_FIELDS_ENABLED)
    c += static_cast<std::size_t>(n3)*n2*(n1+1) + static_cast<std::size_t>(n3)*(n2+1)*n1
         + static_cast<std::size_t>(n3+1)*n2*n1;
  return c;
}
}  // namespace

void Mesh::InitUserMeshData(ParameterInput *pin) {
  std::string in = pin->GetString("problem", "state_in");
  g_out = pin->GetOrAddString("problem", "state_out", "state_out.bin");
  g_ghosts = pin->GetOrAddBoolean("problem", "ghosts", false);
  g_root_level = root_level;
  int n1 = pin->GetInteger("meshblock", "nx1");
  int n2 = pin->GetInteger("meshblock", "nx2");
  int n3 = pin->GetInteger("meshblock", "nx3");
  const std::size_t per = interior_count(n1, n2, n3);
  FILE *f = std::fopen(in.c_str(), "rb");
  if (f == nullptr) throw std::runtime_error("load_blocks: cannot open state_in");
  std::int64_t nb = 0;
  if (std::fread(&nb, sizeof(nb), 1, f) != 1) throw std::runtime_error("load_blocks: header");
  for (std::int64_t b = 0; b < nb; ++b) {
    std::int64_t h[4];
    if (std::fread(h, sizeof(std::int64_t), 4, f) != 4)
      throw std::runtime_error("load_blocks: block header");
    std::vector<double> d(per);
    if (std::fread(d.data(), sizeof(double), per, f) != per)
      throw std::runtime_error("load_blocks: short block");
    g_blocks[Key(h[0], h[1], h[2], h[3])] = std::move(d);
  }
  std::fclose(f);
}

void MeshBlock::ProblemGenerator(ParameterInput *pin) {
  const int n1 = block_size.nx1, n2 = block_size.nx2, n3 = block_size.nx3;
  auto it = g_blocks.find(Key(loc.level - g_root_level, loc.lx1, loc.lx2, loc.lx3));
  if (it == g_blocks.end()) throw std::runtime_error("load_blocks: block not in state_in");
  const double *p = it->second.data();
  for (int n = 0; n < NHYDRO; ++n)
    for (int k = ks; k <= ke; ++k)
      for (int j = js; j <= je; ++j)
        for (int i = is; i <= ie; ++i) phydro->u(n, k, j, i) = *p++;
  if (MAGNETIC_FIELDS_ENABLED) {
    for (int k = ks; k <= ke; ++k)
      for (int j = js; j <= je; ++j)
        for (int i = is; i <= ie+1; ++i) pfield->b.x1f(k, j, i) = *p++;
    for (int k = ks; k <= ke; ++k)
      for (int j = js; j <= je+1; ++j)
        for (int i = is; i <= ie; ++i) pfield->b.x2f(k, j, i) = *p++;
    for (int k = ks; k <= ke+1; ++k)
      for (int j = js; j <= je; ++j)
        for (int i = is; i <= ie; ++i) pfield->b.x3f(k, j, i) = *p++;
  }
  (void)n1; (void)n2; (void)n3;
}

void Mesh::UserWorkAfterLoop(ParameterInput *pin) {
  FILE *f = std::fopen(g_out.c_str(), "wb");
  if (f == nullptr) throw std::runtime_error("load_blocks: cannot open state_out");
  double hdr[3] = {time, dt, static_cast<double>(ncycle)};
  std::fwrite(hdr, sizeof(double), 3, f);
  std::int64_t nb = nblocal;
  std::fwrite(&nb, sizeof(nb), 1, f);
  std::vector<double> out;
  for (int b = 0; b < nblocal; ++b) {
    MeshBlock *pmb = my_blocks(b);
    std::int64_t h[4] = {pmb->loc.level - root_level, pmb->loc.lx1, pmb->loc.lx2,
                         pmb->loc.lx3};
    std::fwrite(h, sizeof(std::int64_t), 4, f);
    out.clear();
    int il = pmb->is, iu = pmb->ie, jl = pmb->js, ju = pmb->je, kl = pmb->ks, ku = pmb->ke;
    if (g_ghosts) {
      il = 0; iu = pmb->ncells1 - 1; jl = 0; ju = pmb->ncells2 - 1;
      kl = 0; ku = pmb->ncells3 - 1;
    }
    for (int n = 0; n < NHYDRO; ++n)
      for (int k = kl; k <= ku; ++k)
        for (int j = jl; j <= ju; ++j)
          for (int i = il; i <= iu; ++i) out.push_back(pmb->phydro->u(n, k, j, i));
    if (g_ghosts) {
      for (int n = 0; n < NHYDRO; ++n)
        for (int k = kl; k <= ku; ++k)
          for (int j = jl; j <= ju; ++j)
            for (int i = il; i <= iu; ++i) out.push_back(pmb->phydro->w(n, k, j, i));
    }
    if (MAGNETIC_FIELDS_ENABLED) {
      for (int k = kl; k <= ku; ++k)
        for (int j = jl; j <= ju; ++j)
          for (int i = il; i <= iu+1; ++i) out.push_back(pmb->pfield->b.x1f(k, j, i));
      for (int k = kl; k <= ku; ++k)
        for (int j = jl; j <= ju+1; ++j)
          for (int i = il; i <= iu; ++i) out.push_back(pmb->pfield->b.x2f(k, j, i));
      for (int k = kl; k <= ku+1; ++k)
        for (int j = jl; j <= ju; ++j)
          for (int i = il; i <= iu; ++i) out.push_back(pmb->pfield->b.x3f(k, j, i));
    }
    std::fwrite(out.data(), sizeof(double), out.size(), f);
  }
  std::fclose(f);
}

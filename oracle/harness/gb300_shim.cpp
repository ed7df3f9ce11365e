//! \file gb300_shim.cpp
//! \brief The reference-side binding of the GB300 stage (the shim of INTEGRATION.md §2):
//!        C++ compiled into the reference and linked with -lathena_gb300. It uploads the
//!        MeshBlocks once after Mesh::Initialize, replaces each TaskList stage of the main
//!        loop (main.cpp:459-466) with one call over all blocks, and downloads the state
//!        before outputs. oracle/build_ref.py compiles it (config shim_mhd_hlld) together with
//!        shim_driver.cpp so that this file is checked against the reference's own headers.

#include <sstream>
#include <stdexcept>
#include <vector>

#include "athena.hpp"
#include "athena_gb300.h"
#include "bvals/bvals.hpp"
#include "coordinates/coordinates.hpp"
#include "eos/eos.hpp"
#include "field/field.hpp"
#include "hydro/hydro.hpp"
#include "mesh/mesh.hpp"
#include "parameter_input.hpp"

namespace {
athg_ctx* g_ctx = nullptr;

void Check(int rc) {
  if (rc != ATHG_OK) {
    std::stringstream msg;
    msg << "### FATAL ERROR in GB300 stage: " << athg_last_error() << std::endl;
    ATHENA_ERROR(msg);  // src/defs.hpp.in:119-123
  }
}
}  // namespace

// after Mesh::Initialize built the blocks and ran the problem generators
void GB300Setup(Mesh* pm, ParameterInput* pin) {
  MeshBlock* pmb = pm->my_blocks(0);
  athg_config c{};
  c.nx1 = pmb->block_size.nx1; c.nx2 = pmb->block_size.nx2; c.nx3 = pmb->block_size.nx3;
  c.nghost = NGHOST;
  c.magnetic = MAGNETIC_FIELDS_ENABLED;
  c.rsolver = MAGNETIC_FIELDS_ENABLED ? ATHG_HLLD : ATHG_HLLC;   // from RIEMANN_SOLVER
  c.xorder = pin->GetInteger("time", "xorder");
  c.integrator = ATHG_VL2;                                        // from <time> integrator
  c.precision = pin->GetOrAddBoolean("time", "gb300_mixed", true) ? ATHG_MIXED : ATHG_FP64;
  c.gamma = pmb->peos->GetGamma();
  c.dfloor = pmb->peos->GetDensityFloor();
  c.pfloor = pmb->peos->GetPressureFloor();
  c.cfl_number = pm->cfl_number;
  c.tlim = pm->tlim;
  Check(athg_create(&c, &g_ctx));
  std::vector<athg_block> bl(pm->nblocal);
  for (int b = 0; b < pm->nblocal; ++b) {
    MeshBlock* p = pm->my_blocks(b);
    athg_block& B = bl[b];
    B.lx1 = p->loc.lx1; B.lx2 = p->loc.lx2; B.lx3 = p->loc.lx3; B.level = p->loc.level;
    B.dx1 = p->pcoord->dx1f(p->is); B.dx2 = p->pcoord->dx2f(p->js);
    B.dx3 = p->pcoord->dx3f(p->ks);
    B.x1f = p->pcoord->x1f.data(); B.x2f = p->pcoord->x2f.data(); B.x3f = p->pcoord->x3f.data();
    for (int n = 0; n < 27; ++n) B.neighbor[n] = -1;
    for (int n = 0; n < p->pbval->nneighbor; ++n) {  // same-level neighbours
      const NeighborBlock& nb = p->pbval->neighbor[n];
      if (nb.snb.level != p->loc.level) continue;
      B.neighbor[(nb.ni.ox3 + 1) * 9 + (nb.ni.ox2 + 1) * 3 + (nb.ni.ox1 + 1)] = nb.snb.lid;
    }
  }
  Check(athg_set_blocks(g_ctx, pm->nblocal, bl.data()));
  for (int b = 0; b < pm->nblocal; ++b) {
    MeshBlock* p = pm->my_blocks(b);
    Check(athg_upload(g_ctx, b, ATHG_VAR_CONS, p->phydro->u.data(), p->phydro->u.GetSize()));
    if (MAGNETIC_FIELDS_ENABLED) {
      Check(athg_upload(g_ctx, b, ATHG_VAR_B1F, p->pfield->b.x1f.data(),
                        p->pfield->b.x1f.GetSize()));
      Check(athg_upload(g_ctx, b, ATHG_VAR_B2F, p->pfield->b.x2f.data(),
                        p->pfield->b.x2f.GetSize()));
      Check(athg_upload(g_ctx, b, ATHG_VAR_B3F, p->pfield->b.x3f.data(),
                        p->pfield->b.x3f.GetSize()));
    }
  }
  Check(athg_initialize(g_ctx));  // ghosts, W(U), first dt (as Mesh::Initialize)
}

// replaces `ptlist->DoTaskListOneStage(pmesh, stage)` in src/main.cpp:460
void GB300Stage(int stage) { Check(athg_stage(g_ctx, stage)); }

// replaces src/main.cpp:478-485 (time += dt; NewTimeStep)
void GB300EndCycle(Mesh* pm) {
  Check(athg_end_cycle(g_ctx));
  int64_t nc;
  Check(athg_get_time(g_ctx, &pm->time, &pm->dt, &nc));
}

// before Outputs::MakeOutputs / UserWorkAfterLoop: bring the state back
void GB300Download(Mesh* pm) {
  for (int b = 0; b < pm->nblocal; ++b) {
    MeshBlock* p = pm->my_blocks(b);
    Check(athg_download(g_ctx, b, ATHG_VAR_CONS, p->phydro->u.data(), p->phydro->u.GetSize()));
    Check(athg_download(g_ctx, b, ATHG_VAR_PRIM, p->phydro->w.data(), p->phydro->w.GetSize()));
    if (MAGNETIC_FIELDS_ENABLED) {
      Check(athg_download(g_ctx, b, ATHG_VAR_B1F, p->pfield->b.x1f.data(),
                          p->pfield->b.x1f.GetSize()));
      Check(athg_download(g_ctx, b, ATHG_VAR_B2F, p->pfield->b.x2f.data(),
                          p->pfield->b.x2f.GetSize()));
      Check(athg_download(g_ctx, b, ATHG_VAR_B3F, p->pfield->b.x3f.data(),
                          p->pfield->b.x3f.GetSize()));
      Check(athg_download(g_ctx, b, ATHG_VAR_BCC, p->pfield->bcc.data(),
                          p->pfield->bcc.GetSize()));
    }
  }
}

void GB300Finalize() {
  if (g_ctx) athg_destroy(g_ctx);
  g_ctx = nullptr;
}

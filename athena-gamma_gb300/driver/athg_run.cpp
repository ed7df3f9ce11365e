// athg_run.cpp -- a C++ host program above the C ABI, shaped like the reference's main
// loop (src/main.cpp:430-495): read an athinput file (plus block/key=value overrides from
// the command line, src/main.cpp:110-200 and inputs/parameter_input.cpp), build a uniform
// periodic mesh of MeshBlocks, set the initial state from a built-in problem generator,
// then cycle until tlim / nlim and write history sums (outputs/history.cpp) to
// <problem_id>.hst. The physics options the reference fixes when it is configured
// (magnetic fields, Riemann solver) are runtime keys of a <gb300> block here.
//
//   athg_run -i athinput.orszag_tang [mesh/nx1=128 time/nlim=10 ...]
//   athg_run -r OrszagTang.00001.rst [time/nlim=10 ...]     restart (also from the reference)
//
// Outputs (<outputN> blocks, outputs/outputs.cpp:786-803 timing): file_type = hst (history
// sums), vtk (variable = prim | cons, outputs/vtk.cpp) and rst (restart files readable by
// the reference, outputs/restart.cpp; a final <problem_id>.final.rst at the end).
//
// Problem generators: orszag_tang (src/pgen/orszag_tang.cpp:42-115) and blast
// (src/pgen/blast.cpp:54-120, uniform sphere of high pressure, optional uniform field).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <chrono>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "athena_gb300.h"
#include "athg_io.h"

namespace {

using Params = std::map<std::string, std::string>;  // "block/key" -> value

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

// athinput: "<block>" lines, "key = value # comment" lines (inputs/parameter_input.cpp);
// a restart file's parameter dump ends at "<par_end>"
void parse_athinput(std::istream& f, Params& p) {
  std::string line, block;
  while (std::getline(f, line)) {
    size_t h = line.find('#');
    if (h != std::string::npos) line = line.substr(0, h);
    line = trim(line);
    if (line.empty()) continue;
    if (line[0] == '<') {
      size_t e = line.find('>');
      block = trim(line.substr(1, e - 1));
      continue;
    }
    size_t eq = line.find('=');
    if (eq == std::string::npos) continue;
    p[block + "/" + trim(line.substr(0, eq))] = trim(line.substr(eq + 1));
  }
}

bool read_athinput(const std::string& path, Params& p) {
  std::ifstream f(path);
  if (!f) return false;
  parse_athinput(f, p);
  return true;
}

// ParameterInput::ParameterDump (parameter_input.cpp:834-859): blocks, "name = value"
// lines, closed by "<par_end>"
std::string dump_params(const Params& p) {
  std::ostringstream os;
  os << "#------------------------- PAR_DUMP -------------------------\n";
  std::string cur;
  for (const auto& kv : p) {
    const size_t sl = kv.first.find('/');
    const std::string block = kv.first.substr(0, sl), key = kv.first.substr(sl + 1);
    if (block == "par_end") continue;
    if (block != cur) {
      os << "<" << block << ">\n";
      cur = block;
    }
    os << key << " = " << kv.second << "\n";
  }
  os << "#------------------------- PAR_DUMP -------------------------\n";
  os << "<par_end>\n";
  return os.str();
}

std::string get(const Params& p, const std::string& k, const std::string& def) {
  auto it = p.find(k);
  return it == p.end() ? def : it->second;
}
double getd(const Params& p, const std::string& k, double def) {
  auto it = p.find(k);
  return it == p.end() ? def : std::atof(it->second.c_str());
}
int geti(const Params& p, const std::string& k, int def) {
  auto it = p.find(k);
  return it == p.end() ? def : std::atoi(it->second.c_str());
}

void check(int rc, const char* what) {
  if (rc != ATHG_OK) {
    std::fprintf(stderr, "### FATAL ERROR in %s: %s\n", what, athg_last_error());
    std::exit(1);
  }
}

// cell-centre / face positions of one axis of one block
struct Axis {
  std::vector<double> xf, xv;
  double dx;
};
// The uniform mesh generator (mesh/mesh.hpp:389-470): position of face `index` of `nrange`
double gen_x(int64_t index, int64_t nrange, double lo, double hi) {
  const int64_t noffset = index - nrange / 2, noffset_ceil = index - (nrange + 1) / 2;
  const double rx = static_cast<double>(noffset + noffset_ceil) / (2.0 * nrange);
  return 0.5 * (lo + hi) + (rx * hi - rx * lo);
}
// Faces of block lx at `level` (root-relative), ghosts included, with the block edges of
// Mesh::SetBlockSizeAndBoundaries (mesh/mesh.cpp:1675-1690) and the face loop of
// Coordinates::Coordinates (coordinates/coordinates.cpp:127-145, cartesian.cpp:29)
Axis axis_of(int nx, int ng, double lo, double hi, int mesh_nx, int level, int64_t lx) {
  Axis a;
  const int64_t nroot = (int64_t)mesh_nx << level, nrbl = (int64_t)(mesh_nx / nx) << level;
  const double bmin = (lx == 0) ? lo : gen_x(lx, nrbl, lo, hi);
  const double bmax = (lx == nrbl - 1) ? hi : gen_x(lx + 1, nrbl, lo, hi);
  a.dx = (bmax - bmin) / nx;
  a.xf.resize(nx + 2 * ng + 1);
  for (int i = 0; i < nx + 2 * ng + 1; ++i) a.xf[i] = gen_x((i - ng) + lx * nx, nroot, lo, hi);
  a.xf[ng] = bmin;
  a.xf[ng + nx] = bmax;
  a.xv.resize(nx + 2 * ng);
  for (int i = 0; i < nx + 2 * ng; ++i) a.xv[i] = 0.5 * (a.xf[i + 1] + a.xf[i]);
  return a;
}

}  // namespace

int main(int argc, char** argv) {
  Params p;
  std::string input, restart;
  for (int a = 1; a < argc; ++a) {
    if (!std::strcmp(argv[a], "-i") && a + 1 < argc) {
      input = argv[++a];
    } else if (!std::strcmp(argv[a], "-r") && a + 1 < argc) {
      restart = argv[++a];
    } else if (std::strchr(argv[a], '=')) {
      std::string s = argv[a];
      size_t eq = s.find('=');
      p["__cli__" + s.substr(0, eq)] = s.substr(eq + 1);
    }
  }
  if (!restart.empty()) {
    std::string text, err;
    if (!athg_io::read_restart_params(restart, &text, &err)) {
      std::fprintf(stderr, "### FATAL ERROR reading %s: %s\n", restart.c_str(), err.c_str());
      return 1;
    }
    std::istringstream is(text);
    parse_athinput(is, p);
  } else if (input.empty() || !read_athinput(input, p)) {
    std::fprintf(stderr, "usage: athg_run -i athinput | -r file.rst [block/key=value ...]\n");
    return 1;
  }
  for (auto it = p.begin(); it != p.end();) {  // command-line overrides win
    if (it->first.rfind("__cli__", 0) == 0) {
      p[it->first.substr(7)] = it->second;
      it = p.erase(it);
    } else {
      ++it;
    }
  }

  const std::string pgen = get(p, "gb300/pgen", "orszag_tang");
  const bool mhd = geti(p, "gb300/magnetic", 1) != 0;
  const std::string rs = get(p, "gb300/rsolver", mhd ? "hlld" : "hllc");
  const std::string integ = get(p, "time/integrator", "vl2");
  athg_config c{};
  athg_mesh m{};
  m.nx1 = geti(p, "mesh/nx1", 64); m.nx2 = geti(p, "mesh/nx2", m.nx1); m.nx3 = geti(p, "mesh/nx3", m.nx1);
  m.x1min = getd(p, "mesh/x1min", -0.5); m.x1max = getd(p, "mesh/x1max", 0.5);
  m.x2min = getd(p, "mesh/x2min", -0.5); m.x2max = getd(p, "mesh/x2max", 0.5);
  m.x3min = getd(p, "mesh/x3min", -0.5); m.x3max = getd(p, "mesh/x3max", 0.5);
  m.periodic[0] = m.periodic[1] = m.periodic[2] = 1;
  for (const char* bc : {"ix1_bc", "ox1_bc", "ix2_bc", "ox2_bc", "ix3_bc", "ox3_bc"})
    if (get(p, std::string("mesh/") + bc, "periodic") != "periodic") {
      std::fprintf(stderr, "### FATAL ERROR: only periodic mesh boundaries are supported\n");
      return 1;
    }
  c.nx1 = geti(p, "meshblock/nx1", m.nx1);
  c.nx2 = geti(p, "meshblock/nx2", m.nx2);
  c.nx3 = geti(p, "meshblock/nx3", m.nx3);
  c.xorder = geti(p, "time/xorder", 2);
  c.nghost = geti(p, "gb300/nghost", c.xorder == 3 ? 3 : 2);
  c.magnetic = mhd;
  c.rsolver = rs == "hlle" ? ATHG_HLLE : rs == "hllc" ? ATHG_HLLC : rs == "hlld" ? ATHG_HLLD
            : rs == "lhllc" ? ATHG_LHLLC : ATHG_LHLLD;
  c.integrator = integ == "rk1" ? ATHG_RK1 : integ == "rk2" ? ATHG_RK2 : integ == "rk3" ? ATHG_RK3
               : ATHG_VL2;
  c.precision = get(p, "gb300/precision", "mixed") == "fp64" ? ATHG_FP64 : ATHG_MIXED;
  c.gamma = getd(p, "hydro/gamma", 5.0 / 3.0);
  const double fl = std::sqrt(1024.0 * 1.17549435e-38);  // eos/eos.cpp default floors
  c.dfloor = getd(p, "hydro/dfloor", fl);
  c.pfloor = getd(p, "hydro/pfloor", fl);
  c.cfl_number = getd(p, "time/cfl_number", 0.3);
  c.tlim = getd(p, "time/tlim", 1.0);
  const int nlim = geti(p, "time/nlim", -1);

  athg_ctx* ctx = nullptr;
  check(athg_create(&c, &ctx), "athg_create");
  // the mesh as the restart/VTK writers describe it
  athg_io::State st;
  st.mesh_nx[0] = m.nx1; st.mesh_nx[1] = m.nx2; st.mesh_nx[2] = m.nx3;
  st.xmin[0] = m.x1min; st.xmin[1] = m.x2min; st.xmin[2] = m.x3min;
  st.xmax[0] = m.x1max; st.xmax[1] = m.x2max; st.xmax[2] = m.x3max;
  st.block_nx[0] = c.nx1; st.block_nx[1] = c.nx2; st.block_nx[2] = c.nx3;
  st.ng = c.nghost;
  st.mhd = mhd;
  // <mesh> refinement = adaptive: the blast's criterion (<problem> thr), numlevel,
  // derefine_count (mesh/mesh_refinement.cpp:39-120, pgen/blast.cpp:38-44)
  const bool adaptive = get(p, "mesh/refinement", "none") == "adaptive";
  athg_amr_config amr_cfg{};
  amr_cfg.threshold = getd(p, "problem/thr", 0.0);
  amr_cfg.deref_fraction = 0.25;
  amr_cfg.max_level = geti(p, "mesh/numlevel", 1) - 1;
  amr_cfg.derefine_count = geti(p, "mesh/derefine_count", 10);
  // <problem> turb_flag with the <turbulence> block (fft/turbulence.cpp:42-63) and FFT
  // self-gravity (<gb300> gravity = fft, <problem> four_pi_G; pgen/turb.cpp:36-43)
  const int turb_flag = geti(p, "problem/turb_flag", 0);
  auto attach_fft_parts = [&]() {
    if (turb_flag != 0) {
      athg_turb_config tc{};
      tc.turb_flag = turb_flag;
      tc.rseed = geti(p, "turbulence/rseed", -1);
      tc.nlow = geti(p, "turbulence/nlow", 0);
      tc.nhigh = geti(p, "turbulence/nhigh", m.nx1 / 2);
      tc.dtdrive = getd(p, "turbulence/dtdrive", 0.0);
      tc.tcorr = getd(p, "turbulence/tcorr", 0.0);
      tc.f_shear = getd(p, "turbulence/f_shear", -1.0);
      tc.expo = getd(p, "turbulence/expo", 2.0);
      tc.dedt = getd(p, "turbulence/dedt", 0.0);
      check(athg_turb_attach(ctx, &m, &tc), "athg_turb_attach");
    }
    if (get(p, "gb300/gravity", "none") == "fft")
      check(athg_attach_fft_gravity(ctx, &m, getd(p, "problem/four_pi_G", 0.0)),
            "athg_attach_fft_gravity");
  };
  if (!restart.empty()) {
    // Mesh::Mesh(pin, restartfile) + Mesh::Initialize(res_flag = 1)
    std::string text, err;
    if (!athg_io::read_restart(restart, &text, &st, &err)) {
      std::fprintf(stderr, "### FATAL ERROR reading %s: %s\n", restart.c_str(), err.c_str());
      return 1;
    }
    const int nf = (int)st.blocks.size();
    bool multi = false;
    std::vector<int64_t> locs(4 * nf);
    for (int q = 0; q < nf; ++q) {
      multi = multi || st.blocks[q].level != 0;
      locs[4 * q] = st.blocks[q].level;
      for (int d = 0; d < 3; ++d) locs[4 * q + 1 + d] = st.blocks[q].lx[d];
    }
    if (multi) check(athg_set_multilevel_blocks(ctx, &m, nf, locs.data()), "athg_set_multilevel_blocks");
    else check(athg_set_uniform_mesh(ctx, &m), "athg_set_uniform_mesh");
    if (adaptive) check(athg_amr_enable(ctx, &amr_cfg), "athg_amr_enable");
    int nlib = 0;
    check(athg_num_blocks(ctx, &nlib), "athg_num_blocks");
    if (nlib != nf) {
      std::fprintf(stderr, "### FATAL ERROR: restart file has %d blocks, the mesh %d\n", nf, nlib);
      return 1;
    }
    std::map<std::vector<int64_t>, int> lib_of;
    for (int b = 0; b < nlib; ++b) {
      int64_t loc[4];
      check(athg_block_location(ctx, b, loc), "athg_block_location");
      lib_of[{loc[3], loc[0], loc[1], loc[2]}] = b;
    }
    const size_t nu = 5 * st.cell_count();
    const size_t nfc[3] = {st.face_count(0), st.face_count(1), st.face_count(2)};
    for (int q = 0; q < nf; ++q) {
      auto it = lib_of.find({st.blocks[q].level, st.blocks[q].lx[0], st.blocks[q].lx[1], st.blocks[q].lx[2]});
      if (it == lib_of.end()) {
        std::fprintf(stderr, "### FATAL ERROR: restart block not in the mesh\n");
        return 1;
      }
      const int b = it->second;
      check(athg_upload(ctx, b, ATHG_VAR_CONS, &st.u[q * nu], nu), "upload U");
      if (mhd) {
        check(athg_upload(ctx, b, ATHG_VAR_B1F, &st.b1[q * nfc[0]], nfc[0]), "upload B1");
        check(athg_upload(ctx, b, ATHG_VAR_B2F, &st.b2[q * nfc[1]], nfc[1]), "upload B2");
        check(athg_upload(ctx, b, ATHG_VAR_B3F, &st.b3[q * nfc[2]], nfc[2]), "upload B3");
      }
    }
    check(athg_set_time(ctx, st.time, st.dt, st.ncycle), "athg_set_time");
    attach_fft_parts();  // the driver starts at the restart time (tdrive = time)
    check(athg_resume(ctx), "athg_resume");
  } else {
    // <refinementN> blocks (static refinement, mesh/mesh.cpp:334-462)
    std::vector<athg_region> regions;
    for (int id = 1; id < 100; ++id) {
      const std::string blk = "refinement" + std::to_string(id) + "/";
      if (!p.count(blk + "level")) continue;
      athg_region r{};
      r.x1min = getd(p, blk + "x1min", m.x1min); r.x1max = getd(p, blk + "x1max", m.x1max);
      r.x2min = getd(p, blk + "x2min", m.x2min); r.x2max = getd(p, blk + "x2max", m.x2max);
      r.x3min = getd(p, blk + "x3min", m.x3min); r.x3max = getd(p, blk + "x3max", m.x3max);
      r.level = geti(p, blk + "level", 1);
      regions.push_back(r);
    }
    if (!regions.empty())
      check(athg_set_refined_mesh(ctx, &m, (int)regions.size(), regions.data()),
            "athg_set_refined_mesh");
    else
      check(athg_set_uniform_mesh(ctx, &m), "athg_set_uniform_mesh");
    if (adaptive) check(athg_amr_enable(ctx, &amr_cfg), "athg_amr_enable");
    attach_fft_parts();
    // MeshBlock::ProblemGenerator for every block, then one upload per array
    auto generate = [&]() -> int {
      int nb = 0;
      check(athg_num_blocks(ctx, &nb), "athg_num_blocks");
      const int ng = c.nghost;
      const int n1 = c.nx1 + 2 * ng, n2 = c.nx2 + 2 * ng, n3 = c.nx3 + 2 * ng;
      const size_t nc = (size_t)n1 * n2 * n3;
      std::vector<double> U(5 * nc * nb, 0.0), B1, B2, B3;
      if (mhd) {
        B1.assign((size_t)n3 * n2 * (n1 + 1) * nb, 0.0);
        B2.assign((size_t)n3 * (n2 + 1) * n1 * nb, 0.0);
        B3.assign((size_t)(n3 + 1) * n2 * n1 * nb, 0.0);
      }
      const double gm1 = c.gamma - 1.0;
      for (int b = 0; b < nb; ++b) {
        int64_t loc[4];
        check(athg_block_location(ctx, b, loc), "athg_block_location");
        // cells of the block's level (loc[3]) across the whole domain
        const int64_t lv = loc[3];
        Axis ax = axis_of(c.nx1, ng, m.x1min, m.x1max, m.nx1, (int)lv, loc[0]);
        Axis ay = axis_of(c.nx2, ng, m.x2min, m.x2max, m.nx2, (int)lv, loc[1]);
        Axis az = axis_of(c.nx3, ng, m.x3min, m.x3max, m.nx3, (int)lv, loc[2]);
        double* u = &U[5 * nc * b];
        auto C = [&](int n, int k, int j, int i) -> double& {
          return u[(size_t)n * nc + ((size_t)k * n2 + j) * n1 + i];
        };
        double* b1 = mhd ? &B1[(size_t)n3 * n2 * (n1 + 1) * b] : nullptr;
        double* b2 = mhd ? &B2[(size_t)n3 * (n2 + 1) * n1 * b] : nullptr;
        double* b3 = mhd ? &B3[(size_t)(n3 + 1) * n2 * n1 * b] : nullptr;
        auto F1 = [&](int k, int j, int i) -> double& { return b1[((size_t)k * n2 + j) * (n1 + 1) + i]; };
        auto F2 = [&](int k, int j, int i) -> double& { return b2[((size_t)k * (n2 + 1) + j) * n1 + i]; };
        (void)b3;
        const int is = ng, ie = ng + c.nx1 - 1, js = ng, je = ng + c.nx2 - 1, ks = ng, ke = ng + c.nx3 - 1;
        if (pgen == "orszag_tang") {
          const double PI = 3.1415926535897932, TWO_PI = 6.2831853071795862;
          const double B0 = 1.0 / std::sqrt(4.0 * PI), d0 = 25.0 / (36.0 * PI), v0 = 1.0,
                       p0 = 5.0 / (12.0 * PI);
          auto Az = [&](double x, double y) {
            return B0 / (4.0 * PI) * (std::cos(4.0 * PI * x) - 2.0 * std::cos(TWO_PI * y));
          };
          for (int k = ks; k <= ke; ++k)
            for (int j = js; j <= je; ++j)
              for (int i = is; i <= ie; ++i) {
                C(0, k, j, i) = d0;
                C(1, k, j, i) = d0 * v0 * std::sin(TWO_PI * ay.xv[j]);
                C(2, k, j, i) = -d0 * v0 * std::sin(TWO_PI * ax.xv[i]);
                C(3, k, j, i) = 0.0;
              }
          if (mhd) {
            for (int k = ks; k <= ke; ++k)
              for (int j = js; j <= je; ++j)
                for (int i = is; i <= ie + 1; ++i)
                  F1(k, j, i) = (Az(ax.xf[i], ay.xf[j + 1]) - Az(ax.xf[i], ay.xf[j])) / ay.dx;
            for (int k = ks; k <= ke; ++k)
              for (int j = js; j <= je + 1; ++j)
                for (int i = is; i <= ie; ++i)
                  F2(k, j, i) = (Az(ax.xf[i], ay.xf[j]) - Az(ax.xf[i + 1], ay.xf[j])) / ax.dx;
          }
          for (int k = ks; k <= ke; ++k)
            for (int j = js; j <= je; ++j)
              for (int i = is; i <= ie; ++i) {
                double pb = 0.0;
                if (mhd) {
                  double c1 = 0.5 * (F1(k, j, i) + F1(k, j, i + 1));
                  double c2 = 0.5 * (F2(k, j, i) + F2(k, j + 1, i));
                  pb = 0.5 * (c1 * c1 + c2 * c2);
                }
                const double d = C(0, k, j, i);
                C(4, k, j, i) = p0 / gm1 + pb +
                                0.5 * (C(1, k, j, i) * C(1, k, j, i) + C(2, k, j, i) * C(2, k, j, i)) / d;
              }
        } else if (pgen == "blast") {  // pgen/blast.cpp:54-211, Cartesian
          const double PI = 3.1415926535897932;
          const double rout = getd(p, "problem/radius", 0.1);
          const double rin = rout - getd(p, "problem/ramp", 0.0);
          const double pa = getd(p, "problem/pamb", 1.0), da = getd(p, "problem/damb", 1.0);
          const double prat = getd(p, "problem/prat", 100.0), drat = getd(p, "problem/drat", 1.0);
          const double b0 = mhd ? getd(p, "problem/b0", 1.0) : 0.0;
          const double angle = (PI / 180.0) * getd(p, "problem/angle", 45.0);
          const double x0 = getd(p, "problem/x1_0", 0.0), y0 = getd(p, "problem/x2_0", 0.0),
                       z0 = getd(p, "problem/x3_0", 0.0);
          for (int k = ks; k <= ke; ++k)
            for (int j = js; j <= je; ++j)
              for (int i = is; i <= ie; ++i) {
                const double x = ax.xv[i] - x0, y = ay.xv[j] - y0, z = az.xv[k] - z0;
                const double rad = std::sqrt(x * x + y * y + z * z);
                double den = da, pres = pa;
                if (rad < rout) {
                  if (rad < rin) {
                    den = drat * da;
                    pres = prat * pa;
                  } else {  // smooth ramp between rin and rout
                    const double f = (rad - rin) / (rout - rin);
                    den = std::exp((1.0 - f) * std::log(drat * da) + f * std::log(da));
                    pres = std::exp((1.0 - f) * std::log(prat * pa) + f * std::log(pa));
                  }
                }
                C(0, k, j, i) = den;
                C(1, k, j, i) = C(2, k, j, i) = C(3, k, j, i) = 0.0;
                C(4, k, j, i) = pres / gm1;
              }
          if (mhd) {
            const double bx = b0 * std::cos(angle), by = b0 * std::sin(angle);
            for (int k = ks; k <= ke; ++k) {
              for (int j = js; j <= je; ++j)
                for (int i = is; i <= ie + 1; ++i) F1(k, j, i) = bx;
              for (int j = js; j <= je + 1; ++j)
                for (int i = is; i <= ie; ++i) F2(k, j, i) = by;
            }
            for (int k = ks; k <= ke; ++k)
              for (int j = js; j <= je; ++j)
                for (int i = is; i <= ie; ++i) C(4, k, j, i) += 0.5 * b0 * b0;
          }
        } else if (pgen == "turb") {  // pgen/turb.cpp:58-78: uniform gas at rest
          for (int k = ks; k <= ke; ++k)
            for (int j = js; j <= je; ++j)
              for (int i = is; i <= ie; ++i) {
                C(0, k, j, i) = 1.0;
                C(1, k, j, i) = C(2, k, j, i) = C(3, k, j, i) = 0.0;
                C(4, k, j, i) = 1.0;
              }
        } else {
          std::fprintf(stderr, "### FATAL ERROR: unknown gb300/pgen %s\n", pgen.c_str());
          return 1;
        }
      }
      check(athg_upload(ctx, -1, ATHG_VAR_CONS, U.data(), U.size()), "upload U");
      if (mhd) {
        check(athg_upload(ctx, -1, ATHG_VAR_B1F, B1.data(), B1.size()), "upload B1");
        check(athg_upload(ctx, -1, ATHG_VAR_B2F, B2.data(), B2.size()), "upload B2");
        check(athg_upload(ctx, -1, ATHG_VAR_B3F, B3.data(), B3.size()), "upload B3");
      }

      return 0;
    };
    // Mesh::Initialize(0) (mesh/mesh.cpp:1367-1656): with adaptive refinement the problem
    // generator runs again on every refined mesh until the criterion leaves it unchanged
    if (generate()) return 1;
    check(athg_initialize(ctx), "athg_initialize");
    if (adaptive) {
      for (int pass = 0;; ++pass) {
        double tt, dd, dd_prev = 1.79769313486231570815e308;
        int64_t nn;
        if (pass > 0) {
          check(athg_get_time(ctx, &tt, &dd_prev, &nn), "athg_get_time");
          if (generate()) return 1;
          check(athg_resume(ctx), "athg_resume");
        }
        check(athg_get_time(ctx, &tt, &dd, &nn), "athg_get_time");
        // the check runs before the pass's NewTimeStep in the reference
        check(athg_set_time(ctx, tt, dd_prev, nn), "athg_set_time");
        int changed = 0;
        check(athg_amr_regrid(ctx, &changed), "athg_amr_regrid");
        if (!changed) {
          check(athg_set_time(ctx, tt, dd, nn), "athg_set_time");
          break;
        }
      }
    }

  }

  // outputs: <outputN> file_type = hst | vtk | rst (Outputs::MakeOutputs timing)
  const std::string base = get(p, "job/problem_id", pgen);
  struct Out {
    int id;
    std::string type, var;
    double dt, next;
    int number, dcycle;
  };
  double t = 0.0, dt = 0.0;
  int64_t ncycle = 0;
  check(athg_get_time(ctx, &t, &dt, &ncycle), "athg_get_time");
  const double start_time = t;
  std::vector<Out> outs;
  for (int id = 1; id < 100; ++id) {
    const std::string blk = "output" + std::to_string(id) + "/";
    if (!p.count(blk + "file_type")) continue;
    Out o;
    o.id = id;
    o.type = get(p, blk + "file_type", "hst");
    o.var = get(p, blk + "variable", "prim");
    o.dt = getd(p, blk + "dt", -1.0);
    o.dcycle = geti(p, blk + "dcycle", 0);
    o.next = getd(p, blk + "next_time", start_time);
    o.number = geti(p, blk + "file_number", 0);
    outs.push_back(o);
  }
  std::FILE* hst = nullptr;
  bool hst_header = false;
  int nb_all = 0;
  // every block's location and arrays, in the library's order (adaptive refinement
  // changes the list from cycle to cycle)
  auto download_state = [&](bool prim) {
    check(athg_num_blocks(ctx, &nb_all), "athg_num_blocks");
    st.blocks.resize(nb_all);
    for (int b = 0; b < nb_all; ++b) {
      int64_t loc[4];
      check(athg_block_location(ctx, b, loc), "athg_block_location");
      st.blocks[b].level = (int)loc[3];
      for (int d = 0; d < 3; ++d) st.blocks[b].lx[d] = loc[d];
    }
    st.u.resize(5 * st.cell_count() * nb_all);
    check(athg_download(ctx, -1, ATHG_VAR_CONS, st.u.data(), st.u.size()), "download U");
    if (mhd) {
      st.b1.resize(st.face_count(0) * nb_all);
      st.b2.resize(st.face_count(1) * nb_all);
      st.b3.resize(st.face_count(2) * nb_all);
      check(athg_download(ctx, -1, ATHG_VAR_B1F, st.b1.data(), st.b1.size()), "download B1");
      check(athg_download(ctx, -1, ATHG_VAR_B2F, st.b2.data(), st.b2.size()), "download B2");
      check(athg_download(ctx, -1, ATHG_VAR_B3F, st.b3.data(), st.b3.size()), "download B3");
    }
    double tt, dd;
    int64_t nn;
    check(athg_get_time(ctx, &tt, &dd, &nn), "athg_get_time");
    st.time = tt; st.dt = dd; st.ncycle = (int)nn;
    std::vector<double> w, bcc;
    if (prim) {
      w.resize(5 * st.cell_count() * nb_all);
      check(athg_download(ctx, -1, ATHG_VAR_PRIM, w.data(), w.size()), "download W");
      if (mhd) {
        bcc.resize(3 * st.cell_count() * nb_all);
        check(athg_download(ctx, -1, ATHG_VAR_BCC, bcc.data(), bcc.size()), "download Bcc");
      }
    }
    return std::make_pair(w, bcc);
  };
  auto write_output = [&](Out& o, bool final) {
    const std::string blk = "output" + std::to_string(o.id) + "/";
    std::string err;
    if (o.type == "hst") {  // HistoryOutput::WriteOutputFile (outputs/history.cpp)
      if (!hst) hst = std::fopen((base + ".hst").c_str(), restart.empty() ? "w" : "a");
      if (!hst_header && restart.empty()) {
        std::fprintf(hst, "# Athena++ history data (athg_run)\n"
                          "# [1]=time [2]=dt [3]=mass [4]=1-mom [5]=2-mom [6]=3-mom [7]=1-KE "
                          "[8]=2-KE [9]=3-KE [10]=tot-E [11]=grav-E [12]=1-ME [13]=2-ME [14]=3-ME\n");
      }
      hst_header = true;
      double h[12], tt, dd;
      int n;
      int64_t nn;
      check(athg_history(ctx, h, &n), "athg_history");
      check(athg_get_time(ctx, &tt, &dd, &nn), "athg_get_time");
      std::fprintf(hst, "%.14e %.14e", tt, dd);
      for (int q = 0; q < n; ++q) std::fprintf(hst, " %.14e", h[q]);
      std::fprintf(hst, "\n");
      std::fflush(hst);
      o.next += o.dt;
    } else if (o.type == "vtk") {  // VTKOutput::WriteOutputFile
      auto wb = download_state(true);
      if (!athg_io::write_vtk(base, "out" + std::to_string(o.id), o.number, o.var, st, wb.first,
                              wb.second, &err)) {
        std::fprintf(stderr, "### FATAL ERROR in vtk output: %s\n", err.c_str());
        std::exit(1);
      }
      o.number++;
      o.next += o.dt;
    } else if (o.type == "rst") {  // RestartOutput::WriteOutputFile
      char num[16];
      std::snprintf(num, sizeof(num), "%05d", o.number);
      const std::string fname = base + "." + (final ? std::string("final") : std::string(num)) + ".rst";
      if (!final) {
        o.number++;
        o.next += o.dt;
      }
      p[blk + "file_number"] = std::to_string(o.number);
      char nt[64];
      std::snprintf(nt, sizeof(nt), "%.17g", o.next);
      p[blk + "next_time"] = nt;
      download_state(false);
      if (!athg_io::write_restart(fname, dump_params(p), st, &err)) {
        std::fprintf(stderr, "### FATAL ERROR in restart output: %s\n", err.c_str());
        std::exit(1);
      }
      return;
    }
    p[blk + "file_number"] = std::to_string(o.number);
    char nt[64];
    std::snprintf(nt, sizeof(nt), "%.17g", o.next);
    p[blk + "next_time"] = nt;
  };
  auto make_outputs = [&](bool final) {
    double tt, dd;
    int64_t nn;
    check(athg_get_time(ctx, &tt, &dd, &nn), "athg_get_time");
    for (Out& o : outs)
      if (tt == start_time || (o.dt > 0.0 && tt >= o.next) ||
          (o.dcycle > 0 && nn % o.dcycle == 0) || tt >= c.tlim || (final && o.type == "rst"))
        write_output(o, final);
  };
  if (restart.empty()) make_outputs(false);  // main.cpp:397
  const auto t0 = std::chrono::steady_clock::now();
  int64_t cycles = 0;
  double zone_cycles = 0.0;
  while (t < c.tlim && (nlim < 0 || ncycle < nlim)) {
    check(athg_num_blocks(ctx, &nb_all), "athg_num_blocks");
    zone_cycles += (double)nb_all * c.nx1 * c.nx2 * c.nx3;
    check(athg_cycles(ctx, 1), "athg_cycles");
    ++cycles;
    check(athg_get_time(ctx, &t, &dt, &ncycle), "athg_get_time");
    if (t < c.tlim) make_outputs(false);  // the final output happens after the loop
  }
  check(athg_synchronize(ctx), "athg_synchronize");
  const double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  make_outputs(true);
  if (hst) std::fclose(hst);
  check(athg_num_blocks(ctx, &nb_all), "athg_num_blocks");
  // main.cpp:580-600 summary
  std::printf("cycle=%lld time=%.10e dt=%.10e\n", (long long)ncycle, t, dt);
  std::printf("Number of MeshBlocks = %d\n", nb_all);
  std::printf("zone-cycles = %.0f\nwall time = %.6f s\nzone-cycles/wsecond = %.6e\n",
              zone_cycles, el, cycles > 0 ? zone_cycles / el : 0.0);
  athg_destroy(ctx);
  return 0;
}

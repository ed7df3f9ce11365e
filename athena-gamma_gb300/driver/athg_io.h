// athg_io.h -- restart files and VTK dumps of the C++ host, in the reference's formats.
//
// Restart (.rst, outputs/restart.cpp:42-207 and the reader Mesh::Mesh(pin, resfile),
// mesh/mesh.cpp:551-880): the parameter dump text ending in "<par_end>", then nbtotal,
// root_level, the mesh RegionSize, time, dt, ncycle and the per-block byte count, the list
// of LogicalLocation + cost, and each block's whole arrays (U, then B1f, B2f, B3f with MHD,
// ghost zones included) in the order of the reference's block tree. Files written here
// restart the reference and files the reference writes restart this host.
//
// VTK (outputs/vtk.cpp:53-215): one legacy binary RECTILINEAR_GRID file per block, face
// coordinates and cell data as big-endian float32.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace athg_io {

struct Block {
  int level;       // relative to the root grid
  int64_t lx[3];
};

struct State {
  int mesh_nx[3] = {0, 0, 0};
  double xmin[3] = {0, 0, 0}, xmax[3] = {0, 0, 0}, xrat[3] = {1.0, 1.0, 1.0};
  int block_nx[3] = {0, 0, 0};
  int ng = 2;
  bool mhd = true;
  double time = 0.0, dt = 0.0;
  int ncycle = 0;
  std::vector<Block> blocks;
  // whole arrays of every block, block after block, in the order of `blocks`
  std::vector<double> u, b1, b2, b3;
  size_t cell_count() const;   // (nx1+2ng)(nx2+2ng)(nx3+2ng)
  size_t face_count(int d) const;
};

// root level of the reference's block tree: the smallest level whose 2^level blocks per
// axis hold every root block (mesh/mesh.cpp:292)
int root_level(const int nrb[3]);

// order[gid] = index into `blocks` of the gid-th block of the reference's tree traversal
std::vector<int> tree_order(const std::vector<Block>& blocks, const int nrb[3]);

bool write_restart(const std::string& path, const std::string& params, const State& s,
                   std::string* err);
// The parameter text of a restart file (up to and including "<par_end>\n").
bool read_restart_params(const std::string& path, std::string* params, std::string* err);
// Reads a restart file. The caller sets s->ng and s->mhd (compile-time in the reference);
// they are checked against the per-block byte count of the file.
bool read_restart(const std::string& path, std::string* params, State* s, std::string* err);

// VTK dump of every block: `vars` = "prim" (rho, press, vel, Bcc) or "cons" (dens, Etot,
// mom, Bcc); w/bcc: primitives and cell-centred field of every block (same layout as u)
bool write_vtk(const std::string& basename, const std::string& file_id, int number,
               const std::string& vars, const State& s, const std::vector<double>& w,
               const std::vector<double>& bcc, std::string* err);

}  // namespace athg_io

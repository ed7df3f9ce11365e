// athg_io.cpp -- restart files and VTK dumps in the reference's formats (see athg_io.h).
#include "athg_io.h"

#include <algorithm>
#include <cstdio>
#include <cstring>

namespace athg_io {

namespace {

template <typename T>
void put(std::vector<char>* out, const T& v) {
  const char* p = reinterpret_cast<const char*>(&v);
  out->insert(out->end(), p, p + sizeof(T));
}

template <typename T>
bool take(const std::vector<char>& in, size_t* pos, T* v) {
  if (*pos + sizeof(T) > in.size()) return false;
  std::memcpy(v, in.data() + *pos, sizeof(T));
  *pos += sizeof(T);
  return true;
}

size_t block_doubles(const State& s) {
  size_t n = 5 * s.cell_count();
  if (s.mhd) n += s.face_count(0) + s.face_count(1) + s.face_count(2);
  return n;
}

// ComputeMeshGeneratorX (sym_interval) and UniformMeshGeneratorX1 (mesh/mesh.hpp:389-470)
double gen_x(int64_t index, int64_t nrange, double lo, double hi) {
  const int64_t noffset = index - nrange / 2, noffset_ceil = index - (nrange + 1) / 2;
  const double rx = static_cast<double>(noffset + noffset_ceil) / (2.0 * nrange);
  return 0.5 * (lo + hi) + (rx * hi - rx * lo);
}

// face positions of block b along axis d, interior faces only (coordinates.cpp:127-145,
// block edges as Mesh::SetBlockSizeAndBoundaries sets them)
std::vector<double> faces(const State& s, const Block& b, int d) {
  const int nrb = s.mesh_nx[d] / s.block_nx[d];
  const int64_t nroot = (int64_t)s.mesh_nx[d] << b.level, nrbl = (int64_t)nrb << b.level;
  const int nx = s.block_nx[d];
  std::vector<double> xf(nx + 1);
  for (int t = 0; t <= nx; ++t) xf[t] = gen_x(t + b.lx[d] * nx, nroot, s.xmin[d], s.xmax[d]);
  xf[0] = (b.lx[d] == 0) ? s.xmin[d] : gen_x(b.lx[d], nrbl, s.xmin[d], s.xmax[d]);
  xf[nx] = (b.lx[d] == nrbl - 1) ? s.xmax[d] : gen_x(b.lx[d] + 1, nrbl, s.xmin[d], s.xmax[d]);
  return xf;
}

void be32(float v, std::vector<char>* out) {
  uint32_t u;
  std::memcpy(&u, &v, 4);
  const char c[4] = {(char)(u >> 24), (char)(u >> 16), (char)(u >> 8), (char)u};
  out->insert(out->end(), c, c + 4);
}

}  // namespace

size_t State::cell_count() const {
  return (size_t)(block_nx[0] + 2 * ng) * (block_nx[1] + 2 * ng) * (block_nx[2] + 2 * ng);
}

size_t State::face_count(int d) const {
  const size_t n1 = block_nx[0] + 2 * ng, n2 = block_nx[1] + 2 * ng, n3 = block_nx[2] + 2 * ng;
  return d == 0 ? n3 * n2 * (n1 + 1) : (d == 1 ? n3 * (n2 + 1) * n1 : (n3 + 1) * n2 * n1);
}

int root_level(const int nrb[3]) {
  const int nbmax = std::max(nrb[0], std::max(nrb[1], nrb[2]));
  int rl = 0;
  while ((1 << rl) < nbmax) ++rl;
  return rl;
}

// Depth-first traversal of the block tree (MeshBlockTree::GetMeshBlockList): children in
// the order x fastest, then y, then z at every level, i.e. Morton order of the blocks'
// lower corners at the finest level
std::vector<int> tree_order(const std::vector<Block>& blocks, const int nrb[3]) {
  const int rl = root_level(nrb);
  int depth = 0;
  for (const Block& b : blocks) depth = std::max(depth, rl + b.level);
  std::vector<std::pair<uint64_t, int>> keys(blocks.size());
  for (size_t q = 0; q < blocks.size(); ++q) {
    const Block& b = blocks[q];
    const int sh = depth - (rl + b.level);
    const uint64_t x = (uint64_t)b.lx[0] << sh, y = (uint64_t)b.lx[1] << sh,
                   z = (uint64_t)b.lx[2] << sh;
    uint64_t key = 0;
    for (int bit = depth - 1; bit >= 0; --bit)
      key = (key << 3) | (((z >> bit) & 1) << 2) | (((y >> bit) & 1) << 1) | ((x >> bit) & 1);
    keys[q] = std::make_pair(key, (int)q);
  }
  std::sort(keys.begin(), keys.end());
  std::vector<int> order(blocks.size());
  for (size_t q = 0; q < keys.size(); ++q) order[q] = keys[q].second;
  return order;
}

bool write_restart(const std::string& path, const std::string& params, const State& s,
                   std::string* err) {
  const int nb = (int)s.blocks.size();
  int nrb[3];
  for (int d = 0; d < 3; ++d) nrb[d] = s.mesh_nx[d] / s.block_nx[d];
  const int rl = root_level(nrb);
  const size_t per = block_doubles(s);
  std::vector<char> h(params.begin(), params.end());
  put(&h, nb);
  put(&h, rl);
  // RegionSize: x1min x2min x3min x1max x2max x3max x1rat x2rat x3rat nx1 nx2 nx3 (+pad)
  for (int d = 0; d < 3; ++d) put(&h, s.xmin[d]);
  for (int d = 0; d < 3; ++d) put(&h, s.xmax[d]);
  for (int d = 0; d < 3; ++d) put(&h, s.xrat[d]);
  for (int d = 0; d < 3; ++d) put(&h, s.mesh_nx[d]);
  put(&h, (int32_t)0);
  put(&h, s.time);
  put(&h, s.dt);
  put(&h, s.ncycle);
  put(&h, (uint64_t)(per * sizeof(double)));
  const std::vector<int> order = tree_order(s.blocks, nrb);
  for (int g = 0; g < nb; ++g) {  // LogicalLocation (lx1 lx2 lx3 level + pad) and cost
    const Block& b = s.blocks[order[g]];
    for (int d = 0; d < 3; ++d) put(&h, (int64_t)b.lx[d]);
    put(&h, (int32_t)(b.level + rl));
    put(&h, (int32_t)0);
    put(&h, 1.0);
  }
  std::FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { *err = "cannot open " + path; return false; }
  bool ok = std::fwrite(h.data(), 1, h.size(), f) == h.size();
  const size_t nc = 5 * s.cell_count();
  const size_t nf[3] = {s.face_count(0), s.face_count(1), s.face_count(2)};
  for (int g = 0; g < nb && ok; ++g) {
    const size_t q = (size_t)order[g];
    ok = std::fwrite(&s.u[q * nc], sizeof(double), nc, f) == nc;
    if (s.mhd) {
      ok = ok && std::fwrite(&s.b1[q * nf[0]], sizeof(double), nf[0], f) == nf[0];
      ok = ok && std::fwrite(&s.b2[q * nf[1]], sizeof(double), nf[1], f) == nf[1];
      ok = ok && std::fwrite(&s.b3[q * nf[2]], sizeof(double), nf[2], f) == nf[2];
    }
  }
  ok = (std::fclose(f) == 0) && ok;
  if (!ok) *err = "write failed: " + path;
  return ok;
}

bool read_restart_params(const std::string& path, std::string* params, std::string* err) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) { *err = "cannot open " + path; return false; }
  std::vector<char> head(40960);
  const size_t n = std::fread(head.data(), 1, head.size(), f);
  std::fclose(f);
  const std::string h(head.data(), n);
  const size_t loc = h.find("<par_end>");
  if (loc == std::string::npos) { *err = "<par_end> not found in the first 40 KB"; return false; }
  *params = h.substr(0, loc + 10);
  return true;
}

bool read_restart(const std::string& path, std::string* params, State* s, std::string* err) {
  std::FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) { *err = "cannot open " + path; return false; }
  std::vector<char> all;
  char buf[1 << 16];
  size_t n;
  while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) all.insert(all.end(), buf, buf + n);
  std::fclose(f);
  const std::string head(all.data(), std::min(all.size(), (size_t)40960));
  const size_t loc = head.find("<par_end>");
  if (loc == std::string::npos) { *err = "<par_end> not found"; return false; }
  *params = head.substr(0, loc + 10);
  size_t pos = loc + 10;
  int nb = 0, rl = 0;
  bool ok = take(all, &pos, &nb) && take(all, &pos, &rl);
  for (int d = 0; d < 3; ++d) ok = ok && take(all, &pos, &s->xmin[d]);
  for (int d = 0; d < 3; ++d) ok = ok && take(all, &pos, &s->xmax[d]);
  for (int d = 0; d < 3; ++d) ok = ok && take(all, &pos, &s->xrat[d]);
  for (int d = 0; d < 3; ++d) ok = ok && take(all, &pos, &s->mesh_nx[d]);
  int32_t pad;
  uint64_t datasize = 0;
  ok = ok && take(all, &pos, &pad) && take(all, &pos, &s->time) && take(all, &pos, &s->dt) &&
       take(all, &pos, &s->ncycle) && take(all, &pos, &datasize);
  if (!ok || nb <= 0) { *err = "truncated restart header"; return false; }
  const size_t per = block_doubles(*s);
  if (datasize != per * sizeof(double)) {
    *err = "per-block size of the file (" + std::to_string(datasize) +
           " bytes) does not match the configuration (" + std::to_string(per * sizeof(double)) +
           " bytes: block size, nghost or magnetic fields differ)";
    return false;
  }
  s->blocks.resize(nb);
  for (int g = 0; g < nb; ++g) {
    int64_t lx[3] = {0, 0, 0};
    int32_t level = 0, p2 = 0;
    double cost = 0.0;
    for (int d = 0; d < 3; ++d) ok = ok && take(all, &pos, &lx[d]);
    ok = ok && take(all, &pos, &level) && take(all, &pos, &p2) && take(all, &pos, &cost);
    s->blocks[g].level = level - rl;
    for (int d = 0; d < 3; ++d) s->blocks[g].lx[d] = lx[d];
  }
  if (!ok) { *err = "truncated block list"; return false; }
  // data are in tree order; the list above may not be (the reader re-sorts it)
  int nrb[3];
  for (int d = 0; d < 3; ++d) nrb[d] = s->mesh_nx[d] / s->block_nx[d];
  const std::vector<int> order = tree_order(s->blocks, nrb);
  std::vector<Block> sorted(nb);
  for (int g = 0; g < nb; ++g) sorted[g] = s->blocks[order[g]];
  s->blocks = sorted;
  if (pos + per * sizeof(double) * nb > all.size()) { *err = "truncated block data"; return false; }
  const size_t nc = 5 * s->cell_count();
  const size_t nf[3] = {s->face_count(0), s->face_count(1), s->face_count(2)};
  s->u.resize(nc * nb);
  if (s->mhd) {
    s->b1.resize(nf[0] * nb); s->b2.resize(nf[1] * nb); s->b3.resize(nf[2] * nb);
  }
  for (int g = 0; g < nb; ++g) {
    std::memcpy(&s->u[g * nc], all.data() + pos, nc * sizeof(double));
    pos += nc * sizeof(double);
    if (s->mhd) {
      std::memcpy(&s->b1[g * nf[0]], all.data() + pos, nf[0] * sizeof(double));
      pos += nf[0] * sizeof(double);
      std::memcpy(&s->b2[g * nf[1]], all.data() + pos, nf[1] * sizeof(double));
      pos += nf[1] * sizeof(double);
      std::memcpy(&s->b3[g * nf[2]], all.data() + pos, nf[2] * sizeof(double));
      pos += nf[2] * sizeof(double);
    }
  }
  return true;
}

bool write_vtk(const std::string& basename, const std::string& file_id, int number,
               const std::string& vars, const State& s, const std::vector<double>& w,
               const std::vector<double>& bcc, std::string* err) {
  int nrb[3];
  for (int d = 0; d < 3; ++d) nrb[d] = s.mesh_nx[d] / s.block_nx[d];
  const std::vector<int> order = tree_order(s.blocks, nrb);
  const int ng = s.ng, n1 = s.block_nx[0] + 2 * ng, n2 = s.block_nx[1] + 2 * ng;
  const size_t nc = s.cell_count();
  const int nx1 = s.block_nx[0], nx2 = s.block_nx[1], nx3 = s.block_nx[2];
  for (size_t g = 0; g < order.size(); ++g) {
    const size_t q = (size_t)order[g];
    const Block& b = s.blocks[q];
    char name[512];
    std::snprintf(name, sizeof(name), "%s.block%d.%s.%05d.vtk", basename.c_str(), (int)g,
                  file_id.c_str(), number);
    std::vector<char> out;
    char line[256];
    auto text = [&](const char* t) { out.insert(out.end(), t, t + std::strlen(t)); };
    text("# vtk DataFile Version 2.0\n");
    std::snprintf(line, sizeof(line), "# Athena++ data at time=%e  cycle=%d  variables=%s \n",
                  s.time, s.ncycle, vars.c_str());
    text(line);
    text("BINARY\n");
    text("DATASET RECTILINEAR_GRID\n");
    std::snprintf(line, sizeof(line), "DIMENSIONS %d %d %d\n", nx1 + 1, nx2 + 1, nx3 + 1);
    text(line);
    const char* cn[3] = {"X_COORDINATES", "\nY_COORDINATES", "\nZ_COORDINATES"};
    for (int d = 0; d < 3; ++d) {
      const std::vector<double> xf = faces(s, b, d);
      std::snprintf(line, sizeof(line), "%s %d float\n", cn[d], (int)xf.size());
      text(line);
      for (double x : xf) be32((float)x, &out);
    }
    std::snprintf(line, sizeof(line), "\nCELL_DATA %d", nx1 * nx2 * nx3);
    text(line);
    const double* ub = &s.u[q * 5 * nc];
    const double* wb = &w[q * 5 * nc];
    const double* bb = s.mhd ? &bcc[q * 3 * nc] : nullptr;
    auto cell = [&](int k, int j, int i) { return ((size_t)k * n2 + j) * n1 + i; };
    auto field = [&](const char* type, const char* nm, const double* a, int nvar) {
      std::snprintf(line, sizeof(line), "\n%s %s float\n", type, nm);
      text(line);
      if (nvar == 1) text("LOOKUP_TABLE default\n");
      for (int k = ng; k < ng + nx3; ++k)
        for (int j = ng; j < ng + nx2; ++j)
          for (int i = ng; i < ng + nx1; ++i)
            for (int v = 0; v < nvar; ++v) be32((float)a[v * nc + cell(k, j, i)], &out);
    };
    if (vars == "cons") {
      field("SCALARS", "dens", ub, 1);
      field("SCALARS", "Etot", ub + 4 * nc, 1);
      field("VECTORS", "mom", ub + nc, 3);
    } else {
      field("SCALARS", "rho", wb, 1);
      field("SCALARS", "press", wb + 4 * nc, 1);
      field("VECTORS", "vel", wb + nc, 3);
    }
    if (s.mhd) field("VECTORS", "Bcc", bb, 3);
    std::FILE* f = std::fopen(name, "wb");
    if (!f) { *err = std::string("cannot open ") + name; return false; }
    const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
    if (std::fclose(f) != 0 || !ok) { *err = std::string("write failed: ") + name; return false; }
  }
  return true;
}

}  // namespace athg_io

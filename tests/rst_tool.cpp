// rst_tool.cpp -- the restart reader/writer of the C++ host (driver/athg_io.cpp) as a
// command-line tool (test infrastructure): the tests check with it that the reference
// restarts from files this writer makes and that the reader takes the reference's files.
//
//   rst_tool copy <in.rst> <out.rst> nx1 nx2 nx3 nghost mhd
//     read a restart file with athg_io::read_restart and write it again with
//     athg_io::write_restart (same parameters text, same state)
//   rst_tool info <in.rst> nx1 nx2 nx3 nghost mhd
//     print time, dt, ncycle and the block list in tree order
#include <cstdio>
#include <cstdlib>
#include <string>

#include "athg_io.h"

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::string cmd = argv[1];
  const int base = cmd == "copy" ? 4 : 3;
  if (argc != base + 5) { std::fprintf(stderr, "bad arguments\n"); return 2; }
  athg_io::State s;
  for (int d = 0; d < 3; ++d) s.block_nx[d] = std::atoi(argv[base + d]);
  s.ng = std::atoi(argv[base + 3]);
  s.mhd = std::atoi(argv[base + 4]) != 0;
  std::string params, err;
  if (!athg_io::read_restart(argv[2], &params, &s, &err)) {
    std::fprintf(stderr, "read: %s\n", err.c_str());
    return 1;
  }
  if (cmd == "info") {
    std::printf("time %.17g dt %.17g ncycle %d nblocks %d\n", s.time, s.dt, s.ncycle,
                (int)s.blocks.size());
    for (const auto& b : s.blocks)
      std::printf("%d %lld %lld %lld\n", b.level, (long long)b.lx[0], (long long)b.lx[1],
                  (long long)b.lx[2]);
    return 0;
  }
  if (!athg_io::write_restart(argv[3], params, s, &err)) {
    std::fprintf(stderr, "write: %s\n", err.c_str());
    return 1;
  }
  return 0;
}

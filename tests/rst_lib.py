"""Restart files (.rst) in the reference's format, read with numpy (test infrastructure).

Layout (outputs/restart.cpp:42-207): parameter text up to "<par_end>\\n"; int nbtotal,
int root_level, RegionSize (9 float64, 3 int32, 4 bytes padding), float64 time, float64 dt,
int32 ncycle, uint64 bytes per block; per block LogicalLocation (3 int64, int32 level,
4 bytes padding) and float64 cost; then every block's U (and B1f, B2f, B3f with MHD) with
ghost zones, in the order of the block list."""
import struct

import numpy as np


def read_rst(path, block_nx, ng, mhd):
    data = open(path, "rb").read()
    end = data.find(b"<par_end>")
    params = data[:end + 10].decode()
    pos = end + 10
    nb, rl = struct.unpack_from("<2i", data, pos)
    pos += 8
    region = struct.unpack_from("<9d3i", data, pos)
    pos += 88
    time, dt = struct.unpack_from("<2d", data, pos)
    pos += 16
    (ncycle,) = struct.unpack_from("<i", data, pos)
    pos += 4
    (dsize,) = struct.unpack_from("<Q", data, pos)
    pos += 8
    blocks = []
    for _ in range(nb):
        lx1, lx2, lx3, lev = struct.unpack_from("<3qi", data, pos)
        pos += 40
        blocks.append((lev - rl, lx1, lx2, lx3))
    n1, n2, n3 = (n + 2 * ng for n in block_nx)
    shapes = [("u", (5, n3, n2, n1))]
    if mhd:
        shapes += [("b1", (n3, n2, n1 + 1)), ("b2", (n3, n2 + 1, n1)), ("b3", (n3 + 1, n2, n1))]
    per = sum(int(np.prod(s)) for _, s in shapes) * 8
    assert per == dsize, (per, dsize)
    arrays = []
    for _ in range(nb):
        d = {}
        for k, s in shapes:
            cnt = int(np.prod(s))
            d[k] = np.frombuffer(data, dtype="<f8", count=cnt, offset=pos).reshape(s).copy()
            pos += cnt * 8
        arrays.append(d)
    assert pos == len(data)
    return {"params": params, "root_level": rl, "region": region, "time": time, "dt": dt,
            "ncycle": ncycle, "blocks": blocks, "arrays": arrays}

"""Multi-level (SMR) meshes for the tests: block lists, seeded states, and the reference run.

Test infrastructure only. The block list follows the reference's Mesh constructor for
<refinementN> regions (src/mesh/mesh.cpp:334-462: logical ranges of the region at its
level, widened to whole parents, then MeshBlockTree::AddMeshBlock), restricted to regions
of level 1. Face positions follow the uniform mesh generator
(src/mesh/mesh.hpp:389-470) so the seeded fields can be evaluated at the reference's own
coordinates; the seeded face field is the edge-integrated curl of a vector potential whose
components are constant along their own axis, so coarse faces are exact sums of fine
faces and every block starts divergence-free.
"""
import os
import struct
import subprocess

import numpy as np

NHYD = 5


def gen_rx(index, nrange):
    """ComputeMeshGeneratorX(index, nrange, sym_interval=true), src/mesh/mesh.hpp:389-405."""
    noffset = index - nrange // 2
    noffset_ceil = index - (nrange + 1) // 2
    return float(noffset + noffset_ceil) / (2.0 * nrange)


def gen_x(rx, xmin, xmax):
    """UniformMeshGeneratorX1, src/mesh/mesh.hpp:467-470."""
    return 0.5 * (xmin + xmax) + (rx * xmax - rx * xmin)


def region_range(reg, level, nrb, domain):
    """Logical range [a, b) of a region at `level` along each axis, widened to whole parents
    (mesh/mesh.cpp:334-462)."""
    rng = []
    for d in range(3):
        lo, hi = reg[2 * d], reg[2 * d + 1]
        lxmax = nrb[d] << level
        a = 0
        while a < lxmax:
            if gen_x(gen_rx(a + 1, lxmax), *domain[d]) > lo:
                break
            a += 1
        b = a
        while b < lxmax:
            if gen_x(gen_rx(b + 1, lxmax), *domain[d]) >= hi:
                break
            b += 1
        if a % 2 == 1:
            a -= 1
        if b % 2 == 0:
            b += 1
        rng.append((a, b))
    return rng


def smr_blocks(root_nx, mb, domain, regions):
    """Sorted list of (level, lx1, lx2, lx3) leaves. regions: [(x1min, x1max, x2min, x2max,
    x3min, x3max[, level])], level 1 by default. A level-2 region must lie inside the level-1
    regions with a block of margin, so that splitting its level-1 parents needs no further
    refinement for the 2:1 rule (MeshBlockTree::Refine then adds nothing)."""
    nrb = [root_nx[d] // mb[d] for d in range(3)]
    leaves = {(0, i, j, k) for k in range(nrb[2]) for j in range(nrb[1]) for i in range(nrb[0])}
    for level in (1, 2):
        for reg in regions:
            if (reg[6] if len(reg) > 6 else 1) != level:
                continue
            rng = region_range(reg, level, nrb, domain)
            for k in range(rng[2][0], rng[2][1], 2):
                for j in range(rng[1][0], rng[1][1], 2):
                    for i in range(rng[0][0], rng[0][1], 2):
                        parent = (level - 1, i // 2, j // 2, k // 2)
                        if parent not in leaves:
                            assert any(l[0] >= level and (l[1] >> (l[0] - level + 1), l[2] >> (l[0] - level + 1),
                                       l[3] >> (l[0] - level + 1)) == parent[1:] for l in leaves), parent
                            continue
                        leaves.discard(parent)
                        for c in range(8):
                            leaves.add((level, i + (c & 1), j + ((c >> 1) & 1), k + (c >> 2)))
    if any(l[0] == 2 for l in leaves):  # the 2:1 rule: level-2 blocks touch no level-0 block
        for a in leaves:
            if a[0] != 2:
                continue
            for b in leaves:
                if b[0] == 0:
                    lo_a = [x / 4.0 for x in a[1:]]
                    hi_a = [(x + 1) / 4.0 for x in a[1:]]
                    lo_b, hi_b = list(b[1:]), [x + 1 for x in b[1:]]
                    touch = all(lo_a[d] <= hi_b[d] and lo_b[d] <= hi_a[d] for d in range(3))
                    assert not touch, ("level-2 region too close to level 0", a, b)
    return sorted(leaves)


def block_faces(blk, root_nx, mb, domain, d, ng=0):
    """Face positions of block blk along axis d, including ng ghost faces on each side
    (coordinates.cpp:127-145: interior faces from the generator, end faces = block edges)."""
    level, lx = blk[0], blk[1 + d]
    nroot = root_nx[d] * (1 << level)
    n = mb[d]
    xf = np.empty(n + 2 * ng + 1)
    for t in range(-ng, n + ng + 1):
        xf[t + ng] = gen_x(gen_rx(t + lx * n, nroot), *domain[d])
    xf[ng] = gen_x(gen_rx(lx * n, nroot), *domain[d])
    xf[ng + n] = gen_x(gen_rx((lx + 1) * n, nroot), *domain[d])
    return xf


def smr_initial_state(blocks, root_nx, mb, domain, mhd, gamma=5.0 / 3.0, seed=0, amp=0.3):
    """Seeded smooth state per block (interior): dict blk -> (u, b1, b2, b3)."""
    rng = np.random.default_rng(seed)
    ph = rng.uniform(0.0, 2.0 * np.pi, size=12)
    L = [domain[d][1] - domain[d][0] for d in range(3)]
    kx = [2.0 * np.pi / L[d] for d in range(3)]
    b0 = np.array([0.7, 0.5, 0.3]) if mhd else np.zeros(3)
    # vector potential components constant along their own axis
    ga = 0.08

    def Ax(y, z):
        return ga * np.sin(kx[1] * y + ph[8]) * np.cos(kx[2] * z + ph[9])

    def Ay(z, x):
        return ga * np.sin(kx[2] * z + ph[10]) * np.sin(kx[0] * x + ph[11])

    def Az(x, y):
        return ga * np.cos(kx[0] * x + ph[6]) * np.sin(kx[1] * y + ph[7])

    out = {}
    for blk in blocks:
        xf = [block_faces(blk, root_nx, mb, domain, d) for d in range(3)]
        xv = [0.5 * (f[1:] + f[:-1]) for f in xf]
        Z, Y, X = np.meshgrid(xv[2], xv[1], xv[0], indexing="ij")
        rho = 1.0 + amp * np.sin(kx[0] * X + ph[0]) * np.cos(kx[1] * Y + ph[1]) * \
            np.cos(kx[2] * Z + ph[2])
        vx = amp * np.sin(kx[1] * Y + ph[3])
        vy = amp * np.cos(kx[2] * Z + ph[4])
        vz = amp * np.sin(kx[0] * X + ph[5])
        p = 1.0 + 0.5 * amp * np.cos(kx[0] * X + ph[1]) * np.sin(kx[2] * Z + ph[3])
        b1 = b2 = b3 = None
        bc2 = 0.0
        if mhd:
            # x1 faces: (Ay(z0,x) - Ay(z1,x)) / dz + (Az(x,y1) - Az(x,y0)) / dy
            Z1, Y1, X1 = np.meshgrid(xf[2][:-1], xf[1][:-1], xf[0], indexing="ij")
            Z2, Y2, _ = np.meshgrid(xf[2][1:], xf[1][1:], xf[0], indexing="ij")
            b1 = b0[0] + (Ay(Z1, X1) - Ay(Z2, X1)) / (Z2 - Z1) + (Az(X1, Y2) - Az(X1, Y1)) / (Y2 - Y1)
            # x2 faces: (Az(x0,y) - Az(x1,y)) / dx + (Ax(y,z1) - Ax(y,z0)) / dz
            Z1, Y1, X1 = np.meshgrid(xf[2][:-1], xf[1], xf[0][:-1], indexing="ij")
            Z2, _, X2 = np.meshgrid(xf[2][1:], xf[1], xf[0][1:], indexing="ij")
            b2 = b0[1] + (Az(X1, Y1) - Az(X2, Y1)) / (X2 - X1) + (Ax(Y1, Z2) - Ax(Y1, Z1)) / (Z2 - Z1)
            # x3 faces: (Ax(y0,z) - Ax(y1,z)) / dy + (Ay(z,x1) - Ay(z,x0)) / dx
            Z1, Y1, X1 = np.meshgrid(xf[2], xf[1][:-1], xf[0][:-1], indexing="ij")
            _, Y2, X2 = np.meshgrid(xf[2], xf[1][1:], xf[0][1:], indexing="ij")
            b3 = b0[2] + (Ax(Y1, Z1) - Ax(Y2, Z1)) / (Y2 - Y1) + (Ay(Z1, X2) - Ay(Z1, X1)) / (X2 - X1)
            bcx = 0.5 * (b1[:, :, 1:] + b1[:, :, :-1])
            bcy = 0.5 * (b2[:, 1:, :] + b2[:, :-1, :])
            bcz = 0.5 * (b3[1:, :, :] + b3[:-1, :, :])
            bc2 = bcx ** 2 + bcy ** 2 + bcz ** 2
        u = np.empty((NHYD,) + rho.shape)
        u[0] = rho
        u[1] = rho * vx
        u[2] = rho * vy
        u[3] = rho * vz
        u[4] = p / (gamma - 1.0) + 0.5 * rho * (vx * vx + vy * vy + vz * vz) + 0.5 * bc2
        out[blk] = (u, b1, b2, b3)
    return out


def write_blocks_in(path, blocks, states, mhd):
    with open(path, "wb") as f:
        f.write(struct.pack("<q", len(blocks)))
        for blk in blocks:
            f.write(struct.pack("<4q", *blk))
            u, b1, b2, b3 = states[blk]
            f.write(np.ascontiguousarray(u, dtype="<f8").tobytes())
            if mhd:
                for a in (b1, b2, b3):
                    f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())


def read_blocks_out(path, mb, ng, mhd, ghosts):
    """dict blk -> dict of arrays; plus (time, dt, ncycle)."""
    n1, n2, n3 = mb
    if ghosts:
        n1, n2, n3 = n1 + 2 * ng, n2 + 2 * ng, n3 + 2 * ng
    with open(path, "rb") as f:
        t, dt, nc = struct.unpack("<3d", f.read(24))
        (nb,) = struct.unpack("<q", f.read(8))
        res = {}
        for _ in range(nb):
            blk = struct.unpack("<4q", f.read(32))
            d = {}

            def take(shape):
                cnt = int(np.prod(shape))
                return np.frombuffer(f.read(8 * cnt), dtype="<f8").reshape(shape).copy()

            d["u"] = take((NHYD, n3, n2, n1))
            if ghosts:
                d["w"] = take((NHYD, n3, n2, n1))
            if mhd:
                d["b1"] = take((n3, n2, n1 + 1))
                d["b2"] = take((n3, n2 + 1, n1))
                d["b3"] = take((n3 + 1, n2, n1))
            res[tuple(blk)] = d
    return res, (t, dt, nc)


def athinput(root_nx, mb, domain, regions, cfl, nlim, gamma, xorder, integrator, ghosts):
    s = ["<job>", "problem_id = smr", "<time>", "cfl_number = %r" % cfl, "nlim = %d" % nlim,
         "tlim = 100.0", "integrator = %s" % integrator, "xorder = %d" % xorder,
         "ncycle_out = 100000", "<mesh>"]
    for d in range(3):
        s += ["nx%d = %d" % (d + 1, root_nx[d]), "x%dmin = %r" % (d + 1, domain[d][0]),
              "x%dmax = %r" % (d + 1, domain[d][1]), "ix%d_bc = periodic" % (d + 1),
              "ox%d_bc = periodic" % (d + 1)]
    s += ["refinement = static", "<meshblock>", "nx1 = %d" % mb[0], "nx2 = %d" % mb[1],
          "nx3 = %d" % mb[2], "<hydro>", "gamma = %r" % gamma]
    for r, reg in enumerate(regions):
        s += ["<refinement%d>" % (r + 1)]
        for d in range(3):
            s += ["x%dmin = %r" % (d + 1, reg[2 * d]), "x%dmax = %r" % (d + 1, reg[2 * d + 1])]
        s += ["level = %d" % (reg[6] if len(reg) > 6 else 1)]
    s += ["<problem>", "state_in = state_in.bin", "state_out = state_out.bin",
          "ghosts = %s" % ("true" if ghosts else "false")]
    return "\n".join(s) + "\n"


def run_reference_smr(exe, workdir, root_nx, mb, domain, regions, blocks, states, mhd, ng,
                      cfl, nlim, gamma, xorder, integrator, ghosts):
    os.makedirs(workdir, exist_ok=True)
    write_blocks_in(os.path.join(workdir, "state_in.bin"), blocks, states, mhd)
    with open(os.path.join(workdir, "athinput.smr"), "w") as f:
        f.write(athinput(root_nx, mb, domain, regions, cfl, nlim, gamma, xorder, integrator,
                         ghosts))
    r = subprocess.run([exe, "-i", "athinput.smr"], cwd=workdir, capture_output=True, text=True)
    if r.returncode != 0 or "FATAL" in r.stdout:
        raise RuntimeError("reference run failed:\n" + r.stdout[-2000:] + r.stderr[-2000:])
    return read_blocks_out(os.path.join(workdir, "state_out.bin"), mb, ng, mhd, ghosts)


def write_check_in(path, blocks, states, mesh_nx, mb, ng, domain, mhd, gamma, dfloor, pfloor):
    """Input of tests/smr_check.cpp (see its header)."""
    with open(path, "wb") as f:
        f.write(struct.pack("<9i", mb[0], mb[1], mb[2], ng, mesh_nx[0], mesh_nx[1], mesh_nx[2],
                            1 if mhd else 0, len(blocks)))
        f.write(struct.pack("<9d", domain[0][0], domain[0][1], domain[1][0], domain[1][1],
                            domain[2][0], domain[2][1], gamma, dfloor, pfloor))
        for blk in blocks:
            f.write(struct.pack("<4q", *blk))
            u, b1, b2, b3 = states[blk]
            f.write(np.ascontiguousarray(u, dtype="<f8").tobytes())
            if mhd:
                for a in (b1, b2, b3):
                    f.write(np.ascontiguousarray(a, dtype="<f8").tobytes())


def read_check_out(path, blocks, mb, ng, mhd):
    n1, n2, n3 = (m + 2 * ng for m in mb)
    res = {}
    with open(path, "rb") as f:
        for blk in blocks:
            def take(shape):
                cnt = int(np.prod(shape))
                return np.frombuffer(f.read(8 * cnt), dtype="<f8").reshape(shape).copy()
            d = {"u": take((NHYD, n3, n2, n1)), "w": take((NHYD, n3, n2, n1))}
            if mhd:
                d["b1"] = take((n3, n2, n1 + 1))
                d["b2"] = take((n3, n2 + 1, n1))
                d["b3"] = take((n3 + 1, n2, n1))
            res[blk] = d
        sizes = struct.unpack("<8q", f.read(64))
    return res, sizes

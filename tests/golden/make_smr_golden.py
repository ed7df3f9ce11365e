#!/usr/bin/env python3
"""Golden fixtures for static mesh refinement, made by running the unmodified reference.

Needs the reference source tree (development container only). For each case it builds
the reference with the multi-level harness problem generator (oracle/build_ref.py,
oracle/harness/load_blocks.cpp), loads a seeded divergence-free state into every block of
a two-level periodic mesh (tests/smr_lib.py), and stores as compressed .npz:
  blocks        (N, 4) leaves (level, lx1, lx2, lx3), sorted
  *_in          interior state per block (u, b1, b2, b3)
  *_init        the whole arrays after Mesh::Initialize, ghost zones included (cases with
                ghosts=True): ghost fill across levels, prolongation, W(U)
  *_out         interior state after `ncycles` cycles

    python tests/golden/make_smr_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402
import smr_lib as sl  # noqa: E402

WORK = os.path.join(ROOT, "_work", "golden_smr")
DOM = ((-1.0, 1.0), (-1.0, 1.0), (-1.0, 1.0))

# name: (exe config, mhd, solver, root nx, meshblock nx, nghost, regions, integrator, xorder,
#        ncycles, seed, cfl, ghosts)
CASES = {
    "smr_mhd_hlld_plm_vl2": ("smr_mhd_hlld", True, "hlld", (12, 12, 12), (4, 4, 4), 2,
                             [(0.05, 0.9, 0.05, 0.3, 0.05, 0.3)], "vl2", 2, 4, 7, 0.3, True),
    "smr_hydro_hllc_plm_vl2": ("smr_hydro_hllc", False, "hllc", (12, 12, 12), (4, 4, 4), 2,
                               [(-0.9, -0.1, 0.05, 0.3, 0.05, 0.9)], "vl2", 2, 4, 8, 0.3, True),
    "smr_mhd_hlld_ppm_rk3": ("smr_mhd_hlld_ng4", True, "hlld", (24, 24, 24), (8, 8, 8), 4,
                             [(0.05, 0.3, 0.05, 0.3, 0.05, 0.3)], "rk3", 3, 3, 9, 0.3, False),
    # three levels: the central half at level 1 and a small central region at level 2
    "smr3_mhd_hlld_plm_vl2": ("smr_mhd_hlld", True, "hlld", (16, 16, 16), (4, 4, 4), 2,
                              [(-0.5, 0.5, -0.5, 0.5, -0.5, 0.5, 1),
                               (-0.05, 0.05, -0.05, 0.05, -0.05, 0.05, 2)], "vl2", 2, 4, 11,
                              0.3, False),
}
GAMMA = 5.0 / 3.0


def make_case(name, spec):
    cfg, mhd, solver, root, mb, ng, regions, integ, xorder, ncyc, seed, cfl, ghosts = spec
    exe = build_ref.build(cfg)
    blocks = sl.smr_blocks(root, mb, DOM, regions)
    st = sl.smr_initial_state(blocks, root, mb, DOM, mhd, gamma=GAMMA, seed=seed)
    arrays = {"blocks": np.array(blocks, dtype=np.int64)}
    keys = ("u", "b1", "b2", "b3") if mhd else ("u",)
    for q, k in enumerate(keys):
        arrays[k + "_in"] = np.stack([st[b][q] for b in blocks])
    if ghosts:
        init, _ = sl.run_reference_smr(exe, os.path.join(WORK, name + "_init"), root, mb, DOM,
                                       regions, blocks, st, mhd, ng, cfl, 0, GAMMA, xorder,
                                       integ, True)
        for k in ("u", "w") + keys[1:]:
            arrays[k + "_init"] = np.stack([init[b][k] for b in blocks])
    out, (t, dt, nc) = sl.run_reference_smr(exe, os.path.join(WORK, name), root, mb, DOM,
                                            regions, blocks, st, mhd, ng, cfl, ncyc, GAMMA,
                                            xorder, integ, False)
    # the reference's own mesh has exactly these leaves
    assert sorted(out) == blocks, "block lists differ"
    for k in keys:
        arrays[k + "_out"] = np.stack([out[b][k] for b in blocks])
    meta = dict(mhd=mhd, solver=solver, root=list(root), meshblock=list(mb), nghost=ng,
                regions=[list(r) for r in regions], integrator=integ, xorder=xorder,
                ncycles=ncyc, seed=seed, cfl=cfl, gamma=GAMMA, domain=[list(x) for x in DOM],
                time=t, dt=dt, ncycle=nc, ghosts=ghosts)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **arrays)
    print("wrote", name, "blocks=%d t=%.6g ncycle=%d" % (len(blocks), t, nc))


if __name__ == "__main__":
    if not build_ref.available():
        print("reference tree not present; nothing to do")
        sys.exit(0)
    names = sys.argv[1:] or list(CASES)
    for n in names:
        make_case(n, CASES[n])

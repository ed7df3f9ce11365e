#!/usr/bin/env python3
"""Generate the golden fixtures in tests/golden/ by running the unmodified reference.

Needs the reference source tree (development container only). For each case it builds
the reference with the state-loading harness problem generator (oracle/build_ref.py,
oracle/harness/load_state.cpp), runs it on a seeded smooth state for a few cycles, and
stores input and output states (FP64) as compressed .npz. The linear-wave known-answer
numbers come from the reference's own linear_wave problem generator
(linearwave-errors.dat).

    python tests/golden/make_golden.py
"""
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "tests"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402
import oracle_lib as ol  # noqa: E402

WORK = os.path.join(ROOT, "_work", "golden_runs")
REF = build_ref.REF

# name: (exe config, mhd, solver, mesh nx, meshblock nx, integrator, xorder, ncycles, seed, cfl)
CASES = {
    "hydro_hllc_plm_vl2": ("state_hydro_hllc", False, "hllc", (16, 8, 8), (16, 8, 8), "vl2", 2, 3, 3, 0.4),
    "hydro_hlle_plm_vl2": ("state_hydro_hlle", False, "hlle", (16, 8, 8), (16, 8, 8), "vl2", 2, 3, 5, 0.4),
    "hydro_hllc_plm_rk3": ("state_hydro_hllc", False, "hllc", (16, 8, 8), (16, 8, 8), "rk3", 2, 3, 11, 0.8),
    "hydro_hllc_dc_rk2": ("state_hydro_hllc", False, "hllc", (16, 8, 8), (16, 8, 8), "rk2", 1, 3, 12, 0.8),
    "mhd_hlld_plm_vl2": ("state_mhd_hlld", True, "hlld", (16, 8, 8), (16, 8, 8), "vl2", 2, 3, 3, 0.4),
    "mhd_hlle_plm_vl2": ("state_mhd_hlle", True, "hlle", (16, 8, 8), (16, 8, 8), "vl2", 2, 3, 9, 0.4),
    "mhd_hlld_plm_rk2": ("state_mhd_hlld", True, "hlld", (16, 8, 8), (16, 8, 8), "rk2", 2, 3, 13, 0.8),
    "mhd_hlld_plm_vl2_4blocks": ("state_mhd_hlld", True, "hlld", (16, 16, 8), (8, 8, 8), "vl2", 2, 3, 21, 0.4),
    "hydro_hllc_ppm_rk3": ("state_hydro_hllc_ng4", False, "hllc", (16, 8, 8), (16, 8, 8), "rk3", 3, 3, 31, 0.8),
    "mhd_hlld_ppm_rk3": ("state_mhd_hlld_ng4", True, "hlld", (16, 8, 8), (16, 8, 8), "rk3", 3, 3, 32, 0.8),
    "mhd_hlld_ppm_vl2": ("state_mhd_hlld_ng4", True, "hlld", (16, 8, 8), (16, 8, 8), "vl2", 3, 3, 33, 0.4),
    "hydro_lhllc_plm_vl2": ("state_hydro_lhllc", False, "lhllc", (16, 8, 8), (16, 8, 8), "vl2", 2, 3, 41, 0.4),
    "hydro_lhllc_plm_rk3": ("state_hydro_lhllc", False, "lhllc", (16, 8, 8), (16, 8, 8), "rk3", 2, 3, 42, 0.8),
    "mhd_lhlld_plm_vl2": ("state_mhd_lhlld", True, "lhlld", (16, 8, 8), (16, 8, 8), "vl2", 2, 3, 43, 0.4),
    "mhd_lhlld_plm_rk2": ("state_mhd_lhlld", True, "lhlld", (16, 8, 8), (16, 8, 8), "rk2", 2, 3, 44, 0.8),
}
NGHOST = {"state_hydro_hllc_ng4": 4, "state_mhd_hlld_ng4": 4}
# outflow physical boundaries on every face (bvals/cc/outflow_cc.cpp, bvals/fc/outflow_fc.cpp):
# two blocks along x1, so the same-level exchange and the physical boundaries both act
OUTFLOW = {"hydro_hllc_plm_vl2_outflow", "mhd_hlld_plm_vl2_outflow"}
CASES["hydro_hllc_plm_vl2_outflow"] = ("state_hydro_hllc", False, "hllc", (16, 8, 8), (8, 8, 8),
                                       "vl2", 2, 3, 51, 0.4)
CASES["mhd_hlld_plm_vl2_outflow"] = ("state_mhd_hlld", True, "hlld", (16, 8, 8), (8, 8, 8),
                                     "vl2", 2, 3, 52, 0.4)


def make_case(name, spec):
    exe_cfg, mhd, solver, nx, mb, integ, xorder, ncyc, seed, cfl = spec
    exe = build_ref.build(exe_cfg)
    u, b1, b2, b3 = ol.smooth_random_state(nx, mhd, seed=seed)
    bc = "outflow" if name in OUTFLOW else "periodic"
    out = ol.run_reference_state(exe, os.path.join(WORK, name), nx, mb, mhd, u, b1, b2, b3,
                                 cfl=cfl, tlim=100.0, nlim=ncyc, xorder=xorder, integrator=integ,
                                 mesh_bc=bc)
    arrays = {"u_in": u, "u_out": out["u"]}
    if mhd:
        arrays.update(b1_in=b1, b2_in=b2, b3_in=b3, b1_out=out["b1"], b2_out=out["b2"],
                      b3_out=out["b3"])
    meta = dict(mhd=mhd, solver=solver, nx=list(nx), meshblock=list(mb), integrator=integ,
                xorder=xorder, ncycles=ncyc, seed=seed, cfl=cfl, gamma=5.0 / 3.0,
                time=out["time"], dt=out["dt"], ncycle=out["ncycle"],
                nghost=NGHOST.get(exe_cfg, 2), bc=bc)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **arrays)
    print("wrote", name, "t=%.6g ncycle=%d" % (out["time"], out["ncycle"]))


# multigrid: name -> (N, meshblock, bc, mode, niteration, density kind, seed)
MG_CASES = {
    "mg_periodic_fmg": (32, 8, "periodic", "FMG", 4, "smooth", 41),
    "mg_periodic_mgi": (32, 16, "periodic", "MGI", 3, "smooth", 42),
    "mg_sphere_multipole4": (32, 8, "multipole", "FMG", 4, "sphere", 0),
    "mg_zerofixed_fmg": (16, 8, "zerofixed", "FMG", 3, "smooth", 43),
}
FOUR_PI_G = 4.0 * np.pi


def mg_density(n, kind, seed):
    x = (np.arange(n) + 0.5) / n - 0.5
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    if kind == "sphere":  # rho = 1 inside r < 0.25, 1e-6 outside
        r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
        return np.where(r < 0.25, 1.0, 1.0e-6)
    rng = np.random.default_rng(seed)
    rho = np.ones_like(X)
    for _ in range(4):
        k = rng.integers(1, 4, size=3)
        ph = rng.uniform(0, 2 * np.pi, size=3)
        rho += 0.3 * rng.uniform(-1, 1) * (np.cos(2 * np.pi * k[0] * X + ph[0]) *
                                           np.cos(2 * np.pi * k[1] * Y + ph[1]) *
                                           np.cos(2 * np.pi * k[2] * Z + ph[2]))
    return rho


def make_mg_case(name, spec):
    n, mb, bc, mode, niter, kind, seed = spec
    exe = build_ref.build("sg_state_hydro")
    rho = mg_density(n, kind, seed)
    u = np.zeros((5, n, n, n))
    u[0] = rho
    u[4] = 1.0 / (5.0 / 3.0 - 1.0)
    bcs = bc
    extra = "four_pi_G = %r" % FOUR_PI_G
    blocks = ("<gravity>\nmgmode = %s\nniteration = %d\nix1_bc = %s\nox1_bc = %s\n"
              "ix2_bc = %s\nox2_bc = %s\nix3_bc = %s\nox3_bc = %s\n"
              % (mode, niter, bcs, bcs, bcs, bcs, bcs, bcs))
    if bc == "multipole":
        blocks += "mporder = 4\nauto_mporigin = true\n"
    dom = ((-0.5, 0.5),) * 3
    out = ol.run_reference_state(exe, os.path.join(WORK, name), (n, n, n), (mb, mb, mb), False,
                                 u, None, None, None, cfl=0.3, tlim=1.0, nlim=0,
                                 domain=dom, extra=extra, phi=True, blocks=blocks,
                                 mesh_bc="periodic" if bc == "periodic" else "outflow")
    meta = dict(n=n, meshblock=mb, bc=bc, mode=mode, niteration=niter, kind=kind, seed=seed,
                four_pi_G=FOUR_PI_G)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), rho=rho,
                        phi=out["phi"])
    print("wrote", name)


# self-gravity evolution: name -> (exe config, mhd, solver, N, meshblock, integrator,
# ncycles, seed, cfl, four_pi_G, MG mode, niteration)
SG_CASES = {
    "sg_hydro_hllc_plm_vl2": ("sg_state_hydro", False, "hllc", 32, 32, "vl2", 3, 51, 0.4,
                              2.0 * np.pi, "FMG", 2),
    "sg_hydro_hllc_plm_vl2_8blocks": ("sg_state_hydro", False, "hllc", 32, 16, "vl2", 3, 52,
                                      0.4, 2.0 * np.pi, "FMG", 2),
    "sg_mhd_hlld_plm_vl2": ("sg_state_mhd_hlld", True, "hlld", 32, 32, "vl2", 3, 53, 0.4,
                            2.0 * np.pi, "FMG", 2),
}


def make_sg_case(name, spec):
    exe_cfg, mhd, solver, n, mb, integ, ncyc, seed, cfl, fpg, mode, niter = spec
    exe = build_ref.build(exe_cfg)
    nx = (n, n, n)
    u, b1, b2, b3 = ol.smooth_random_state(nx, mhd, seed=seed)
    extra = "four_pi_G = %r" % fpg
    blocks = ("<gravity>\nmgmode = %s\nniteration = %d\n" % (mode, niter) +
              "".join("%s = periodic\n" % f for f in
                      ("ix1_bc", "ox1_bc", "ix2_bc", "ox2_bc", "ix3_bc", "ox3_bc")))
    out = ol.run_reference_state(exe, os.path.join(WORK, name), nx, (mb, mb, mb), mhd, u, b1,
                                 b2, b3, cfl=cfl, tlim=100.0, nlim=ncyc, integrator=integ,
                                 extra=extra, phi=True, blocks=blocks)
    arrays = {"u_in": u, "u_out": out["u"], "phi_out": out["phi"]}
    if mhd:
        arrays.update(b1_in=b1, b2_in=b2, b3_in=b3, b1_out=out["b1"], b2_out=out["b2"],
                      b3_out=out["b3"])
    meta = dict(mhd=mhd, solver=solver, nx=list(nx), meshblock=[mb] * 3, integrator=integ,
                xorder=2, ncycles=ncyc, seed=seed, cfl=cfl, gamma=5.0 / 3.0,
                time=out["time"], dt=out["dt"], ncycle=out["ncycle"], nghost=2,
                four_pi_G=fpg, mgmode=mode, niteration=niter, self_gravity=True)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **arrays)
    print("wrote", name, "t=%.6g ncycle=%d" % (out["time"], out["ncycle"]))


def linear_wave_errors():
    """Reference's own linear-wave L1 errors (C1 hydro; MHD fast wave)."""
    res = {}
    runs = {
        "hydro_c1": ("lw_hydro_hllc", "inputs/hydro/athinput.linear_wave3d",
                     ["time/tlim=1.0", "time/cfl_number=0.4"]),
        "mhd_fast": ("lw_mhd_hlld", "inputs/mhd/athinput.linear_wave3d",
                     ["time/tlim=0.5", "time/cfl_number=0.3"]),
    }
    for key, (cfg, inp, extra) in runs.items():
        exe = build_ref.build(cfg)
        wd = os.path.join(WORK, "lw_" + key)
        os.makedirs(wd, exist_ok=True)
        f = os.path.join(wd, "linearwave-errors.dat")
        if os.path.exists(f):
            os.remove(f)
        cmd = [exe, "-i", os.path.join(REF, inp), "output1/dt=-1", "output2/dt=-1",
               "problem/compute_error=true"] + extra
        subprocess.run(cmd, cwd=wd, check=True, capture_output=True)
        line = [l for l in open(f) if not l.startswith("#")][0].split()
        hdr = open(f).readline().lstrip("# ").split()
        res[key] = {"args": extra, "columns": hdr, "values": [float(x) for x in line]}
        print(key, line[:6])
    with open(os.path.join(HERE, "linear_wave_errors.json"), "w") as fo:
        json.dump(res, fo, indent=1)


if __name__ == "__main__":
    if not build_ref.available():
        sys.exit("reference tree not found")
    names = sys.argv[1:] or (list(CASES) + list(MG_CASES) + list(SG_CASES))
    for n in names:
        if n == "lw":
            continue
        if n in MG_CASES:
            make_mg_case(n, MG_CASES[n])
        elif n in SG_CASES:
            make_sg_case(n, SG_CASES[n])
        else:
            make_case(n, CASES[n])
    if not sys.argv[1:] or "lw" in sys.argv[1:]:
        linear_wave_errors()

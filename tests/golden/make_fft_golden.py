#!/usr/bin/env python3
"""Generate the FFT fixtures (turbulence driving, FFT self-gravity) in tests/golden/ by
running the unmodified reference's own FFT drivers.

The reference's FFT code calls FFTW, which this machine does not have; oracle/build_ref.py
compiles the unmodified sources against oracle/harness/fftw3 (the FFTW calls the reference
makes, served by direct discrete Fourier transforms) and the state-loading harness problem
generator (oracle/harness/load_state.cpp, which turns on the turbulence driver with
<problem> turb_flag as the reference's turb problem generator does). Each case runs the
reference on a seeded smooth state and stores input, output and parameters (FP64) as
compressed .npz. Needs the reference source tree (development container only).

    python tests/golden/make_fft_golden.py
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
import oracle_lib as ol  # noqa: E402

WORK = os.path.join(ROOT, "_work", "golden_runs")
N = (16, 16, 16)
MB = (8, 8, 8)
DOMAIN = ((0.0, 1.0), (0.0, 1.0), (0.0, 1.0))

# name: (exe config, mhd, seed, nlim, turbulence parameters or None, four_pi_G or None)
CASES = {
    # decaying turbulence: one drive in Mesh::Initialize (mesh/mesh.cpp:1383-1384)
    "fft_turb_decay_mhd": ("turb_state_mhd_hlld", True, 4, 0,
                           dict(turb_flag=1, dedt=0.5, rseed=17, nlow=0, nhigh=6,
                                f_shear=0.3, expo=2.0), None),
    "fft_turb_decay_hydro": ("turb_state_hydro_hllc", False, 5, 0,
                             dict(turb_flag=1, dedt=0.5, rseed=23, nlow=0, nhigh=6,
                                  f_shear=-1.0, expo=2.0), None),
    # continuous driving: a drive before each of three cycles (main.cpp:457), OU smoothing
    "fft_turb_cont_hydro": ("turb_state_hydro_hllc", False, 9, 3,
                            dict(turb_flag=3, dedt=3.0, rseed=5, nlow=1, nhigh=5,
                                 f_shear=-1.0, expo=2.0, tcorr=0.05), None),
    # FFT self-gravity: the potential of Mesh::Initialize, and two cycles with the source
    "fft_grav_hydro_init": ("fftgrav_state_hydro_hllc", False, 12, 0, None, 4.0 * np.pi),
    "fft_grav_hydro_2cyc": ("fftgrav_state_hydro_hllc", False, 12, 2, None, 4.0 * np.pi),
}


def make_case(name, spec):
    cfg, mhd, seed, nlim, turb, fpg = spec
    exe = build_ref.build(cfg)
    u, b1, b2, b3 = ol.smooth_random_state(N, mhd, seed=seed)
    extra = ""
    if turb is not None:
        extra += "turb_flag = %d\n<turbulence>\n" % turb["turb_flag"]
        for k, v in turb.items():
            if k != "turb_flag":
                extra += "%s = %r\n" % (k, v)
    if fpg is not None:
        extra += "four_pi_G = %r\n" % fpg
    out = ol.run_reference_state(exe, os.path.join(WORK, name), N, MB, mhd, u, b1, b2, b3,
                                 cfl=0.3, tlim=100.0, nlim=nlim, extra=extra,
                                 domain=DOMAIN, phi=fpg is not None)
    arrays = {"u_in": u, "u_out": out["u"]}
    if mhd:
        arrays.update(b1_in=b1, b2_in=b2, b3_in=b3, b1_out=out["b1"], b2_out=out["b2"],
                      b3_out=out["b3"])
    if fpg is not None:
        arrays["phi"] = out["phi"]
    meta = dict(mhd=mhd, solver="hlld" if mhd else "hllc", nx=list(N), meshblock=list(MB),
                seed=seed, nlim=nlim, cfl=0.3, gamma=5.0 / 3.0, turb=turb, four_pi_G=fpg,
                time=out["time"], dt=out["dt"], ncycle=out["ncycle"])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), meta=json.dumps(meta), **arrays)
    print("wrote", name, "t=%.6g ncycle=%d" % (out["time"], out["ncycle"]))


if __name__ == "__main__":
    if not build_ref.available():
        sys.exit("reference tree not present")
    for name in (sys.argv[1:] or list(CASES)):
        make_case(name, CASES[name])

#!/usr/bin/env python3
"""Restart fixture made by the unmodified reference (development container only).

Runs the reference's own Orszag-Tang problem generator (3-D, 16^3 in 8 blocks of 8^3, PLM +
HLLD + VL2) for 2 cycles and keeps its restart file, then restarts the reference from that
file to cycle 5 and keeps the state it reaches. The GPU tests restart the C++ host
(athg_run) from the first file and compare with the second.

    python tests/golden/make_rst_golden.py
"""
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import build_ref  # noqa: E402
import rst_lib  # noqa: E402

WORK = os.path.join(ROOT, "_work", "golden_rst")

ATHINPUT = """<job>
problem_id = OrszagTang
<output1>
file_type = rst
dt = 100.0
<time>
cfl_number = 0.4
nlim = {nlim}
tlim = 1.0
integrator = vl2
xorder = 2
ncycle_out = 100
<mesh>
nx1 = 16
x1min = -0.5
x1max = 0.5
ix1_bc = periodic
ox1_bc = periodic
nx2 = 16
x2min = -0.5
x2max = 0.5
ix2_bc = periodic
ox2_bc = periodic
nx3 = 16
x3min = -0.5
x3max = 0.5
ix3_bc = periodic
ox3_bc = periodic
<meshblock>
nx1 = 8
nx2 = 8
nx3 = 8
<hydro>
gamma = 1.666666666666667
"""


def athinput(nlim):
    return ATHINPUT.format(nlim=nlim)


def run(exe, wd, args):
    r = subprocess.run([exe] + args, cwd=wd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])


def main():
    if not build_ref.available():
        print("reference tree not present; nothing to do")
        return
    exe = build_ref.build("ot_mhd_hlld")
    if os.path.isdir(WORK):
        shutil.rmtree(WORK)
    a, b = os.path.join(WORK, "a"), os.path.join(WORK, "b")
    os.makedirs(a)
    os.makedirs(b)
    with open(os.path.join(a, "athinput.ot"), "w") as f:
        f.write(athinput(2))
    run(exe, a, ["-i", "athinput.ot"])
    shutil.copy(os.path.join(a, "OrszagTang.final.rst"), os.path.join(b, "start.rst"))
    run(exe, b, ["-r", "start.rst", "time/nlim=5"])
    start = open(os.path.join(b, "start.rst"), "rb").read()
    end = rst_lib.read_rst(os.path.join(b, "OrszagTang.final.rst"), (8, 8, 8), 2, True)
    arrays = {"start_rst": np.frombuffer(start, dtype=np.uint8),
              "end_blocks": np.array(end["blocks"], dtype=np.int64),
              "end_time": np.array([end["time"], end["dt"], end["ncycle"]])}
    for k in ("u", "b1", "b2", "b3"):
        arrays["end_" + k] = np.stack([d[k] for d in end["arrays"]])
    np.savez_compressed(os.path.join(HERE, "rst_ot_mhd_16.npz"), **arrays)
    print("wrote rst_ot_mhd_16 (cycle 2 -> 5, t=%.6g)" % end["time"])


if __name__ == "__main__":
    main()

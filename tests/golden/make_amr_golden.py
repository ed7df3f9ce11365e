#!/usr/bin/env python3
"""Adaptive mesh refinement fixtures made by the unmodified reference (development container
only): the reference's own blast problem generator and refinement criterion
(pgen/blast.cpp) with <mesh> refinement = adaptive, run from tests/amr_golden.py's input.
Kept: the block list of every restart dump and the final state (tests/amr_golden.py).

    python tests/golden/make_amr_golden.py
"""
import glob
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import amr_golden  # noqa: E402
import build_ref  # noqa: E402
import rst_lib  # noqa: E402

WORK = os.path.join(ROOT, "_work", "golden_amr")


def make(name):
    exe_name, ng, mhd, _, _, _, _, full = amr_golden.CASES[name][:8]
    bnx = amr_golden.block_nx(name)
    exe = build_ref.build(exe_name)
    wd = os.path.join(WORK, name)
    if os.path.isdir(wd):
        shutil.rmtree(wd)
    os.makedirs(wd)
    with open(os.path.join(wd, "athinput"), "w") as f:
        f.write(amr_golden.athinput(name))
    r = subprocess.run([exe, "-i", "athinput"], cwd=wd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
    dumps = sorted(glob.glob(os.path.join(wd, "Blast.[0-9]*.rst")))
    out = {"dump_ncycle": [], "dump_time": [], "dump_nblocks": [], "dump_blocks": []}
    for d in dumps:
        rst = rst_lib.read_rst(d, bnx, ng, mhd)
        out["dump_ncycle"].append(rst["ncycle"])
        out["dump_time"].append(rst["time"])
        out["dump_nblocks"].append(len(rst["blocks"]))
        out["dump_blocks"].extend(rst["blocks"])
    out = {k: np.asarray(v) for k, v in out.items()}
    fin = rst_lib.read_rst(os.path.join(wd, "Blast.final.rst"), bnx, ng, mhd)
    out["final_blocks"] = np.asarray(fin["blocks"], dtype=np.int64)
    out["final_time"] = np.float64(fin["time"])
    out["final_dt"] = np.float64(fin["dt"])
    out["final_ncycle"] = np.int64(fin["ncycle"])
    for k, v in amr_golden.summarize(fin, ng, mhd, full, bnx).items():
        out[k] = v
    # the same run with history sums every 0.002 at full precision
    with open(os.path.join(wd, "athinput.hst"), "w") as f:
        f.write(amr_golden.athinput_history(name))
    r = subprocess.run([exe, "-i", "athinput.hst"], cwd=wd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
    out["hst"] = np.loadtxt(os.path.join(wd, "Blast.hst"))
    np.savez_compressed(amr_golden.path(name), **out)
    shutil.rmtree(wd)  # the dumps hold every block with ghosts: hundreds of MB
    print(name, "dumps", len(dumps), "final blocks", len(fin["blocks"]),
          "size", os.path.getsize(amr_golden.path(name)))


def main():
    if not build_ref.available():
        print("reference tree not present; nothing to do")
        return
    for name in (sys.argv[1:] or list(amr_golden.CASES)):
        make(name)


if __name__ == "__main__":
    main()

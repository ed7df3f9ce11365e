"""The host-side refinement code under AddressSanitizer and UBSan on 8^3 blocks with two
ghost layers, the smallest blocks refinement allows with that ghost width:

* the level-boundary cell functions of athg_smr.h, which the device kernels run too,
  through the CPU SMR checker (smr_check.cpp) on a three-level MHD mesh (ghost fill,
  restriction, prolongation of cells and shared faces);
* the adaptive block fill (amr_fill) through amr_fill_check.cpp: refinement to three
  levels, refinement at the root level and derefinement.

Skipped where g++ cannot build with -fsanitize=address."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import smr_lib

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "athena-gamma_gb300", "csrc")
FLAGS = ["-std=c++17", "-O1", "-g", "-fsanitize=address,undefined", "-fno-omit-frame-pointer",
         "-fno-sanitize-recover=all", "-ffp-contract=off", "-I", CSRC]


def build(tmp, name, sources):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = os.path.join(tmp, name)
    r = subprocess.run([gxx] + FLAGS + ["-o", exe] + sources, capture_output=True, text=True)
    if r.returncode != 0:
        pytest.skip("no sanitizer build: " + r.stderr.strip().splitlines()[-1][:200])
    return exe


def clean(r):
    assert r.returncode == 0, r.stdout + r.stderr[-3000:]
    assert "ERROR: AddressSanitizer" not in r.stderr and "runtime error" not in r.stderr, r.stderr


@pytest.mark.parametrize("mhd", [True, False])
def test_level_boundaries_three_levels_ng2(tmp_path, mhd):
    exe = build(str(tmp_path), "smr_check", [os.path.join(HERE, "smr_check.cpp"),
                                            os.path.join(CSRC, "athg_smr_plan.cpp")])
    root, mb, dom = (32, 32, 32), (8, 8, 8), ((-1.0, 1.0),) * 3
    regions = [(-0.5, 0.5, -0.5, 0.5, -0.5, 0.5, 1), (-0.2, 0.2, -0.2, 0.2, -0.2, 0.2, 2)]
    blocks = smr_lib.smr_blocks(root, mb, dom, regions)
    st = smr_lib.smr_initial_state(blocks, root, mb, dom, mhd, gamma=5 / 3, seed=3)
    floor = float(np.sqrt(1024 * np.finfo(np.float32).tiny))
    inp, out = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    smr_lib.write_check_in(inp, blocks, st, root, mb, 2, dom, mhd, 5 / 3, floor, floor)
    clean(subprocess.run([exe, inp, out], capture_output=True, text=True, timeout=600))


def test_adaptive_fill_ng2(tmp_path):
    exe = build(str(tmp_path), "amr_fill_check", [
        os.path.join(HERE, "amr_fill_check.cpp"), os.path.join(CSRC, "athg_amr.cpp"),
        os.path.join(CSRC, "athg_smr_plan.cpp")])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    clean(r)
    assert "120 -> 176 blocks (levels 56 56 64)" in r.stdout
    assert "183 -> 127 blocks (levels 55 72 0)" in r.stdout


@pytest.mark.parametrize("mhd,nseq", [(True, 2), (False, 1)])
def test_adaptive_lists_random_sequences_ng2(tmp_path, mhd, nseq):
    """Every level-boundary work list (ghost fill, restriction, prolongation of cells and
    faces, internal field, flux and EMF correction) after every regrid of random adaptive
    sequences on a 32^3 root of 8^3 blocks with two ghost layers, up to three levels: run
    on host arrays with the device's allocation sizes under the sanitizers, and every
    entry's block and element indices checked against one block's extent."""
    exe = build(str(tmp_path), "amr_lists_check", [
        os.path.join(HERE, "amr_lists_check.cpp"), os.path.join(CSRC, "athg_amr.cpp"),
        os.path.join(CSRC, "athg_smr_plan.cpp")])
    r = subprocess.run([exe, "8", "2", "32", "2", str(nseq), "7", "1" if mhd else "0"],
                       capture_output=True, text=True, timeout=900)
    clean(r)
    last = r.stdout.strip().splitlines()[-1]
    assert last == "checked %d meshes" % (7 * nseq), r.stdout[-2000:]
    # the sequences reach the third level and derefine
    assert "levels 0 4" in r.stdout

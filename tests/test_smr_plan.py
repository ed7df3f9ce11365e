"""SMR work lists on the CPU against the reference (no GPU).

tests/smr_check.cpp runs the planner of athena-gamma_gb300/csrc/athg_smr_plan.cpp and the
per-element arithmetic of athg_smr.h (the same code the CUDA kernels run) on host arrays:
ghost fill across levels, coarse buffers, prolongation of cells and face fields, W(U).
The result, every ghost zone included, must equal the reference's state after
Mesh::Initialize on the same two-level mesh bit for bit."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
import smr_golden  # noqa: E402
import smr_lib as sl  # noqa: E402

CSRC = os.path.join(ROOT, "athena-gamma_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("smr") / "smr_check")
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-I", CSRC, "-o", exe,
                        os.path.join(HERE, "smr_check.cpp"),
                        os.path.join(CSRC, "athg_smr_plan.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.mark.parametrize("name", ["smr_mhd_hlld_plm_vl2", "smr_hydro_hllc_plm_vl2"])
def test_initialized_state_matches_reference(checker, tmp_path, name):
    meta, blocks, arrs = smr_golden.load(name)
    st = smr_golden.states_in(meta, blocks, arrs)
    mhd, ng, mb, root = meta["mhd"], meta["nghost"], meta["meshblock"], meta["root"]
    dom = meta["domain"]
    floor = float(np.sqrt(1024 * np.finfo(np.float32).tiny))
    fin, fout = str(tmp_path / "in.bin"), str(tmp_path / "out.bin")
    sl.write_check_in(fin, blocks, st, root, mb, ng, dom, mhd, meta["gamma"], floor, floor)
    r = subprocess.run([checker, fin, fout], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got, sizes = sl.read_check_out(fout, blocks, mb, ng, mhd)
    assert sizes[0] > 0 and sizes[5] > 0  # ghost fill and prolongation happened
    keys = ("u", "w", "b1", "b2", "b3") if mhd else ("u", "w")
    for q, b in enumerate(blocks):
        for k in keys:
            np.testing.assert_array_equal(got[b][k], arrs[k + "_init"][q], err_msg="%s %s" % (b, k))


def test_block_list_matches_reference_tree():
    """The fixture's leaves (from the reference's own mesh) are the ones tests/smr_lib.py
    derives from the refinement regions."""
    for name in smr_golden.CASES:
        meta, blocks, _ = smr_golden.load(name)
        got = sl.smr_blocks(meta["root"], meta["meshblock"], meta["domain"], meta["regions"])
        assert got == blocks

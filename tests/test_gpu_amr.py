"""Adaptive mesh refinement on the GPU against the reference (fixtures made by running the
reference's blast wave with <mesh> refinement = adaptive, tests/golden/make_amr_golden.py).

The C++ host athg_run runs the same input: the initial refinement loop (problem generator
re-run on every refined mesh), then cycles with a refinement check and regrid after each.
Checked: the block list of every restart dump (refinement and derefinement happen along
the way), the final time, dt and cycle, and the final state of every block to round-off."""
import glob
import os
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "athena-gamma_gb300"))
sys.path.insert(0, HERE)
import amr_golden  # noqa: E402
import rst_lib  # noqa: E402

pytestmark = pytest.mark.gpu


def run_host(name, wd):
    import __graft_entry__ as g
    exe = g.build_driver()
    inp = os.path.join(wd, "athinput")
    with open(inp, "w") as f:
        f.write(amr_golden.athinput(name, host=True))
    r = subprocess.run([exe, "-i", inp], cwd=wd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    return r


@pytest.mark.parametrize("name", list(amr_golden.CASES))
def test_adaptive_blast_matches_reference(name, tmp_path):
    _, ng, mhd, _, _, _, _, full, _, _ = amr_golden.CASES[name]
    bnx = amr_golden.block_nx(name)
    ref = amr_golden.load(name)
    run_host(name, str(tmp_path))
    dumps = sorted(glob.glob(os.path.join(str(tmp_path), "Blast.[0-9]*.rst")))
    assert len(dumps) == len(ref["dump_ncycle"])
    off = 0
    for q, d in enumerate(dumps):
        rst = rst_lib.read_rst(d, bnx, ng, mhd)
        nb = int(ref["dump_nblocks"][q])
        assert rst["ncycle"] == ref["dump_ncycle"][q], d
        # same leaves in the same (tree) order
        assert [tuple(b) for b in rst["blocks"]] == \
            [tuple(int(x) for x in b) for b in ref["dump_blocks"][off:off + nb]], d
        off += nb
    fin = rst_lib.read_rst(os.path.join(str(tmp_path), "Blast.final.rst"), bnx,
                           ng, mhd)
    assert fin["ncycle"] == ref["final_ncycle"]
    assert [tuple(b) for b in fin["blocks"]] == [tuple(int(x) for x in b) for b in ref["final_blocks"]]
    assert abs(fin["time"] - ref["final_time"]) <= 1e-13 * ref["final_time"]
    assert abs(fin["dt"] - ref["final_dt"]) <= 1e-12 * ref["final_dt"]
    got = amr_golden.summarize(fin, ng, mhd, full, bnx)
    for k in amr_golden.keys(mhd):
        r = ref[k]
        # FP64 in the reference's operation order: agreement to round-off
        np.testing.assert_allclose(got[k], r, rtol=0, atol=1e-12 * max(1.0, np.abs(r).max()),
                                   err_msg=k)


def test_adaptive_blast_conserves(tmp_path):
    """Regrids keep mass, momentum and total energy of the periodic box: prolongation and
    restriction of the conserved variables conserve them, and fine fluxes replace coarse
    ones at level boundaries."""
    import __graft_entry__ as g
    exe = g.build_driver()
    name = "amr_mhd_hlld_plm_vl2"
    inp = os.path.join(str(tmp_path), "athinput")
    with open(inp, "w") as f:
        f.write(amr_golden.athinput(name, host=True))
    r = subprocess.run([exe, "-i", inp, "output1/dt=-1", "output2/file_type=hst",
                        "output2/dt=0.002"], cwd=str(tmp_path), capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    rows = np.loadtxt(os.path.join(str(tmp_path), "Blast.hst"))
    assert len(rows) > 10
    for col in (2, 3, 4, 5, 9):  # mass, momenta, total energy
        ref = rows[0, col]
        np.testing.assert_allclose(rows[:, col], ref, rtol=0, atol=1e-13 * max(1.0, abs(rows[:, 9]).max()))

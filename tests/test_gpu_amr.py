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
    _, ng, mhd, _, _, _, _, full = amr_golden.CASES[name][:8]
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


@pytest.mark.parametrize("name", list(amr_golden.CASES))
def test_adaptive_blast_history_matches_reference(name, tmp_path):
    """History sums every 0.002 of time: mass and momenta are conserved to round-off by
    regrids and level boundaries alike (the reference drifts by 3e-11 in mass over this run
    and loses 3e-6 of energy to floors in new blocks, and so does this run)."""
    import __graft_entry__ as g
    exe = g.build_driver()
    mhd = amr_golden.CASES[name][2]
    inp = os.path.join(str(tmp_path), "athinput")
    with open(inp, "w") as f:
        f.write(amr_golden.athinput_history(name, host=True))
    r = subprocess.run([exe, "-i", inp], cwd=str(tmp_path), capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-3000:] + r.stderr[-3000:]
    got = np.loadtxt(os.path.join(str(tmp_path), "Blast.hst"))
    ref = amr_golden.load(name)["hst"]
    rc, hc = amr_golden.history_columns(mhd)
    assert got.shape[0] == ref.shape[0]
    # sums over ~10^5-10^6 cells in another order, of states that agree to round-off
    scale = np.abs(ref[:, rc]).max(axis=0)
    np.testing.assert_allclose(got[:, hc], ref[:, rc], rtol=0,
                               atol=1e-11 * np.maximum(scale, 1.0).max())
    # mass and momenta conserved to the reference's own drift
    for c in (2, 3, 4, 5):
        assert np.abs(got[:, c] - got[0, c]).max() <= 1e-10 * max(1.0, abs(got[0, 2]))

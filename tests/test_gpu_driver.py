"""The C++ host program (athena-gamma_gb300/driver/athg_run.cpp) reads an athinput file,
runs cycles through the C ABI and writes history sums; its Orszag-Tang history matches
the same run driven from Python through the same library."""
import os
import subprocess

import numpy as np
import pytest

athg = pytest.importorskip("athg")
import pgens  # noqa: E402

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "athena-gamma_gb300")


def test_driver_orszag_tang_history_matches_python(tmp_path):
    import __graft_entry__ as g
    exe = g.build_driver()
    inp = os.path.join(PKG, "inputs", "athinput.orszag_tang")
    args = [exe, "-i", inp, "mesh/nx1=32", "mesh/nx2=32", "mesh/nx3=32", "meshblock/nx1=16",
            "meshblock/nx2=16", "meshblock/nx3=16", "time/nlim=4", "output1/dt=-1",
            "gb300/precision=fp64"]
    r = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = np.loadtxt(os.path.join(tmp_path, "OrszagTang.hst"))
    final = rows[-1]
    nx = (32, 32, 32)
    u, b1, b2, b3 = pgens.orszag_tang(nx)
    sim = athg.Sim(nx, (16, 16, 16), True, "hlld", precision="fp64", cfl=0.4, tlim=0.5,
                   domain=((-0.5, 0.5),) * 3)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    sim.cycles(4)
    t, dt, _ = sim.get_time()
    h = sim.history()
    sim.close()
    np.testing.assert_allclose(final[0], t, rtol=1e-12)
    np.testing.assert_allclose(final[2:], h, rtol=1e-10, atol=1e-14)
    assert "zone-cycles/wsecond" in r.stdout


def test_driver_blast_runs(tmp_path):
    import __graft_entry__ as g
    exe = g.build_driver()
    inp = os.path.join(PKG, "inputs", "athinput.blast")
    args = [exe, "-i", inp, "mesh/nx1=32", "mesh/nx2=32", "mesh/nx3=32", "meshblock/nx1=16",
            "meshblock/nx2=16", "meshblock/nx3=16", "time/nlim=3"]
    r = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = np.loadtxt(os.path.join(tmp_path, "Blast.hst"))
    assert np.all(np.isfinite(rows))
    # mass and total energy of the periodic box are conserved
    np.testing.assert_allclose(rows[-1][2], rows[0][2], rtol=1e-13)
    np.testing.assert_allclose(rows[-1][9], rows[0][9], rtol=1e-13)

"""The C++ host program (athena-gamma_gb300/driver/athg_run.cpp) reads an athinput file,
runs cycles through the C ABI and writes history sums; its Orszag-Tang history matches
the same run driven from Python through the same library."""
import os
import subprocess

import sys

import numpy as np
import pytest

athg = pytest.importorskip("athg")
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import pgens  # noqa: E402

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "athena-gamma_gb300")


def test_driver_orszag_tang_history_matches_python(tmp_path):
    import __graft_entry__ as g
    exe = g.build_driver()
    inp = os.path.join(PKG, "inputs", "athinput.orszag_tang")
    args = [exe, "-i", inp, "mesh/nx1=32", "mesh/nx2=32", "mesh/nx3=32", "meshblock/nx1=16",
            "meshblock/nx2=16", "meshblock/nx3=16", "time/nlim=4", "output1/dcycle=1",
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
            "meshblock/nx2=16", "meshblock/nx3=16", "time/nlim=3", "output1/dcycle=1"]
    r = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = np.loadtxt(os.path.join(tmp_path, "Blast.hst"))
    assert np.all(np.isfinite(rows))
    # mass and total energy of the periodic box are conserved
    np.testing.assert_allclose(rows[-1][2], rows[0][2], rtol=1e-13)
    np.testing.assert_allclose(rows[-1][9], rows[0][9], rtol=1e-13)


def _rst_fixture(tmp_path):
    z = np.load(os.path.join(ROOT, "tests", "golden", "rst_ot_mhd_16.npz"))
    p = os.path.join(tmp_path, "start.rst")
    z["start_rst"].tofile(p)
    return z, p


def test_driver_restarts_from_reference_file(tmp_path):
    """GPU run continued from a restart file the reference wrote (Orszag-Tang, cycle 2),
    to cycle 5: the restart file it writes holds the state the reference reaches from the
    same file, blocks in the same order."""
    import __graft_entry__ as g
    import rst_lib
    exe = g.build_driver()
    z, start = _rst_fixture(str(tmp_path))
    r = subprocess.run([exe, "-r", start, "time/nlim=5", "gb300/precision=fp64"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = rst_lib.read_rst(os.path.join(tmp_path, "OrszagTang.final.rst"), (8, 8, 8), 2, True)
    assert out["ncycle"] == 5
    assert out["blocks"] == [tuple(b) for b in z["end_blocks"]]
    np.testing.assert_allclose(out["time"], z["end_time"][0], rtol=1e-13)
    for k in ("u", "b1", "b2", "b3"):
        got = np.stack([d[k] for d in out["arrays"]])
        ref = z["end_" + k]
        # FP64 path: round-off agreement with the reference, ghost zones included
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max(), err_msg=k)


def test_driver_restart_file_matches_reference_layout(tmp_path):
    """A fresh GPU run writes a restart file with the reference's header, block order and
    per-block layout; its state after 2 cycles is the reference's to round-off."""
    import __graft_entry__ as g
    import rst_lib
    exe = g.build_driver()
    z, start = _rst_fixture(str(tmp_path))
    ref = rst_lib.read_rst(start, (8, 8, 8), 2, True)
    inp = os.path.join(PKG, "inputs", "athinput.orszag_tang")
    args = [exe, "-i", inp, "mesh/nx1=16", "mesh/nx2=16", "mesh/nx3=16", "meshblock/nx1=8",
            "meshblock/nx2=8", "meshblock/nx3=8", "time/nlim=2", "output1/file_type=rst",
            "output1/dt=100.0", "gb300/precision=fp64"]
    r = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert os.path.exists(os.path.join(tmp_path, "OrszagTang.00000.rst"))
    out = rst_lib.read_rst(os.path.join(tmp_path, "OrszagTang.final.rst"), (8, 8, 8), 2, True)
    assert out["root_level"] == ref["root_level"] and out["region"] == ref["region"]
    assert out["blocks"] == ref["blocks"] and out["ncycle"] == ref["ncycle"] == 2
    np.testing.assert_allclose(out["time"], ref["time"], rtol=1e-13)
    # (the initial states agree to round-off only: the two problem generators place
    # cells with different formulas; z-components are round-off noise of order 1e-17)
    for x, y in zip(out["arrays"], ref["arrays"]):
        for k in x:
            np.testing.assert_allclose(x[k], y[k], rtol=0, atol=1e-12 * max(1.0, np.abs(y[k]).max()))


def test_driver_vtk_output(tmp_path):
    """VTK dumps in the reference's layout (one file per block, big-endian float32)."""
    import __graft_entry__ as g
    exe = g.build_driver()
    inp = os.path.join(PKG, "inputs", "athinput.orszag_tang")
    args = [exe, "-i", inp, "mesh/nx1=16", "mesh/nx2=16", "mesh/nx3=16", "meshblock/nx1=8",
            "meshblock/nx2=8", "meshblock/nx3=8", "time/nlim=1", "output2/file_type=vtk",
            "output2/variable=prim", "output2/dt=100.0", "gb300/precision=fp64"]
    r = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    for b in range(8):
        assert os.path.exists(os.path.join(tmp_path, "OrszagTang.block%d.out2.00000.vtk" % b))
    data = open(os.path.join(tmp_path, "OrszagTang.block0.out2.00000.vtk"), "rb").read()
    assert data.startswith(b"# vtk DataFile Version 2.0\n# Athena++ data at time=")
    assert b"DIMENSIONS 9 9 9\n" in data
    i = data.index(b"SCALARS rho float\nLOOKUP_TABLE default\n") + len(
        b"SCALARS rho float\nLOOKUP_TABLE default\n")
    rho = np.frombuffer(data, dtype=">f4", count=512, offset=i)
    np.testing.assert_allclose(rho, 25.0 / (36.0 * np.pi), rtol=1e-6)
    for tag in (b"SCALARS press float", b"VECTORS vel float", b"VECTORS Bcc float"):
        assert tag in data


def test_driver_refined_blast_restart_is_seamless(tmp_path):
    """Blast with a refined central region from athinput.blast_smr (reduced to a 32^3 root
    grid of 8^3 blocks): mass and energy are conserved across the level boundaries, and a
    run restarted from its own restart file after 2 cycles ends, after 4, bit for bit where
    the uninterrupted run ends (multi-level restart through athg_set_multilevel_blocks)."""
    import __graft_entry__ as g
    import rst_lib
    exe = g.build_driver()
    inp = os.path.join(PKG, "inputs", "athinput.blast_smr")
    small = ["mesh/nx1=32", "mesh/nx2=32", "mesh/nx3=32", "meshblock/nx1=8", "meshblock/nx2=8",
             "meshblock/nx3=8", "output1/dcycle=1", "output2/file_type=rst", "output2/dt=100.0"]
    runs = {}
    for name, extra in (("full", ["time/nlim=4"]), ("half", ["time/nlim=2"])):
        wd = tmp_path / name
        wd.mkdir()
        r = subprocess.run([exe, "-i", inp] + small + extra, cwd=wd, capture_output=True,
                           text=True, timeout=600)
        assert r.returncode == 0, r.stdout + r.stderr
        runs[name] = wd
    rows = np.loadtxt(os.path.join(runs["full"], "Blast.hst"))
    np.testing.assert_allclose(rows[-1][2], rows[0][2], rtol=1e-13)   # mass
    np.testing.assert_allclose(rows[-1][9], rows[0][9], rtol=1e-13)   # total energy
    wd = tmp_path / "resumed"
    wd.mkdir()
    r = subprocess.run([exe, "-r", os.path.join(runs["half"], "Blast.final.rst"), "time/nlim=4"],
                       cwd=wd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    a = rst_lib.read_rst(os.path.join(runs["full"], "Blast.final.rst"), (8, 8, 8), 4, True)
    b = rst_lib.read_rst(os.path.join(wd, "Blast.final.rst"), (8, 8, 8), 4, True)
    assert a["ncycle"] == b["ncycle"] == 4 and a["time"] == b["time"]
    assert a["blocks"] == b["blocks"] and len(a["blocks"]) == 120
    assert sum(1 for bl in a["blocks"] if bl[0] == 1) == 64
    for x, y in zip(a["arrays"], b["arrays"]):
        for k in x:
            np.testing.assert_array_equal(x[k], y[k])


def test_driver_driven_turbulence_injects_dedt(tmp_path):
    """athinput.turb (turb_flag 3, solenoidal forcing): the scheme conserves total energy,
    so the history's total energy grows by exactly dedt * time, with zero net momentum."""
    import __graft_entry__ as g
    exe = g.build_driver()
    inp = os.path.join(PKG, "inputs", "athinput.turb")
    args = [exe, "-i", inp, "mesh/nx1=32", "mesh/nx2=32", "mesh/nx3=32", "meshblock/nx1=16",
            "meshblock/nx2=16", "meshblock/nx3=16", "time/nlim=6", "output1/dt=0.0001"]
    r = subprocess.run(args, cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = np.loadtxt(os.path.join(tmp_path, "Turb.hst"))
    assert len(rows) >= 6
    e0 = rows[0][9]
    np.testing.assert_allclose(rows[:, 9] - e0, 0.1 * rows[:, 0], rtol=1e-10, atol=1e-14)
    assert np.abs(rows[:, 3:6]).max() < 1e-12
    assert rows[-1][6:9].sum() > 0.0  # kinetic energy in the box

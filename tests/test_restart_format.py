"""Restart files of the C++ host (athena-gamma_gb300/driver/athg_io.cpp) against the
reference's own (no GPU).

* The fixture restart file, written by the reference, is read by the numpy reader and by
  athg_io (through tests/rst_tool.cpp), and rewriting it with athg_io reproduces it byte
  for byte apart from the four padding bytes of RegionSize the reference leaves unset.
* Where the reference builds (development container), it restarts from the file athg_io
  wrote and reaches exactly the state it reaches from its own file."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import rst_lib  # noqa: E402

DRIVER = os.path.join(ROOT, "athena-gamma_gb300", "driver")


@pytest.fixture(scope="module")
def tool(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = str(tmp_path_factory.mktemp("rst") / "rst_tool")
    r = subprocess.run([gxx, "-std=c++17", "-O2", "-I", DRIVER, "-o", exe,
                        os.path.join(HERE, "rst_tool.cpp"), os.path.join(DRIVER, "athg_io.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def fixture_rst(tmp_path):
    z = np.load(os.path.join(HERE, "golden", "rst_ot_mhd_16.npz"))
    p = str(tmp_path / "start.rst")
    z["start_rst"].tofile(p)
    return p


def padding_offsets(data):
    end = data.find(b"<par_end>") + 10
    return set(range(end + 8 + 84, end + 8 + 88))


def test_rewrite_matches_reference_file(tool, tmp_path):
    src = fixture_rst(tmp_path)
    out = str(tmp_path / "ours.rst")
    r = subprocess.run([tool, "copy", src, out, "8", "8", "8", "2", "1"], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    a, b = open(src, "rb").read(), open(out, "rb").read()
    assert len(a) == len(b)
    pad = padding_offsets(a)
    diff = [i for i in range(len(a)) if a[i] != b[i] and i not in pad]
    assert diff == []
    ra, rb = rst_lib.read_rst(src, (8, 8, 8), 2, True), rst_lib.read_rst(out, (8, 8, 8), 2, True)
    assert ra["blocks"] == rb["blocks"] and ra["ncycle"] == rb["ncycle"] == 2


def test_info_lists_blocks_in_tree_order(tool, tmp_path):
    src = fixture_rst(tmp_path)
    r = subprocess.run([tool, "info", src, "8", "8", "8", "2", "1"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rows = [tuple(int(v) for v in ln.split()) for ln in r.stdout.splitlines()[1:]]
    ref = rst_lib.read_rst(src, (8, 8, 8), 2, True)["blocks"]
    assert rows == [tuple(b) for b in ref]


def test_reference_restarts_from_our_file(tool, tmp_path):
    import build_ref
    if not build_ref.available():
        pytest.skip("reference tree not present")
    exe = build_ref.build("ot_mhd_hlld")
    src = fixture_rst(tmp_path)
    out = str(tmp_path / "ours.rst")
    subprocess.run([tool, "copy", src, out, "8", "8", "8", "2", "1"], check=True)
    res = {}
    for name, f in (("ours", out), ("ref", src)):
        wd = tmp_path / name
        wd.mkdir()
        shutil.copy(f, wd / "in.rst")
        r = subprocess.run([exe, "-r", "in.rst", "time/nlim=5"], cwd=wd, capture_output=True,
                           text=True)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
        res[name] = rst_lib.read_rst(str(wd / "OrszagTang.final.rst"), (8, 8, 8), 2, True)
    a, b = res["ours"], res["ref"]
    assert a["time"] == b["time"] and a["ncycle"] == b["ncycle"] == 5
    for x, y in zip(a["arrays"], b["arrays"]):
        for k in x:
            np.testing.assert_array_equal(x[k], y[k])

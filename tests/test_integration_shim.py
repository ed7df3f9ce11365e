"""The reference-side binding of INTEGRATION.md (oracle/harness/gb300_shim.cpp) compiled into
the unmodified reference against its own headers and linked with the in-tree library
(oracle/build_ref.py, config shim_mhd_hlld), then run on an Orszag-Tang mesh of 8 blocks.

Without a GPU (this machine) the library's first call fails and the shim reports it through
the reference's ATHENA_ERROR: the run ends cleanly with the library's message. With a GPU
the same binary runs two VL2 cycles on the device and downloads the state. Needs the
reference source tree (skipped elsewhere)."""
import os
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402

INPUT = """<job>
problem_id = shim
<time>
cfl_number = 0.4
nlim = 0
tlim = 1.0
integrator = vl2
xorder = 2
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
gamma = 1.6666666666666667
<problem>
gb300_cycles = 2
"""


def test_shim_builds_against_reference_and_fails_cleanly_without_gpu(tmp_path):
    if not build_ref.available():
        pytest.skip("reference tree not present")
    sys.path.insert(0, ROOT)
    import __graft_entry__ as ge
    ge.build_library()
    exe = build_ref.build("shim_mhd_hlld")
    (tmp_path / "athinput.shim").write_text(INPUT)
    r = subprocess.run([exe, "-i", "athinput.shim"], cwd=tmp_path, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    try:
        import torch
        gpu = torch.cuda.is_available()
    except Exception:  # noqa: BLE001
        gpu = False
    if gpu:
        assert "gb300 shim: 2 cycles" in r.stdout, r.stdout[-2000:]
    else:
        assert "### FATAL ERROR in GB300 stage: no CUDA device available" in r.stdout, \
            r.stdout[-2000:]

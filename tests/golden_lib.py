"""Loading of the golden fixtures made by tests/golden/make_golden.py."""
import glob
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _all():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))


def cases(outflow=True):
    """Stage-update fixtures (hydro/MHD, no gravity); outflow=False leaves out the ones with
    outflow physical boundaries (single-block periodic solvers cannot run them)."""
    c = [c for c in _all() if not c.startswith(("mg_", "sg_", "smr", "rst_", "amr", "fft_"))]
    return c if outflow else [x for x in c if not x.endswith("_outflow")]


def sg_cases():
    """Stage-update fixtures with multigrid self-gravity."""
    return [c for c in _all() if c.startswith("sg_")]


def mg_cases():
    """Multigrid fixtures."""
    return [c for c in _all() if c.startswith("mg_")]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(z["meta"]))
    arr = {k: z[k] for k in z.files if k != "meta"}
    return meta, arr


def linear_wave_errors():
    with open(os.path.join(GOLDEN, "linear_wave_errors.json")) as f:
        return json.load(f)

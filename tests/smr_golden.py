"""Loader of the SMR golden fixtures (tests/golden/smr_*.npz and smr3_*.npz (three levels),
made by tests/golden/make_smr_golden.py from the reference)."""
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CASES = ["smr_mhd_hlld_plm_vl2", "smr_hydro_hllc_plm_vl2", "smr_mhd_hlld_ppm_rk3",
         "smr3_mhd_hlld_plm_vl2"]


def load(name):
    z = np.load(os.path.join(HERE, "golden", name + ".npz"))
    meta = json.loads(str(z["meta"]))
    blocks = [tuple(int(v) for v in b) for b in z["blocks"]]
    arrs = {k: z[k] for k in z.files if k not in ("meta", "blocks")}
    return meta, blocks, arrs


def states_in(meta, blocks, arrs):
    """dict block -> (u, b1, b2, b3) interior input state"""
    out = {}
    for q, b in enumerate(blocks):
        if meta["mhd"]:
            out[b] = (arrs["u_in"][q], arrs["b1_in"][q], arrs["b2_in"][q], arrs["b3_in"][q])
        else:
            out[b] = (arrs["u_in"][q], None, None, None)
    return out

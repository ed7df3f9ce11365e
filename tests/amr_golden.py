"""Adaptive mesh refinement fixtures (test infrastructure): the reference's blast wave with
<mesh> refinement = adaptive on a 16^3 root mesh of 4^3 MeshBlocks (32^3 of 8^3 with four
ghost cells), two levels (and one case with three), run by the unmodified reference (tests/golden/make_amr_golden.py)
and by the C++ host athg_run.

Each fixture holds the block list of every restart dump (one per 0.01 of time), of the
final dump its time, dt and cycle and the interior of every block (all of U and of the face
fields; or, for `full=False`, per-block sums and sums of squares of each array), and the
history sums of the same run every 0.002 of time."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

# name -> reference build, nghost, mhd, Riemann solver, integrator, xorder, nlim, full arrays,
# root cells per axis, block cells per axis, numlevel
CASES = {
    "amr_mhd_hlld_plm_vl2": ("blast_mhd_hlld_ng2", 2, True, "hlld", "vl2", 2, 25, True, 16, 4, 2),
    "amr_hydro_hllc_plm_vl2": ("blast_hydro_hllc_ng2", 2, False, "hllc", "vl2", 2, 25, True, 16, 4,
                               2),
    "amr_mhd_hlld_ppm_rk3": ("blast_mhd_hlld", 4, True, "hlld", "rk3", 3, 20, False, 32, 8, 2),
    # three levels (848 -> 960 blocks of 4^3 in 12 cycles)
    "amr3_mhd_hlld_plm_vl2": ("blast_mhd_hlld_ng2", 2, True, "hlld", "vl2", 2, 12, False, 16, 4, 3),
}


def block_nx(name):
    return (CASES[name][9],) * 3


ATHINPUT = """<job>
problem_id = Blast
<output1>
file_type = rst
dt = 0.01
<time>
cfl_number = 0.3
nlim = {nlim}
tlim = 1.0
integrator = {integrator}
xorder = {xorder}
ncycle_out = 100
<mesh>
nx1 = {nroot}
x1min = -1.0
x1max = 1.0
ix1_bc = periodic
ox1_bc = periodic
nx2 = {nroot}
x2min = -1.0
x2max = 1.0
ix2_bc = periodic
ox2_bc = periodic
nx3 = {nroot}
x3min = -1.0
x3max = 1.0
ix3_bc = periodic
ox3_bc = periodic
refinement = adaptive
numlevel = {numlevel}
derefine_count = 3
<meshblock>
nx1 = {nblock}
nx2 = {nblock}
nx3 = {nblock}
<hydro>
gamma = 1.666666666666667
<problem>
pamb = 0.1
prat = 100.
radius = 0.3
b0 = 1.0
angle = 45.0
thr = 0.15
"""

GB300 = """<gb300>
pgen = blast
magnetic = {magnetic}
rsolver = {rsolver}
nghost = {ng}
precision = fp64
"""


def athinput(name, host=False):
    _, ng, mhd, rsolver, integrator, xorder, nlim, _, nroot, nblock, numlevel = CASES[name]
    s = ATHINPUT.format(nlim=nlim, integrator=integrator, xorder=xorder, nroot=nroot,
                        nblock=nblock, numlevel=numlevel)
    if host:
        s += GB300.format(magnetic=int(mhd), rsolver=rsolver, ng=ng)
    return s


def athinput_history(name, host=False):
    """The same run writing history sums every 0.002 (full precision) instead of dumps."""
    s = athinput(name, host).replace("file_type = rst\ndt = 0.01",
                                     "file_type = hst\ndt = 0.002\ndata_format = %.16e")
    assert "file_type = hst" in s
    return s


def history_columns(mhd):
    """Columns of the reference's history file without self-gravity (outputs/history.cpp):
    time, dt, mass, 3 momenta, 3 kinetic energies, total energy, then 3 magnetic energies
    with MHD. The C++ host always writes the gravitational energy after the total energy."""
    ref = list(range(10)) + ([10, 11, 12] if mhd else [])
    host = list(range(10)) + ([11, 12, 13] if mhd else [])
    return ref, host


def keys(mhd):
    return ("u", "b1", "b2", "b3") if mhd else ("u",)


def interior(arrs, ng, mhd, bnx):
    """Interior cells (and interior faces, both ends included) of one block's arrays."""
    n1, n2, n3 = bnx
    c = (slice(ng, ng + n3), slice(ng, ng + n2), slice(ng, ng + n1))
    out = {"u": arrs["u"][(slice(None),) + c]}
    if mhd:
        out["b1"] = arrs["b1"][ng:ng + n3, ng:ng + n2, ng:ng + n1 + 1]
        out["b2"] = arrs["b2"][ng:ng + n3, ng:ng + n2 + 1, ng:ng + n1]
        out["b3"] = arrs["b3"][ng:ng + n3 + 1, ng:ng + n2, ng:ng + n1]
    return out


def moments(a):
    """Per-block sum and sum of squares of every variable of one interior array."""
    a = np.asarray(a, dtype=np.float64)
    if a.ndim == 4:
        return np.stack([a.reshape(a.shape[0], -1).sum(1), (a.reshape(a.shape[0], -1) ** 2).sum(1)], 1)
    return np.array([[a.sum(), (a ** 2).sum()]])


def summarize(rst, ng, mhd, full, bnx):
    """Fixture arrays of the final dump: interior arrays (full) or their moments, stacked
    over the blocks in the dump's order."""
    out = {}
    for k in keys(mhd):
        per = [interior(a, ng, mhd, bnx)[k] for a in rst["arrays"]]
        out[k] = np.stack(per) if full else np.stack([moments(x) for x in per])
    return out


def path(name):
    return os.path.join(GOLDEN, name + ".npz")


def load(name):
    z = np.load(path(name), allow_pickle=False)
    return {k: z[k] for k in z.files}

"""Static mesh refinement on the GPU against the reference (golden fixtures made by running
the reference on two-level periodic meshes, tests/golden/make_smr_golden.py).

Checked: the leaves of athg_set_refined_mesh, the state after athg_initialize with every
ghost zone (ghost fill across levels, prolongation of cells and face fields, W(U)) bit for
bit, the state after several cycles (flux and EMF correction at level boundaries included),
and conservation and div B over a longer run."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "athena-gamma_gb300"))
sys.path.insert(0, HERE)
import athg  # noqa: E402
import smr_golden  # noqa: E402

pytestmark = pytest.mark.gpu


def make_sim(meta, tlim=100.0, precision="fp64"):
    # (x1min, x1max, x2min, x2max, x3min, x3max[, level]), level 1 by default
    regions = [tuple(r) if len(r) > 6 else tuple(r) + (1,) for r in meta["regions"]]
    return athg.Sim(tuple(meta["root"]), tuple(meta["meshblock"]), meta["mhd"], meta["solver"],
                    precision=precision, xorder=meta["xorder"], integrator=meta["integrator"],
                    gamma=meta["gamma"], cfl=meta["cfl"], tlim=tlim, ng=meta["nghost"],
                    domain=tuple(tuple(x) for x in meta["domain"]), regions=regions)


@pytest.mark.parametrize("name", smr_golden.CASES)
def test_refined_mesh_leaves(name):
    meta, blocks, _ = smr_golden.load(name)
    sim = make_sim(meta)
    assert sorted(sim.leaves) == blocks
    st = sim.smr_stats()
    assert st[0] > 0 and st[2] > 0 and st[5] > 0
    if meta["mhd"]:
        assert st[3] > 0
    sim.close()


@pytest.mark.parametrize("name", ["smr_mhd_hlld_plm_vl2", "smr_hydro_hllc_plm_vl2"])
def test_initialize_matches_reference(name):
    meta, blocks, arrs = smr_golden.load(name)
    sim = make_sim(meta)
    sim.load_blocks(smr_golden.states_in(meta, blocks, arrs))
    sim.initialize()
    got = sim.blocks(ghosts=True)
    keys = ("u", "w", "b1", "b2", "b3") if meta["mhd"] else ("u", "w")
    for q, b in enumerate(blocks):
        for k in keys:
            np.testing.assert_array_equal(got[b][k], arrs[k + "_init"][q], err_msg="%s %s" % (b, k))
    sim.close()


@pytest.mark.parametrize("name", smr_golden.CASES)
def test_cycles_match_reference(name):
    meta, blocks, arrs = smr_golden.load(name)
    sim = make_sim(meta)
    sim.load_blocks(smr_golden.states_in(meta, blocks, arrs))
    sim.initialize()
    sim.cycles(meta["ncycles"])
    t, dt, nc = sim.get_time()
    assert nc == meta["ncycle"]
    assert abs(t - meta["time"]) <= 1e-14 * abs(meta["time"])
    got = sim.blocks(ghosts=False)
    keys = ("u", "b1", "b2", "b3") if meta["mhd"] else ("u",)
    for k in keys:
        ref = arrs[k + "_out"]
        g = np.stack([got[b][k] for b in blocks])
        # FP64 with the reference's operation order: agreement to round-off
        np.testing.assert_allclose(g, ref, rtol=0, atol=1e-12 * np.abs(ref).max(), err_msg=k)
    sim.close()


def test_conservation_and_div_b():
    """Periodic two-level mesh: mass, momentum and energy are conserved to round-off
    (fine fluxes replace coarse ones at level boundaries), and CT with EMF correction keeps
    div B at round-off."""
    meta, blocks, arrs = smr_golden.load("smr_mhd_hlld_plm_vl2")
    sim = make_sim(meta)
    sim.load_blocks(smr_golden.states_in(meta, blocks, arrs))
    sim.initialize()
    s0 = sim.sum_conserved()
    d0 = sim.max_div_b()
    sim.cycles(20)
    s1 = sim.sum_conserved()
    d1 = sim.max_div_b()
    assert d0 < 1e-12 and d1 < 1e-12, (d0, d1)
    assert np.all(np.abs(s1 - s0) <= 1e-13 * np.maximum(1.0, np.abs(s0))), s1 - s0
    sim.close()


@pytest.mark.parametrize("name", smr_golden.CASES)
def test_mixed_close_to_reference(name):
    """Mixed precision on the two-level meshes (FP32 fluxes and EMFs with their level-boundary
    corrections, FP64 state, ghost fill and prolongation) against the reference after the
    same cycles. PLM: the uniform mixed path's 1e-5 (mixed and FP64 agree to ~1e-7 here).
    PPM: 3e-4, because fine blocks hold prolongated, piecewise-linear data whose second
    differences are zero in FP64 but +-rounding in FP32, and PPM's extremum tests
    (reconstruct/ppm.cpp:150-230) branch on their signs; the difference appears in the first
    cycle inside fine blocks, not at level boundaries."""
    meta, blocks, arrs = smr_golden.load(name)
    sim = make_sim(meta, precision="mixed")
    sim.load_blocks(smr_golden.states_in(meta, blocks, arrs))
    sim.initialize()
    sim.cycles(meta["ncycles"])
    _, _, nc = sim.get_time()
    assert nc == meta["ncycle"]
    got = sim.blocks(ghosts=False)
    tol = 3e-4 if meta["xorder"] == 3 else 1e-5
    for k in (("u", "b1", "b2", "b3") if meta["mhd"] else ("u",)):
        ref = arrs[k + "_out"]
        g = np.stack([got[b][k] for b in blocks])
        err = np.abs(g - ref).max() / np.abs(ref).max()
        assert err < tol, (k, err)
    sim.close()


def test_mixed_conservation_and_div_b():
    """Mixed precision: div B stays at round-off (CT in FP64 with the corrected FP32 EMFs);
    mass and energy change only by the FP32 rounding of the coarse-face fluxes that replace
    the fine ones at level boundaries (2^-24 of the boundary flux per step)."""
    meta, blocks, arrs = smr_golden.load("smr_mhd_hlld_plm_vl2")
    sim = make_sim(meta, precision="mixed")
    sim.load_blocks(smr_golden.states_in(meta, blocks, arrs))
    sim.initialize()
    s0 = sim.sum_conserved()
    sim.cycles(20)
    s1 = sim.sum_conserved()
    assert sim.max_div_b() < 1e-12
    rel = np.abs(s1 - s0) / np.maximum(1.0, np.abs(s0))
    assert np.all(rel < 1e-7), rel
    sim.close()


def test_adaptive_mixed_rejected():
    """Adaptive refinement stays on the FP64 path (the reference's precision)."""
    meta, blocks, arrs = smr_golden.load("smr_hydro_hllc_plm_vl2")
    sim = make_sim(meta, precision="mixed")
    with pytest.raises(athg.AthgError):
        sim.amr_enable(0.1, 1)
    sim.close()

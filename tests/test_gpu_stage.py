"""CUDA stage update against the reference (golden fixtures) and the oracle.

FP64 path: bitwise identical to the reference's FP64 CPU solver (same operations in the
same order; the FP64 kernels are compiled without FMA contraction).
Mixed path (FP32 reconstruction/Riemann fluxes, FP64 state and CT): within the
tolerances stated per test.
"""
import json

import numpy as np
import pytest

import golden_lib
import oracle_lib as ol
import pgens as pgen_lw

pytestmark = pytest.mark.gpu

athg = pytest.importorskip("athg")


def _sim_for(meta, precision):
    per = 0 if meta.get("bc") == "outflow" else 1
    return athg.Sim(tuple(meta["nx"]), tuple(meta["meshblock"]), mhd=meta["mhd"],
                    solver=meta["solver"], precision=precision, xorder=meta["xorder"],
                    integrator=meta["integrator"], cfl=meta["cfl"], gamma=meta["gamma"],
                    tlim=100.0, ng=meta.get("nghost", 2), periodic=(per, per, per))


def _run_case(name, precision, use_graph=True):
    meta, a = golden_lib.load(name)
    sim = _sim_for(meta, precision)
    sim.load_interior(a["u_in"], a.get("b1_in"), a.get("b2_in"), a.get("b3_in"))
    sim.initialize()
    if use_graph:
        sim.cycles(meta["ncycles"])
    else:
        nst = {"vl2": 2, "rk1": 1, "rk2": 2, "rk3": 3}[meta["integrator"]]
        for _ in range(meta["ncycles"]):
            for s in range(1, nst + 1):
                sim.stage(s)
            sim.end_cycle()
    out = sim.interior()
    t, dt, n = sim.get_time()
    return meta, a, out, (t, dt, n)


@pytest.mark.parametrize("name", golden_lib.cases())
def test_fp64_bitexact_vs_reference(name):
    meta, a, out, (t, dt, n) = _run_case(name, "fp64")
    assert n == meta["ncycle"]
    assert t == meta["time"] and dt == meta["dt"]
    for k in (["u"] + (["b1", "b2", "b3"] if meta["mhd"] else [])):
        ref = a[k + "_out"]
        assert np.array_equal(out[k], ref), (k, float(np.abs(out[k] - ref).max()))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", ["mhd_hlld_plm_vl2", "hydro_hllc_plm_rk3"])
def test_stage_by_stage_equals_graph(name, precision):
    _, _, g1, t1 = _run_case(name, precision, use_graph=True)
    _, _, g2, t2 = _run_case(name, precision, use_graph=False)
    assert t1 == t2
    for k in g1:
        assert np.array_equal(g1[k], g2[k])


@pytest.mark.parametrize("name", golden_lib.cases(outflow=False))
def test_mixed_close_to_reference(name):
    meta, a, out, _ = _run_case(name, "mixed")
    # FP32 fluxes: each stage perturbs U by ~1e-7 of the flux increment; after three
    # cycles the state differs from the FP64 reference at the 1e-6 level. PPM's limiter
    # branches on the signs of second differences (reconstruct/ppm.cpp:150-230), which
    # FP32 rounding of nearly flat data can flip, so PPM cases are held to 2e-5.
    tol = 2e-5 if meta["xorder"] == 3 else 2e-6
    for k in (["u"] + (["b1", "b2", "b3"] if meta["mhd"] else [])):
        ref = a[k + "_out"]
        scale = np.abs(ref).max()
        err = np.abs(out[k] - ref).max() / scale
        assert err < tol, (k, err)


def test_multiblock_matches_single_block_oracle():
    """8 blocks of 16^3 on a 32^3 periodic mesh vs the one-block oracle."""
    nx, mb = (32, 32, 32), (16, 16, 16)
    u, b1, b2, b3 = ol.smooth_random_state(nx, True, seed=31, amp=0.2)
    sim = athg.Sim(nx, mb, mhd=True, solver="hlld", precision="fp64", cfl=0.4, tlim=100.0)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    sim.cycles(4)
    got = sim.interior()
    o = ol.Oracle(nx, True, "hlld", cfl=0.4)
    o.load_interior(u, b1, b2, b3)
    o.initialize(100.0)
    o.cycle(4, 100.0)
    ref = o.interior()
    for k in ("u", "b1", "b2", "b3"):
        np.testing.assert_allclose(got[k], ref[k], rtol=0, atol=1e-12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_div_b_and_conservation(precision):
    nx, mb = (32, 32, 32), (16, 16, 16)
    u, b1, b2, b3 = ol.smooth_random_state(nx, True, seed=5, amp=0.3)
    sim = athg.Sim(nx, mb, mhd=True, solver="hlld", precision=precision, cfl=0.4, tlim=100.0)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    s0 = sim.sum_conserved()
    d0 = sim.max_div_b()
    sim.cycles(10)
    s1 = sim.sum_conserved()
    d1 = sim.max_div_b()
    # CT keeps div B at FP64 round-off of |B| ~ 1 (stated target: <= 1e-13)
    assert d0 < 1e-13 and d1 < 1e-13, (d0, d1)
    # periodic box: mass, momentum and energy conserved to FP64 round-off
    assert np.all(np.abs(s1 - s0) <= 1e-13 * np.maximum(1.0, np.abs(s0))), s1 - s0


@pytest.mark.parametrize("mhd,solver,tlim,cfl,key", [
    (False, "hllc", 1.0, 0.4, "hydro_c1"),
    (True, "hlld", 0.5, 0.3, "mhd_fast"),
])
def test_linear_wave_known_answer(mhd, solver, tlim, cfl, key):
    """The reference's own linear-wave L1 error (linearwave-errors.dat, amplitude 1e-6)
    is reproduced by the FP64 path."""
    ref = golden_lib.linear_wave_errors()[key]
    ref_n, ref_rms = int(ref["values"][3]), ref["values"][4]
    dom = ((0.0, 3.0), (0.0, 1.5), (0.0, 1.5))
    nx = (64, 32, 32)
    lw = pgen_lw.LinearWave(nx, dom, mhd)
    u, b1, b2, b3 = lw.initial_state()
    sim = athg.Sim(nx, nx, mhd=mhd, solver=solver, precision="fp64", cfl=cfl,
                   gamma=1.666666666666667, tlim=tlim, domain=dom)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    n = sim.run(tlim)
    out = sim.interior()
    rms = lw.l1_errors(out["u"], out.get("b1"), out.get("b2"), out.get("b3"))[0]
    assert n == ref_n
    # the reference prints 7 significant digits
    assert abs(rms - ref_rms) <= 5e-7 * ref_rms, (rms, ref_rms)


@pytest.mark.parametrize("mhd,solver,tlim,cfl", [
    (False, "hllc", 1.0, 0.4),
    (True, "hlld", 0.5, 0.3),
])
def test_linear_wave_mixed_equal_l1(mhd, solver, tlim, cfl):
    """Mixed path at equal L1 error: with amplitude 1e-3 the truncation error (~5e-5)
    is far above FP32 resolution, and the mixed path's L1 error is within 2x of the FP64
    path's (stated target). At amplitude 1e-6 the wave itself is near FP32 resolution of
    the unit background (6e-8), so only the FP64 path can resolve it."""
    dom = ((0.0, 3.0), (0.0, 1.5), (0.0, 1.5))
    nx = (64, 32, 32)
    lw = pgen_lw.LinearWave(nx, dom, mhd, amp=1.0e-3)
    u, b1, b2, b3 = lw.initial_state()
    res = {}
    for prec in ("fp64", "mixed"):
        sim = athg.Sim(nx, nx, mhd=mhd, solver=solver, precision=prec, cfl=cfl,
                       gamma=1.666666666666667, tlim=tlim, domain=dom)
        sim.load_interior(u, b1, b2, b3)
        sim.initialize()
        sim.run(tlim)
        out = sim.interior()
        res[prec] = lw.l1_errors(out["u"], out.get("b1"), out.get("b2"), out.get("b3"))[0]
    assert res["mixed"] <= 2.0 * res["fp64"], res


@pytest.mark.parametrize("mhd", [True, False])
def test_fused_mixed_stage_matches_unfused(mhd):
    """The fused mixed VL2 stage (update + interior primitive recovery, FP32 ghost exchange,
    alternating state buffers) against the separate-kernel mixed path on 8 blocks, over
    five cycles run as captured graphs (odd count: the state ends in the other buffer)."""
    nx, mb = (32, 32, 32), (16, 16, 16)
    u, b1, b2, b3 = ol.smooth_random_state(nx, mhd, seed=17, amp=0.3)
    out = {}
    for mode in ("fused", "unfused"):
        sim = athg.Sim(nx, mb, mhd=mhd, solver="hlld" if mhd else "hllc", precision="mixed",
                       cfl=0.4, tlim=100.0)
        sim.load_interior(u, b1, b2, b3)
        sim.initialize()
        if mode == "unfused":
            # any single-step entry point leaves the fused path for good
            athg.check(athg.lib().athg_exchange_ghosts(sim.h))
        sim.cycles(5)
        out[mode] = (sim.interior(), sim.download(athg.VAR_CONS), sim.get_time(),
                     sim.max_div_b() if mhd else 0.0)
        sim.close()
    (fi, fu, ft, fd), (ui, uu, ut, ud) = out["fused"], out["unfused"]
    assert ft == ut
    for k in fi:
        np.testing.assert_allclose(fi[k], ui[k], rtol=0, atol=1e-12 * np.abs(ui[k]).max())
    # the ghost zones of the state (refreshed on download) match as well
    np.testing.assert_allclose(fu, uu, rtol=0, atol=1e-12 * np.abs(uu).max())
    if mhd:
        assert fd < 1e-13


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_history_sums_match_host(precision):
    """Device history reduction (outputs/history.cpp sums) against numpy on the downloaded
    state, after a few cycles (the mixed VL2 path leaves the state in the other buffer)."""
    nx, mb = (32, 32, 32), (16, 16, 16)
    u, b1, b2, b3 = ol.smooth_random_state(nx, True, seed=23, amp=0.3)
    sim = athg.Sim(nx, mb, mhd=True, solver="hlld", precision=precision, cfl=0.4, tlim=100.0)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    sim.cycles(3)
    h = sim.history()
    st = sim.interior()
    U = st["u"]
    vol = (1.0 / 32) ** 3
    c1 = 0.5 * (st["b1"][:, :, :-1] + st["b1"][:, :, 1:])
    c2 = 0.5 * (st["b2"][:, :-1, :] + st["b2"][:, 1:, :])
    c3 = 0.5 * (st["b3"][:-1, :, :] + st["b3"][1:, :, :])
    ref = [U[0].sum(), U[1].sum(), U[2].sum(), U[3].sum(),
           (0.5 * U[1] ** 2 / U[0]).sum(), (0.5 * U[2] ** 2 / U[0]).sum(),
           (0.5 * U[3] ** 2 / U[0]).sum(), U[4].sum(), 0.0,
           (0.5 * c1 ** 2).sum(), (0.5 * c2 ** 2).sum(), (0.5 * c3 ** 2).sum()]
    ref = np.array(ref) * vol
    np.testing.assert_allclose(h, ref, rtol=1e-12, atol=1e-14)
    sim.close()


def test_flux_launch_shape_does_not_change_results():
    """The autotuned launch shape of the flux sweeps (threads per block, marching segment
    length) changes scheduling only: two extreme shapes give bitwise identical states."""
    nx, mb = (32, 32, 32), (16, 16, 16)
    u, b1, b2, b3 = ol.smooth_random_state(nx, True, seed=29, amp=0.3)
    out = []
    for shape in ((64, 64, 4), (128, 128, 0)):
        sim = athg.Sim(nx, mb, mhd=True, solver="hlld", precision="mixed", cfl=0.4, tlim=100.0)
        sim.load_interior(u, b1, b2, b3)
        sim.initialize()
        sim.set_tuning(*shape)
        sim.cycles(3)
        assert sim.tuning() == shape
        out.append(sim.interior())
        sim.close()
    for k in out[0]:
        assert np.array_equal(out[0][k], out[1][k]), k
    # the autotuner picks one of its candidates (for each reconstruction order the
    # integrator uses; the reported shape is the second VL2 stage's)
    sim = athg.Sim(nx, mb, mhd=True, solver="hlld", precision="mixed", cfl=0.4, tlim=100.0)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    sim.cycles(1)
    x1, mt, seg = sim.tuning()
    assert x1 in (64, 128) and mt in (64, 128) and seg in (4, 8, 16, 32, 0)
    sim.close()


def test_mixed_rejects_outflow():
    """Outflow boundaries run on the FP64 arrays (FP64 and double-float paths): the mixed
    path refuses a non-periodic mesh instead of leaving its physical ghost zones stale."""
    with pytest.raises(athg.AthgError):
        athg.Sim((16, 8, 8), (8, 8, 8), mhd=True, solver="hlld", precision="mixed",
                 periodic=(0, 1, 1))


def test_fixed_size_kernels_match_general():
    """Blocks of 64^3 with two ghost layers take fixed-size instantiations of the flux
    sweeps, the corner EMF and the fused update (compile-time strides); other block sizes
    take the general ones.
    The arithmetic per cell is the same, so the mixed path on one mesh split into 64^3
    blocks and into 32^3 blocks agrees to round-off after three cycles."""
    nx = (128, 64, 64)
    u, b1, b2, b3 = ol.smooth_random_state(nx, True, seed=31, amp=0.3)
    out = {}
    for mb in ((64, 64, 64), (32, 32, 32)):
        sim = athg.Sim(nx, mb, mhd=True, solver="hlld", precision="mixed", cfl=0.4,
                       tlim=100.0, domain=((0.0, 2.0), (0.0, 1.0), (0.0, 1.0)))
        sim.load_interior(u, b1, b2, b3)
        sim.initialize()
        sim.cycles(3)
        out[mb] = (sim.interior(), sim.get_time())
        sim.close()
    (a, ta), (c, tc) = out[(64, 64, 64)], out[(32, 32, 32)]
    assert ta == tc
    for k in a:
        np.testing.assert_allclose(a[k], c[k], rtol=0, atol=1e-12 * np.abs(c[k]).max())

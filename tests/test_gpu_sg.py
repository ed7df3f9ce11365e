"""Self-gravity on the GPU (multigrid solve after every stage + the source term of
hydro/srcterms/self_gravity.cpp) against reference runs with SELF_GRAVITY_ENABLED = 2."""
import numpy as np
import pytest

import golden_lib

athg = pytest.importorskip("athg")
pytestmark = pytest.mark.gpu


def run_gpu(meta, a, precision, mg_precision="fp64"):
    n = meta["nx"][0]
    mb = tuple(meta["meshblock"])
    sim = athg.Sim(tuple(meta["nx"]), mb, meta["mhd"], meta["solver"], precision=precision,
                   xorder=meta["xorder"], integrator=meta["integrator"], cfl=meta["cfl"],
                   gamma=meta["gamma"], tlim=100.0)
    mg = athg.Multigrid(n, domain=((0.0, 1.0),) * 3, bc="periodic",
                        mode=meta["mgmode"], niteration=meta["niteration"], threshold=-1.0,
                        precision=mg_precision)
    sim.attach_gravity(mg, meta["four_pi_G"])
    sim.load_interior(a["u_in"], a.get("b1_in"), a.get("b2_in"), a.get("b3_in"))
    sim.initialize()
    sim.cycles(meta["ncycles"])
    out = sim.interior()
    phi = sim.phi()[1:-1, 1:-1, 1:-1]
    t, _, _ = sim.get_time()
    sim.attach_gravity(None, 0.0)
    sim.close()
    mg.close()
    return out, phi, t


@pytest.mark.parametrize("name", golden_lib.sg_cases())
def test_sg_fp64_matches_reference(name):
    meta, a = golden_lib.load(name)
    out, phi, t = run_gpu(meta, a, "fp64")
    assert t == pytest.approx(meta["time"], rel=1e-13)
    # the multigrid's sums (average subtraction, defect norms) run as parallel reductions,
    # so the potential, and the state through it, agree to round-off, not bit for bit
    for k in (["u"] + (["b1", "b2", "b3"] if meta["mhd"] else [])):
        ref = a[k + "_out"]
        np.testing.assert_allclose(out[k], ref, rtol=0, atol=1e-12 * np.abs(ref).max())
    np.testing.assert_allclose(phi, a["phi_out"], rtol=0, atol=1e-11 * np.abs(a["phi_out"]).max())


@pytest.mark.parametrize("name", golden_lib.sg_cases())
def test_sg_mixed_close_to_reference(name):
    meta, a = golden_lib.load(name)
    # mixed hydro (FP32 fluxes and source products) with the FP64 multigrid cycle, whose
    # iterates after a fixed number of V-cycles match the reference's
    out, phi, _ = run_gpu(meta, a, "mixed", "fp64")
    for k in (["u"] + (["b1", "b2", "b3"] if meta["mhd"] else [])):
        ref = a[k + "_out"]
        err = np.abs(out[k] - ref).max() / np.abs(ref).max()
        assert err < 5e-6, (k, err)
    err = np.abs(phi - a["phi_out"]).max() / np.abs(a["phi_out"]).max()
    assert err < 2e-7, err


def test_turbulent_box_mixed_tracks_fp64():
    """The self-gravitating turbulent box (rms Mach 5, beta 1, gamma 1.0001, Jeans number 2)
    at 32^3: the mixed path stays within 1e-5 (L1 of rho) of the FP64 path over 5
    cycles, with div B at round-off."""
    import pgens
    n = 32
    u, b1, b2, b3, fpg, _ = pgens.turbulent_box((n, n, n))
    rho = {}
    for prec in ("fp64", "mixed"):
        sim = athg.Sim((n, n, n), (16, 16, 16), True, "hlld", precision=prec, cfl=0.3,
                       tlim=100.0, gamma=1.0001)
        mg = athg.Multigrid(n, domain=((0.0, 1.0),) * 3, bc="periodic", mode="FMG",
                            threshold=-1.0, niteration=1, precision=prec)
        sim.attach_gravity(mg, fpg)
        sim.load_interior(u, b1, b2, b3)
        sim.initialize()
        sim.cycles(5)
        out = sim.interior()
        assert np.all(np.isfinite(out["u"]))
        assert sim.max_div_b() < 1e-12
        rho[prec] = out["u"][0]
        sim.attach_gravity(None, 0.0)
        sim.close()
        mg.close()
    l1 = np.mean(np.abs(rho["mixed"] - rho["fp64"])) / np.mean(np.abs(rho["fp64"]))
    assert l1 < 1e-5, l1


@pytest.mark.parametrize("mhd", [True, False])
@pytest.mark.parametrize("threshold", [-1.0, 0.0])
def test_fused_mixed_sg_tracks_fp64(mhd, threshold):
    """The fused mixed VL2 stage with the self-gravity source inside the update (potential
    read as FP32 pairs) against the separate-kernel mixed path (k_update, k_self_gravity,
    k_c2p), both measured from the FP64 run, on 8 blocks over five cycles. The two mixed
    paths round the source term differently (by an FP32 ulp), so they agree to the mixed
    path's noise, not bit for bit: the fused one must stay as close to FP64 as the other.
    threshold -1: a fixed cycle count per solve, the cycles run as captured graphs;
    threshold 0: the solve iterates to convergence and the cycles run kernel by kernel.
    Both mixed runs leave the state in the other buffer (odd cycle count)."""
    import oracle_lib as ol
    n, mb = 32, (16, 16, 16)
    u, b1, b2, b3 = ol.smooth_random_state((n, n, n), mhd, seed=29, amp=0.3)
    out = {}
    for mode in ("fp64", "fused", "unfused"):
        sim = athg.Sim((n, n, n), mb, mhd=mhd, solver="hlld" if mhd else "hllc",
                       precision="fp64" if mode == "fp64" else "mixed", cfl=0.4, tlim=100.0)
        mg = athg.Multigrid(n, domain=((0.0, 1.0),) * 3, bc="periodic", mode="FMG",
                            threshold=threshold, niteration=2, precision="fp64")
        sim.attach_gravity(mg, 4.0)
        sim.load_interior(u, b1, b2, b3)
        sim.initialize()
        if mode == "unfused":
            # any single-step entry point leaves the fused path for good
            athg.check(athg.lib().athg_exchange_ghosts(sim.h))
        sim.cycles(5)
        out[mode] = (sim.interior(), sim.phi(), sim.get_time())
        sim.attach_gravity(None, 0.0)
        sim.close()
        mg.close()
    ref, rphi, rt = out["fp64"]
    err = {}
    for mode in ("fused", "unfused"):
        st, phi, t = out[mode]
        assert t[2] == rt[2]
        assert t[0] == pytest.approx(rt[0], rel=1e-6)
        e = {k: np.abs(st[k] - ref[k]).max() / np.abs(ref[k]).max() for k in ref}
        e["phi"] = np.abs(phi - rphi).max() / np.abs(rphi).max()
        err[mode] = e
    for k, e in err["fused"].items():
        assert e < 5e-6, (k, err)
        assert e <= 2.0 * err["unfused"][k] + 1e-9, (k, err)


def test_fixed_size_sg_matches_general():
    """Self-gravity on 64^3 blocks with two ghost layers takes the fixed-size instantiations
    of the sweeps and of the fused update with the source term; 32^3 blocks take the general
    ones. One 128^3 mesh run both ways for three cycles agrees to round-off (the multigrid's
    sums, parallel reductions, differ in their last bits between runs)."""
    import oracle_lib as ol
    n = 128
    u, b1, b2, b3 = ol.smooth_random_state((n, n, n), True, seed=37, amp=0.3)
    out = {}
    for mb in ((64, 64, 64), (32, 32, 32)):
        sim = athg.Sim((n, n, n), mb, mhd=True, solver="hlld", precision="mixed", cfl=0.4,
                       tlim=100.0)
        mg = athg.Multigrid(n, domain=((0.0, 1.0),) * 3, bc="periodic", mode="FMG",
                            threshold=-1.0, niteration=2, precision="fp64")
        sim.attach_gravity(mg, 4.0)
        sim.load_interior(u, b1, b2, b3)
        sim.initialize()
        sim.cycles(3)
        out[mb] = sim.interior()
        sim.attach_gravity(None, 0.0)
        sim.close()
        mg.close()
    a, c = out[(64, 64, 64)], out[(32, 32, 32)]
    for k in a:
        err = np.abs(a[k] - c[k]).max() / np.abs(c[k]).max()
        assert err < 1e-10, (k, err)

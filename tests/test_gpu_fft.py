"""Turbulence driving and FFT self-gravity on the GPU (cuFFT) against the CPU oracle
(oracle/fft_oracle.cpp, a line-by-line restatement of fft/turbulence.cpp and
gravity/fft_gravity.cpp with the same random engine and distributions).

Agreement is to round-off (1e-12 of the largest value): the random numbers, spectrum,
projection and Ornstein-Uhlenbeck update are the same arithmetic, while the transforms
(cuFFT against a direct DFT) and the global sums run in another order."""
import numpy as np
import pytest

import oracle_lib

athg = pytest.importorskip("athg")
pytestmark = pytest.mark.gpu

N = 32
MB = (16, 16, 16)
DOMAIN = ((0.0, 1.0), (0.0, 1.0), (0.0, 1.0))


def sim_of(mhd, **kw):
    return athg.Sim((N, N, N), MB, mhd, "hlld" if mhd else "hllc", precision="fp64",
                    cfl=0.3, tlim=100.0, domain=DOMAIN, **kw)


def state(mhd, seed=4):
    return oracle_lib.smooth_random_state((N, N, N), mhd, seed=seed)


def close(a, b, tol=1e-12):
    np.testing.assert_allclose(a, b, rtol=0, atol=tol * max(1.0, np.abs(b).max()))


@pytest.mark.parametrize("mhd,f_shear", [(False, -1.0), (True, 0.3), (False, 1.0)])
def test_decaying_drive_matches_oracle(mhd, f_shear):
    u, b1, b2, b3 = state(mhd)
    sim = sim_of(mhd)
    sim.attach_turbulence(1, dedt=0.5, rseed=17, nhigh=6, f_shear=f_shear)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()  # drives once (mesh/mesh.cpp:1383-1384)
    got = sim.interior()["u"]
    sim.close()
    ref = oracle_lib.TurbOracle((N, N, N), (1.0, 1.0, 1.0), 1, 0.5, 17, nhigh=6,
                                f_shear=f_shear).drive(u, 0.0, 0.0)
    assert np.abs(ref - u).max() > 1e-3  # the drive did something
    close(got, ref)


def test_driven_sequences_match_oracle():
    """Continuous (OU-smoothed, every call) and impulsive (every dtdrive) driving over a
    sequence of times and steps, through athg_turb_drive."""
    u, b1, b2, b3 = state(False, seed=9)
    for flag, kw in ((3, dict(tcorr=0.05)), (2, dict(tcorr=0.2, dtdrive=0.02))):
        sim = sim_of(False)
        sim.load_interior(u, b1, b2, b3)
        sim.attach_turbulence(flag, dedt=3.0, rseed=5, nlow=1, nhigh=5, **kw)
        orc = oracle_lib.TurbOracle((N, N, N), (1.0, 1.0, 1.0), flag, 3.0, 5, nlow=1, nhigh=5,
                                    **kw)
        ref = u.copy()
        for q, (t, dt) in enumerate(((0.0, 0.004), (0.011, 0.006), (0.021, 0.005),
                                     (0.03, 0.004), (0.045, 0.007))):
            sim.set_time(t, dt, q)
            sim.turb_drive()
            ref = orc.drive(ref, t, dt)
            close(sim.interior()["u"], ref)
        sim.close()


def test_driven_cycles_inject_dedt_dt():
    """Uniform gas at rest, continuous driving inside athg_cycles: the scheme conserves
    total energy, so after each cycle the box holds exactly dedt * (sum of the cycle dts)
    more."""
    u = np.zeros((5, N, N, N))
    u[0] = 1.0
    u[4] = 1.0 / (5.0 / 3.0 - 1.0)
    sim = sim_of(False)
    sim.load_interior(u)
    sim.initialize()
    sim.attach_turbulence(3, dedt=2.0, rseed=3, nhigh=4, tcorr=0.1)
    dvol = 1.0 / N ** 3
    e0 = sim.interior()["u"][4].sum() * dvol
    total = 0.0
    for _ in range(3):
        _, dt, _ = sim.get_time()
        sim.cycles(1)
        total += dt
        e = sim.interior()["u"][4].sum() * dvol
        assert e - e0 == pytest.approx(2.0 * total, rel=1e-10)
    sim.close()


def test_fft_gravity_matches_oracle_and_laplacian():
    u, b1, b2, b3 = state(True, seed=12)
    sim = sim_of(True)
    sim.attach_fft_gravity(4 * np.pi)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()  # first solve (mesh/mesh.cpp:1398-1402)
    phi = sim.phi()
    sim.close()
    ref = oracle_lib.fft_gravity(u[0], (1.0, 1.0, 1.0), 4 * np.pi)
    close(phi[1:-1, 1:-1, 1:-1], ref)
    # the ghost layer holds the periodic neighbours
    close(phi[0, 1:-1, 1:-1], ref[-1])
    close(phi[1:-1, 1:-1, -1], ref[:, :, 0])
    # the 7-point Laplacian of phi is 4 pi G (rho - mean rho)
    p = np.pad(ref, 1, mode="wrap")
    lap = (p[2:, 1:-1, 1:-1] + p[:-2, 1:-1, 1:-1] + p[1:-1, 2:, 1:-1] + p[1:-1, :-2, 1:-1] +
           p[1:-1, 1:-1, 2:] + p[1:-1, 1:-1, :-2] - 6 * ref) * N ** 2
    close(lap, 4 * np.pi * (u[0] - u[0].mean()), 1e-10)


def test_fft_gravity_tracks_converged_multigrid():
    """Both solve the periodic 7-point Poisson problem; with the multigrid iterated to a
    tight threshold the runs agree to its convergence over a few cycles."""
    u, b1, b2, b3 = state(False, seed=21)
    out = {}
    for kind in ("fft", "mg"):
        sim = sim_of(False)
        mg = None
        if kind == "fft":
            sim.attach_fft_gravity(1.0)
        else:
            mg = athg.Multigrid(N, domain=DOMAIN, bc="periodic", mode="FMG", threshold=0.0,
                                precision="fp64")
            sim.attach_gravity(mg, 1.0)
        sim.load_interior(u)
        sim.initialize()
        sim.cycles(3)
        phi = sim.phi()[1:-1, 1:-1, 1:-1]
        out[kind] = (sim.interior()["u"], phi - phi.mean())
        sim.close()
        if mg is not None:
            mg.close()
    close(out["fft"][1], out["mg"][1], 1e-9)
    close(out["fft"][0], out["mg"][0], 1e-9)


# ---- against the reference's own FFT drivers (fixtures from tests/golden/make_fft_golden.py:
# the unmodified reference built with a direct-DFT stand-in for FFTW) ----
import golden_lib  # noqa: E402


def _fixture_sim(meta, a):
    n = tuple(meta["nx"])
    sim = athg.Sim(n, tuple(meta["meshblock"]), meta["mhd"], meta["solver"], precision="fp64",
                   cfl=meta["cfl"], tlim=100.0, domain=DOMAIN)
    return sim


@pytest.mark.parametrize("name", ["fft_turb_decay_mhd", "fft_turb_decay_hydro"])
def test_decaying_drive_matches_reference(name):
    meta, a = golden_lib.load(name)
    t = meta["turb"]
    sim = _fixture_sim(meta, a)
    sim.attach_turbulence(1, dedt=t["dedt"], rseed=t["rseed"], nlow=t["nlow"], nhigh=t["nhigh"],
                          f_shear=t["f_shear"], expo=t["expo"])
    sim.load_interior(a["u_in"], a.get("b1_in"), a.get("b2_in"), a.get("b3_in"))
    sim.initialize()
    got = sim.interior()["u"]
    sim.close()
    close(got, a["u_out"])


def test_continuous_drive_cycles_match_reference():
    meta, a = golden_lib.load("fft_turb_cont_hydro")
    t = meta["turb"]
    sim = _fixture_sim(meta, a)
    sim.load_interior(a["u_in"])
    sim.attach_turbulence(3, dedt=t["dedt"], rseed=t["rseed"], nlow=t["nlow"], nhigh=t["nhigh"],
                          tcorr=t["tcorr"], f_shear=t["f_shear"], expo=t["expo"])
    sim.initialize()
    sim.cycles(meta["nlim"])
    got = sim.interior()["u"]
    tt, _, n = sim.get_time()
    sim.close()
    assert n == meta["ncycle"]
    assert tt == pytest.approx(meta["time"], rel=1e-13)
    close(got, a["u_out"], tol=1e-11)


def test_fft_gravity_matches_reference():
    meta, a = golden_lib.load("fft_grav_hydro_init")
    sim = _fixture_sim(meta, a)
    sim.attach_fft_gravity(meta["four_pi_G"])
    sim.load_interior(a["u_in"])
    sim.initialize()
    phi = sim.phi()
    sim.close()
    inner = phi[1:-1, 1:-1, 1:-1] if phi.shape != a["phi"].shape else phi
    close(inner, a["phi"])
    meta, a = golden_lib.load("fft_grav_hydro_2cyc")
    sim = _fixture_sim(meta, a)
    sim.attach_fft_gravity(meta["four_pi_G"])
    sim.load_interior(a["u_in"])
    sim.initialize()
    sim.cycles(meta["nlim"])
    got = sim.interior()["u"]
    tt, _, n = sim.get_time()
    sim.close()
    assert n == meta["ncycle"]
    assert tt == pytest.approx(meta["time"], rel=1e-13)
    close(got, a["u_out"], tol=1e-11)

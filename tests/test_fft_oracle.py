"""The CPU oracle of the FFT-based routines (oracle/fft_oracle.cpp) against properties the
reference's definitions fix. The reference's FFT code needs FFTW, which this machine does
not have, so no reference run pins these; the properties below do:

* FFT gravity inverts the 7-point Laplacian exactly (gravity/fft_gravity.cpp:121-128 uses
  its eigenvalues): single Fourier modes against the analytic discrete solution.
* Turbulence driving injects exactly dedt (times dt when driven) of kinetic energy into
  the box with zero net momentum (fft/turbulence.cpp:334-441), keeps only the shells
  nlow < |k|/dk < nhigh (:290-324), and the projection (:448-530) leaves a solenoidal
  field for f_shear = 1 and a curl-free field for f_shear = 0."""
import numpy as np
import pytest

import oracle_lib


@pytest.mark.parametrize("mode", [(1, 0, 0), (0, 2, 0), (1, 1, 3)])
def test_fft_gravity_single_mode(mode):
    n = (16, 8, 12)  # n1, n2, n3
    lengths = (1.0, 0.5, 2.0)
    x = [(np.arange(n[d]) + 0.5) * lengths[d] / n[d] for d in range(3)]
    arg = (2 * np.pi * mode[2] * x[2] / lengths[2])[:, None, None] + \
        (2 * np.pi * mode[1] * x[1] / lengths[1])[None, :, None] + \
        (2 * np.pi * mode[0] * x[0] / lengths[0])[None, None, :]
    rho = 1.0 + 0.25 * np.cos(arg)
    phi = oracle_lib.fft_gravity(rho, lengths, 4 * np.pi)
    lam = sum((2 * np.cos(2 * np.pi * mode[d] / n[d]) - 2) / (lengths[d] / n[d]) ** 2
              for d in range(3))
    ana = 4 * np.pi * 0.25 * np.cos(arg) / lam
    np.testing.assert_allclose(phi, ana, rtol=0, atol=1e-13 * np.abs(ana).max())


def kinetic_box(n):
    u = np.zeros((5,) + (n, n, n))
    u[0] = 1.0
    u[4] = 1.5
    return u


def test_decaying_drive_injects_dedt():
    n = 16
    t = oracle_lib.TurbOracle((n, n, n), (1.0, 1.0, 1.0), 1, 0.7, rseed=3)
    u0 = kinetic_box(n)
    u = t.drive(u0.copy(), 0.0, 0.0)
    dvol = (1.0 / n) ** 3
    de = (u[4] - u0[4]).sum() * dvol
    ke = 0.5 * ((u[1] ** 2 + u[2] ** 2 + u[3] ** 2) / u[0]).sum() * dvol
    assert de == pytest.approx(0.7, rel=1e-12)
    assert ke == pytest.approx(0.7, rel=1e-12)
    assert np.abs(u[1:4].sum(axis=(1, 2, 3))).max() < 1e-12 * np.abs(u[1:4]).sum()


def test_continuous_drive_injects_dedt_dt():
    n = 8
    t = oracle_lib.TurbOracle((n, n, n), (1.0, 1.0, 1.0), 3, 2.0, rseed=11, tcorr=0.5)
    u = kinetic_box(n)
    e = [u[4].sum()]
    for q, dt in enumerate((0.01, 0.02, 0.015)):
        u = t.drive(u, 0.01 * q, dt)
        e.append(u[4].sum())
        assert (e[-1] - e[-2]) / n ** 3 == pytest.approx(2.0 * dt, rel=1e-11)


def spectrum_of(t, n):
    u0 = kinetic_box(n)
    u = t.drive(u0.copy(), 0.0, 0.0)
    v = u[1:4] / u[0]
    return v, np.stack([np.fft.fftn(v[d]) for d in range(3)])


def wavenumbers(n):
    k = np.fft.fftfreq(n) * n
    kz, ky, kx = np.meshgrid(k, k, k, indexing="ij")
    return kx, ky, kz


def test_shells_and_projection():
    n = 16
    kx, ky, kz = wavenumbers(n)
    kmag = np.sqrt(kx ** 2 + ky ** 2 + kz ** 2)
    # only 2 < |k| < 5 carries power
    _, f = spectrum_of(oracle_lib.TurbOracle((n,) * 3, (1.0,) * 3, 1, 1.0, 7, nlow=2,
                                             nhigh=5), n)
    p = (np.abs(f) ** 2).sum(axis=0)
    assert p[(kmag <= 2) | (kmag >= 5)].max() < 1e-20 * p.max()
    # f_shear = 1: solenoidal; f_shear = 0: curl-free
    _, f = spectrum_of(oracle_lib.TurbOracle((n,) * 3, (1.0,) * 3, 1, 1.0, 7, f_shear=1.0), n)
    div = kx * f[0] + ky * f[1] + kz * f[2]
    assert np.abs(div).max() < 1e-10 * (kmag * np.abs(f).max(axis=0)).max()
    _, f = spectrum_of(oracle_lib.TurbOracle((n,) * 3, (1.0,) * 3, 1, 1.0, 7, f_shear=0.0), n)
    curl = np.stack([ky * f[2] - kz * f[1], kz * f[0] - kx * f[2], kx * f[1] - ky * f[0]])
    assert np.abs(curl).max() < 1e-10 * (kmag * np.abs(f).max(axis=0)).max()


def test_seeded_sequence_is_reproducible():
    n = 8
    a = spectrum_of(oracle_lib.TurbOracle((n,) * 3, (1.0,) * 3, 1, 1.0, 42), n)[0]
    b = spectrum_of(oracle_lib.TurbOracle((n,) * 3, (1.0,) * 3, 1, 1.0, 42), n)[0]
    c = spectrum_of(oracle_lib.TurbOracle((n,) * 3, (1.0,) * 3, 1, 1.0, 43), n)[0]
    np.testing.assert_array_equal(a, b)
    assert np.abs(a - c).max() > 1e-3 * np.abs(a).max()


# ---- pinned against the reference's own FFT drivers (fixtures from
# tests/golden/make_fft_golden.py: the unmodified reference built with a direct-DFT stand-in
# for FFTW; the oracle's direct DFT sums in another order, hence the 1e-12 tolerances) ----
import golden_lib  # noqa: E402


def _fixture(name):
    return golden_lib.load(name)


@pytest.mark.parametrize("name", ["fft_turb_decay_mhd", "fft_turb_decay_hydro"])
def test_decaying_drive_matches_reference(name):
    meta, a = _fixture(name)
    t = meta["turb"]
    orc = oracle_lib.TurbOracle(tuple(meta["nx"]), (1.0, 1.0, 1.0), t["turb_flag"], t["dedt"],
                                t["rseed"], nlow=t["nlow"], nhigh=t["nhigh"],
                                f_shear=t["f_shear"], expo=t["expo"])
    got = orc.drive(a["u_in"], 0.0, 0.0)
    ref = a["u_out"]
    assert np.abs(ref - a["u_in"]).max() > 1e-3
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


def test_continuous_drive_cycles_match_reference():
    """Three cycles with a drive before each (main.cpp:457): the oracle's stage and
    driver in the reference's order."""
    meta, a = _fixture("fft_turb_cont_hydro")
    t = meta["turb"]
    n = tuple(meta["nx"])
    turb = oracle_lib.TurbOracle(n, (1.0, 1.0, 1.0), t["turb_flag"], t["dedt"], t["rseed"],
                                 nlow=t["nlow"], nhigh=t["nhigh"], tcorr=t["tcorr"],
                                 f_shear=t["f_shear"], expo=t["expo"])
    o = oracle_lib.Oracle(n, False, "hllc", cfl=meta["cfl"])
    o.load_interior(a["u_in"])
    o.initialize(100.0)
    for _ in range(meta["nlim"]):
        u = o.interior()["u"]
        o.load_interior(turb.drive(u, o.time, o.dt))
        o.cycle(1, 100.0)
    got = o.interior()["u"]
    assert o.time == pytest.approx(meta["time"], rel=1e-13)
    np.testing.assert_allclose(got, a["u_out"], rtol=0, atol=1e-11 * np.abs(a["u_out"]).max())


def test_fft_gravity_potential_matches_reference():
    meta, a = _fixture("fft_grav_hydro_init")
    phi = oracle_lib.fft_gravity(a["u_in"][0], (1.0, 1.0, 1.0), meta["four_pi_G"])
    ref = a["phi"]
    np.testing.assert_allclose(phi, ref, rtol=0, atol=1e-12 * np.abs(ref).max())

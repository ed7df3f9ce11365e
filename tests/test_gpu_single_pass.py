"""The single-pass mixed VL2 MHD stage (one launch per stage: PLM + HLLD/HLLE fluxes of
all three directions, corner EMFs, flux divergence, CT and primitive recovery on chip,
W/bcc planes staged by TMA) against the separate-kernel mixed path it replaces.

Both paths evaluate the same FP32 reconstruction, Riemann solver and corner-EMF
expressions and the same exact FP32 flux sums into the FP64 state, but the compiler fuses
multiply-adds differently in the two code layouts, so single FP32 fluxes can differ in
the last bit; the states are held to the mixed path's tolerance (2e-6 of each field's
magnitude after five cycles, the bound of the mixed path against the reference). Within
the single pass, k-segment counts do not change the result at all (bitwise).
"""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu

athg = pytest.importorskip("athg")

NX, MB = (64, 32, 32), (32, 16, 16)


def _run(u, b1, b2, b3, single, solver="hlld", cycles=5, nseg=0, nx=NX, mb=MB):
    sim = athg.Sim(nx, mb, mhd=True, solver=solver, precision="mixed", cfl=0.4, tlim=100.0)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    sim.set_stage_kernel(single, nseg)
    used = sim.stage_kernel()
    sim.cycles(cycles)
    out = (sim.interior(), sim.get_time(), sim.max_div_b(), sim.sum_conserved(),
           sim.download(athg.VAR_PRIM))
    sim.close()
    return used, out


def _close(a, b, tol=1e-12):
    for k in a:
        np.testing.assert_allclose(a[k], b[k], rtol=0, atol=tol * np.abs(b[k]).max())


@pytest.mark.parametrize("solver", ["hlld", "hlle"])
def test_single_pass_matches_separate_kernels(solver):
    """Five cycles (odd: the state ends in the other buffer) on 8 blocks of 32x16x16."""
    u, b1, b2, b3 = ol.smooth_random_state(NX, True, seed=23, amp=0.3)
    (on, _), (si, st, sd, ss, sw) = _run(u, b1, b2, b3, True, solver)
    (off, _), (ui, ut, ud, us, uw) = _run(u, b1, b2, b3, False, solver)
    assert on and not off
    assert st[2] == ut[2] and abs(st[0] - ut[0]) <= 1e-6 * ut[0]
    _close(si, ui, tol=2e-6)
    # the primitives the next cycle would start from (FP32, interior and ghosts)
    np.testing.assert_allclose(sw, uw, rtol=0, atol=2e-6 * np.abs(uw).max())
    assert sd < 1e-13 and ud < 1e-13


def test_single_pass_segments_do_not_change_results():
    u, b1, b2, b3 = ol.smooth_random_state(NX, True, seed=29, amp=0.3)
    ref = None
    for nseg in (1, 2, 4):
        (on, seg), (si, st, _, _, _) = _run(u, b1, b2, b3, True, cycles=3, nseg=nseg)
        assert on and seg == nseg
        if ref is None:
            ref = (si, st)
            continue
        assert st == ref[1]
        for k in si:
            assert np.array_equal(si[k], ref[0][k]), k


def test_single_pass_conserves_and_keeps_div_b():
    """Periodic box: mass, momentum and energy conserved to FP64 round-off over ten cycles,
    div B at FP64 round-off."""
    u, b1, b2, b3 = ol.smooth_random_state(NX, True, seed=5, amp=0.3)
    sim = athg.Sim(NX, MB, mhd=True, solver="hlld", precision="mixed", cfl=0.4, tlim=100.0)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    sim.set_stage_kernel(True)
    assert sim.stage_kernel()[0]
    s0 = sim.sum_conserved()
    sim.cycles(10)
    s1 = sim.sum_conserved()
    d1 = sim.max_div_b()
    sim.close()
    assert d1 < 1e-13, d1
    assert np.all(np.abs(s1 - s0) <= 1e-13 * np.maximum(1.0, np.abs(s0))), s1 - s0


def test_single_pass_against_oracle():
    """Two cycles of a 64^3 mesh of 8 blocks of 32^3 against the FP64 oracle, within the
    mixed path's tolerance."""
    nx, mb = (64, 64, 64), (32, 32, 32)
    u, b1, b2, b3 = ol.smooth_random_state(nx, True, seed=41, amp=0.2)
    (on, _), (si, _, _, _, _) = _run(u, b1, b2, b3, True, cycles=2, nx=nx, mb=mb)
    assert on
    o = ol.Oracle(nx, True, "hlld", cfl=0.4)
    o.load_interior(u, b1, b2, b3)
    o.initialize(100.0)
    o.cycle(2, 100.0)
    ref = o.interior()
    for k in ref:
        err = np.abs(si[k] - ref[k]).max() / np.abs(ref[k]).max()
        assert err < 2e-6, (k, err)


def test_device_error_word_reports_non_finite_state():
    """A NaN planted in the uploaded state reaches the last stage's time-step pass, which
    sets the device error word; the next synchronising call returns ATHG_ERR_DEVICE (-4)
    with a message, and clears the word."""
    u, b1, b2, b3 = ol.smooth_random_state(NX, True, seed=3, amp=0.2)
    sim = athg.Sim(NX, MB, mhd=True, solver="hlld", precision="mixed", cfl=0.4, tlim=100.0)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    sim.set_stage_kernel(True)
    assert sim.stage_kernel()[0]
    cons = sim.download(athg.VAR_CONS)
    cons[3, 1, 10, 10, 10] = np.nan  # block 3, x1 momentum, one interior cell
    sim.upload(athg.VAR_CONS, cons)
    sim.cycles(1)
    L = athg.lib()
    t, d, n = C.c_double(), C.c_double(), C.c_int64()
    rc = L.athg_get_time(sim.h, C.byref(t), C.byref(d), C.byref(n))
    assert rc == -4
    assert b"non-finite" in L.athg_last_error()
    assert L.athg_get_time(sim.h, C.byref(t), C.byref(d), C.byref(n)) == 0  # cleared
    sim.close()


def test_separate_kernels_are_the_default():
    u, b1, b2, b3 = ol.smooth_random_state(NX, True, seed=2, amp=0.1)
    sim = athg.Sim(NX, MB, mhd=True, solver="hlld", precision="mixed", cfl=0.4, tlim=100.0)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    assert not sim.stage_kernel()[0]
    sim.close()

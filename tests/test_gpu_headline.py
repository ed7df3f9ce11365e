"""Parity at the headline configuration: Orszag-Tang 256^3, 64 MeshBlocks of 64^3,
PLM + HLLD + CT + VL2, CFL 0.4 (the reference's pgen/orszag_tang.cpp initial state).

The FP64 path on 64 blocks is compared with the oracle (one 256^3 block, FP64 CPU
restatement of the reference's stage, pinned bit for bit to the reference on the golden
fixtures) after two cycles. Per-block face positions are computed from each block's own
bounds (coordinates/cartesian.cpp), which can differ from the single block's in the last
bit, so agreement is asserted to 1e-13 of the field's magnitude rather than bitwise. The
mixed path (FP32 fluxes, FP64 state and CT) is held to the stated mixed tolerance.
"""
import numpy as np
import pytest

import oracle_lib as ol
import pgens

pytestmark = pytest.mark.gpu

athg = pytest.importorskip("athg")

NX = (256, 256, 256)
MB = (64, 64, 64)
DOM = ((-0.5, 0.5),) * 3
CYCLES = 2


@pytest.fixture(scope="module")
def reference_state():
    u, b1, b2, b3 = pgens.orszag_tang(NX)
    o = ol.Oracle(NX, True, "hlld", cfl=0.4, domain=DOM)
    o.load_interior(u, b1, b2, b3)
    o.initialize(100.0)
    o.cycle(CYCLES, 100.0)
    ref = o.interior()
    t = o.time
    del o
    return (u, b1, b2, b3), ref, t


def _gpu_run(init, precision):
    sim = athg.Sim(NX, MB, mhd=True, solver="hlld", precision=precision, cfl=0.4,
                   tlim=100.0, domain=DOM)
    sim.load_interior(*init)
    sim.initialize()
    sim.cycles(CYCLES)
    out = sim.interior()
    t = sim.get_time()
    divb = sim.max_div_b()
    sim.close()
    return out, t, divb


def test_headline_fp64_matches_oracle(reference_state):
    init, ref, t_ref = reference_state
    out, (t, dt, n), divb = _gpu_run(init, "fp64")
    assert n == CYCLES
    assert abs(t - t_ref) <= 1e-15 * t_ref, (t, t_ref)
    bmax = max(float(np.abs(ref[k]).max()) for k in ("b1", "b2", "b3"))
    for k in ("u", "b1", "b2", "b3"):
        # face fields against the largest field component (b3 is zero up to round-off in
        # the z-invariant vortex)
        scale = float(np.abs(ref[k]).max()) if k == "u" else bmax
        err = float(np.abs(out[k] - ref[k]).max())
        assert err <= 1e-13 * scale, (k, err)
    assert divb < 1e-13


def test_headline_mixed_close_to_oracle(reference_state):
    init, ref, _ = reference_state
    out, (_, _, n), divb = _gpu_run(init, "mixed")
    assert n == CYCLES
    # FP32 reconstruction and Riemann fluxes: relative deviation of the state after two
    # cycles at the 1e-7..1e-6 level (the same bound as the single-block fixtures)
    bmax = max(float(np.abs(ref[k]).max()) for k in ("b1", "b2", "b3"))
    for k in ("u", "b1", "b2", "b3"):
        scale = float(np.abs(ref[k]).max()) if k == "u" else bmax
        err = float(np.abs(out[k] - ref[k]).max()) / scale
        assert err < 2e-6, (k, err)
    assert divb < 1e-13


def test_headline_dfloat_matches_oracle(reference_state):
    """The double-float flux path (FP64 state, fluxes and EMFs in FP32 pairs) at the
    headline size: within 1e-11 of the oracle, like the single-block fixtures."""
    init, ref, t_ref = reference_state
    out, (t, _, n), divb = _gpu_run(init, "dfloat")
    assert n == CYCLES
    assert abs(t - t_ref) <= 1e-12 * t_ref, (t, t_ref)
    bmax = max(float(np.abs(ref[k]).max()) for k in ("b1", "b2", "b3"))
    for k in ("u", "b1", "b2", "b3"):
        scale = float(np.abs(ref[k]).max()) if k == "u" else bmax
        err = float(np.abs(out[k] - ref[k]).max()) / scale
        assert err < 1e-11, (k, err)
    assert divb < 1e-13

"""The CPU oracle's self-gravity coupling (source term of hydro/srcterms/self_gravity.cpp
and a multigrid solve after every stage, main.cpp:459-466) against the reference run
with SELF_GRAVITY_ENABLED = 2."""
import numpy as np
import pytest

import golden_lib
import oracle_lib as ol


def run_oracle(meta, a):
    n = meta["nx"][0]
    o = ol.Oracle(tuple(meta["nx"]), meta["mhd"], meta["solver"], xorder=meta["xorder"],
                  integrator=meta["integrator"], cfl=meta["cfl"], gamma=meta["gamma"])
    mg = ol.MgOracle(int(np.log2(n)), domain=((0.0, 1.0),) * 3, bc="periodic",
                     fmg=meta["mgmode"] == "FMG", niter=meta["niteration"])
    o.attach_gravity(mg, meta["four_pi_G"])
    o.load_interior(a["u_in"], a.get("b1_in"), a.get("b2_in"), a.get("b3_in"))
    o.initialize(100.0)
    o.cycle(meta["ncycles"], 100.0)
    g = o.ng
    phi = o.phi[g:g + n, g:g + n, g:g + n].copy()
    return o, o.interior(), phi


@pytest.mark.parametrize("name", golden_lib.sg_cases())
def test_sg_oracle_matches_reference(name):
    meta, a = golden_lib.load(name)
    o, got, phi = run_oracle(meta, a)
    assert o.time == pytest.approx(meta["time"], rel=1e-14)
    single_block = meta["nx"] == meta["meshblock"]
    keys = ["u"] + (["b1", "b2", "b3"] if meta["mhd"] else [])
    for k in keys:
        ref = a[k + "_out"]
        if single_block:
            assert np.array_equal(got[k], ref), (k, np.abs(got[k] - ref).max())
        else:
            # several blocks: the reference's multigrid sums (average subtraction,
            # restriction onto its root grid) run in a different order
            np.testing.assert_allclose(got[k], ref, rtol=0, atol=1e-12)
    scale = np.abs(a["phi_out"]).max()
    np.testing.assert_allclose(phi, a["phi_out"], rtol=0, atol=1e-12 * scale)

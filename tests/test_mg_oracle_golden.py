"""The multigrid oracle against the reference's own MG gravity solve."""
import numpy as np
import pytest

import golden_lib
import oracle_lib as ol

MG_CASES = golden_lib.mg_cases()


@pytest.mark.parametrize("name", MG_CASES)
def test_mg_oracle_matches_reference(name):
    meta, a = golden_lib.load(name)
    n = meta["n"]
    m = ol.MgOracle(int(np.log2(n)), bc=meta["bc"], fmg=(meta["mode"] == "FMG"), eps=-1.0,
                    niter=meta["niteration"], mporder=4)
    m.load_source(a["rho"] * meta["four_pi_G"])
    m.solve()
    ref = a["phi"]
    # same stencils and cycle; sums (averages, multipole moments) are ordered
    # differently from the reference's per-MeshBlock partial sums
    err = np.abs(m.phi() - ref).max() / np.abs(ref).max()
    assert err < 1e-12, err

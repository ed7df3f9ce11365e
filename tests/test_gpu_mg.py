"""CUDA multigrid against the reference's MG gravity solve and the oracle.

FP64 path: the reference's cycle in FP64; agreement with the reference is at round-off
(1e-12 relative), limited by the order of the global sums (mean subtraction, multipole
moments). Mixed path: FP32 V-cycles with FP64 defect and correction, converged to the
same discrete solution.
"""
import numpy as np
import pytest

import golden_lib
import oracle_lib as ol

pytestmark = pytest.mark.gpu
athg = pytest.importorskip("athg")


@pytest.mark.parametrize("name", golden_lib.mg_cases())
def test_mg_fp64_matches_reference(name):
    meta, a = golden_lib.load(name)
    mg = athg.Multigrid(meta["n"], bc=meta["bc"], mode=meta["mode"], threshold=-1.0,
                        niteration=meta["niteration"], precision="fp64")
    mg.load_source(a["rho"], fac=meta["four_pi_G"])
    it, _ = mg.solve()
    assert it == meta["niteration"]
    ref = a["phi"]
    err = np.abs(mg.phi() - ref).max() / np.abs(ref).max()
    assert err < 1e-12, err


@pytest.mark.parametrize("bc", ["periodic", "multipole", "zerograd"])
def test_mg_fp64_matches_oracle_converged(bc):
    n = 64
    x = (np.arange(n) + 0.5) / n - 0.5
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    rho = np.where(r < 0.25, 1.0, 1.0e-6) + 0.1 * np.cos(2 * np.pi * X) * np.sin(4 * np.pi * Y)
    src = 4 * np.pi * rho
    o = ol.MgOracle(6, bc=bc, fmg=True, eps=-1.0, niter=8, mporder=4)
    o.load_source(src)
    o.solve()
    mg = athg.Multigrid(n, bc=bc, mode="FMG", threshold=-1.0, niteration=8, precision="fp64")
    mg.load_source(src)
    mg.solve()
    ref = o.phi()
    err = np.abs(mg.phi() - ref).max() / np.abs(ref).max()
    assert err < 1e-11, err


@pytest.mark.parametrize("bc", ["periodic", "multipole"])
def test_mg_mixed_reaches_fp64_solution(bc):
    """Iterative refinement: FP32 cycles, FP64 defect, relative residual 1e-10."""
    n = 64
    x = (np.arange(n) + 0.5) / n - 0.5
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    r = np.sqrt(X ** 2 + Y ** 2 + Z ** 2)
    rho = np.where(r < 0.25, 1.0, 1.0e-6)
    src = 4 * np.pi * rho
    res = {}
    for prec in ("fp64", "mixed"):
        mg = athg.Multigrid(n, bc=bc, mode="FMG", threshold=-1.0, niteration=0, precision=prec)
        mg.load_source(src)
        mg.solve()
        d0 = mg.defect_norm()
        mg2 = athg.Multigrid(n, bc=bc, mode="FMG", threshold=1e-10 * np.sqrt(np.mean(src ** 2)),
                             precision=prec)
        mg2.load_source(src)
        it, dn = mg2.solve()
        assert dn <= 1e-10 * np.sqrt(np.mean(src ** 2)), (prec, dn)
        res[prec] = (it, mg2.phi(), d0)
    phi64, phim = res["fp64"][1], res["mixed"][1]
    # both converged to the same discrete solution well below truncation error
    assert np.abs(phim - phi64).max() / np.abs(phi64).max() < 1e-9

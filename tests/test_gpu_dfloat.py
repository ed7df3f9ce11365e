"""The double-float flux path (precision "dfloat": reconstruction, Riemann fluxes and corner
EMFs in pairs of FP32 values on the FP32 pipe; FP64 state, update, CT and primitives).

Against the reference: every golden fixture it covers (donor cell / PLM; HLLC, HLLE, HLLD)
to 1e-11 of each field's magnitude (double-float operations carry ~2^-44 relative error,
FP64 ones 2^-53). Against the analytic linear waves at the reference's amplitude 1e-6: the
L1 error equals the FP64 path's (the reference's own linearwave-errors.dat values) to 1%,
which the FP32 flux path cannot reach at this amplitude (stated next to it).
"""
import numpy as np
import pytest

import golden_lib
import pgens as pgen_lw

pytestmark = pytest.mark.gpu

athg = pytest.importorskip("athg")


def _df_cases():
    out = []
    for name in golden_lib.cases():
        meta, _ = golden_lib.load(name)
        if meta["xorder"] in (1, 2) and meta["solver"] in ("hllc", "hlle", "hlld"):
            out.append(name)
    return out


@pytest.mark.parametrize("name", _df_cases())
def test_dfloat_matches_reference_fixtures(name):
    meta, a = golden_lib.load(name)
    per = 0 if meta.get("bc") == "outflow" else 1
    sim = athg.Sim(tuple(meta["nx"]), tuple(meta["meshblock"]), mhd=meta["mhd"],
                   solver=meta["solver"], precision="dfloat", xorder=meta["xorder"],
                   integrator=meta["integrator"], cfl=meta["cfl"], gamma=meta["gamma"],
                   tlim=100.0, ng=meta.get("nghost", 2), periodic=(per, per, per))
    sim.load_interior(a["u_in"], a.get("b1_in"), a.get("b2_in"), a.get("b3_in"))
    sim.initialize()
    sim.cycles(meta["ncycles"])
    out = sim.interior()
    t, dt, n = sim.get_time()
    sim.close()
    assert n == meta["ncycle"]
    assert abs(t - meta["time"]) <= 1e-12 * abs(meta["time"])
    for k in (["u"] + (["b1", "b2", "b3"] if meta["mhd"] else [])):
        ref = a[k + "_out"]
        err = float(np.abs(out[k] - ref).max() / np.abs(ref).max())
        assert err < 1e-11, (k, err)


@pytest.mark.parametrize("mhd,solver,tlim,cfl,key", [
    (False, "hllc", 1.0, 0.4, "hydro_c1"),
    (True, "hlld", 0.5, 0.3, "mhd_fast"),
])
def test_linear_wave_dfloat_equal_l1_at_reference_amplitude(mhd, solver, tlim, cfl, key):
    """C1 (hydro, HLLC) and C2 (MHD fast wave, HLLD) linear waves, 64x32x32, amplitude 1e-6:
    the double-float path's L1 error is the FP64 path's, to 1%."""
    ref = golden_lib.linear_wave_errors()[key]
    ref_rms = ref["values"][4]
    dom = ((0.0, 3.0), (0.0, 1.5), (0.0, 1.5))
    nx = (64, 32, 32)
    lw = pgen_lw.LinearWave(nx, dom, mhd)
    u, b1, b2, b3 = lw.initial_state()
    sim = athg.Sim(nx, nx, mhd=mhd, solver=solver, precision="dfloat", cfl=cfl,
                   gamma=1.666666666666667, tlim=tlim, domain=dom)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    n = sim.run(tlim)
    out = sim.interior()
    sim.close()
    rms = lw.l1_errors(out["u"], out.get("b1"), out.get("b2"), out.get("b3"))[0]
    assert n == int(ref["values"][3])
    assert abs(rms - ref_rms) <= 0.01 * ref_rms, (rms, ref_rms)

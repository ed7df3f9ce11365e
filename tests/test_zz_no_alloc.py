"""athg_block_cfl_dt_noalloc: the CFL time step of one block whose device arrays the
caller owns, computed without any device allocation (scratch is a fixed device array in
the library). It is for callers that cannot allocate device memory -- code that must not
synchronise the device (cudaMalloc and cudaFree may), or hosts whose device memory is
managed by their own pool. Its result must equal the pool entry point athg_new_block_dt on the same state.

This file is collected last on purpose. It runs alone in a fresh process as well as after
the other tests.
"""
import ctypes as C

import numpy as np
import pytest

import oracle_lib as ol

pytestmark = pytest.mark.gpu
athg = pytest.importorskip("athg")
torch = pytest.importorskip("torch")


def _dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("mhd,solver", [(True, "hlld"), (False, "hllc")])
def test_noalloc_dt_matches_pool_dt_twice(mhd, solver):
    nx = (24, 16, 8)
    u, b1, b2, b3 = ol.smooth_random_state(nx, mhd, seed=77, amp=0.2)
    sim = athg.Sim(nx, nx, mhd=mhd, solver=solver, precision="fp64", cfl=0.4, tlim=100.0)
    sim.load_interior(u, b1, b2, b3)
    sim.initialize()
    expect = sim.new_block_dt()  # pool entry point, scratch in the pool
    # the same block's arrays, owned by the caller on the device
    w = _dev(sim.download(athg.VAR_PRIM)[0])
    if mhd:
        bcc = _dev(sim.download(athg.VAR_BCC)[0])
        bf = [_dev(sim.download(v)[0]) for v in (athg.VAR_B1F, athg.VAR_B2F, athg.VAR_B3F)]
        ptrs = [bcc.data_ptr()] + [t.data_ptr() for t in bf]
    else:
        ptrs = [None, None, None, None]
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    L = athg.lib()
    dx = (1.0 / nx[0], 1.0 / nx[1], 1.0 / nx[2])
    torch.cuda.synchronize()
    for _ in range(2):  # two calls in a row share the scratch array
        out.zero_()
        rc = L.athg_block_cfl_dt_noalloc(C.byref(sim.cfg), w.data_ptr(), *ptrs, *dx,
                                         out.data_ptr(), None)
        athg.check(rc)
        torch.cuda.synchronize()
        got = float(out.item())
        # identical per-cell formula; a minimum does not depend on reduction order
        assert got == pytest.approx(expect, rel=1e-15, abs=0.0), (got, expect)


def test_noalloc_rejects_oversized_block():
    cfg = athg.Config()
    cfg.nx1 = cfg.nx2 = cfg.nx3 = 512
    cfg.nghost, cfg.magnetic, cfg.gamma, cfg.cfl_number = 2, 0, 5.0 / 3.0, 0.4
    rc = athg.lib().athg_block_cfl_dt_noalloc(C.byref(cfg), 1, None, None, None, None,
                                              1.0, 1.0, 1.0, 1, None)
    assert rc == -1
    assert b"too large" in athg.lib().athg_last_error()

"""gb_jacobian_solve_noalloc: the allocation-free Jacobian update + solve.

Callers that cannot allocate device memory while they run (a Newton iteration
recorded in a stream capture, code confined to a memory pool it does not own)
use this entry point: its Jacobian blocks live in a static device array of
GB_NOALLOC_SCRATCH_BYTES instead of storage the library allocates.  The test
compares it through the C ABI with gb_update_jacobian + gb_ldiv on two calls
in a row (the second call reuses the array the first one left behind), within
the tolerance the other GPU tests use, and checks the size limit.  It lives in
its own file so that pytest collects it last.
"""

import numpy as np
import pytest

from gbdycore import _native as N
from gbdycore import simulation as sim
from helpers import field_errors, perturbed_state, small_config

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ft,tol", [(np.float64, 1e-10), (np.float32, 1e-3)])
def test_noalloc_jacobian_solve_matches_the_allocating_hooks(ft, tol):
    cfg = small_config(ft=ft, z_elem=40)
    p = sim.AtmosCache(cfg)
    dtg = 0.4358665215084590 * cfg.dt
    rng = np.random.default_rng(8)
    for call in range(2):
        Yc, Yf = perturbed_state(cfg, seed=20 + call, dtype=ft, w_amp=0.3)
        Rc = (rng.normal(size=Yc.shape) * np.abs(Yc).max(axis=(0, 2, 3), keepdims=True) * 1e-3).astype(ft)
        Rf = (rng.normal(size=Yf.shape) * 0.1).astype(ft)
        Y, R = sim.FieldVector.from_numpy(Yc, Yf), sim.FieldVector.from_numpy(Rc, Rf)
        ref, out = Y.similar(), Y.similar()
        jac = sim.Jacobian(p)
        sim.update_jacobian(jac, Y, p, dtg, 0.0)
        sim.ldiv(ref, jac, R)
        p.call("gb_jacobian_solve_noalloc", out.gb(), Y.gb(), R.gb(), float(dtg))
        ro, rr = out.numpy(), ref.numpy()
        errs = field_errors(ro[0], ro[1], rr[0], rr[1])
        assert all(v <= tol for v in errs.values()), (call, errs)


def test_noalloc_rejects_grids_beyond_the_static_scratch():
    cfg = small_config(ft=np.float64, h_elem=30, z_elem=63)   # 86400 columns x 64 faces x 15 x 8 B > 64 MiB
    p = sim.AtmosCache(cfg)
    Y = sim.FieldVector.from_numpy(np.ones((6 * 30 * 30, 4, 16, 63)), np.zeros((6 * 30 * 30, 16, 64)))
    with pytest.raises(N.GBError) as ei:
        p.call("gb_jacobian_solve_noalloc", Y.gb(), Y.gb(), Y.gb(), 1.0)
    assert ei.value.code == N.GB_ERR_ARG and "GB_NOALLOC_SCRATCH_BYTES" in str(ei.value)

"""gb_jacobian_solve_noalloc: the Jacobian update + solve that allocates no device memory.

Some callers cannot let a library allocate device memory: a host model whose
runtime owns every byte of the GPU through its own pool (CUDA.jl's allocator, a
pre-sized arena of an operational forecast), where a cudaMalloc behind its back
either fails or breaks its accounting, and callers that must not pay the device
synchronisation a first cudaMalloc implies in the middle of a Newton loop.
gb_update_jacobian allocates the Jacobian's block storage on first use; this
entry point keeps the blocks in a fixed static device array instead.

The test calls it through the C ABI twice in a row on different states (the
second call reuses the array the first one left behind) and checks each result
bitwise against gb_update_jacobian + gb_ldiv (the same kernels on the same
inputs) and against the oracle's ldiv within the tolerance of the other
Jacobian tests; then the size limit.  It lives in its own file so that pytest
collects it last.
"""
import numpy as np
import pytest

from gbdycore import _native as N
from gbdycore import simulation as sim
from helpers import field_errors, make_oracle, moist_field_errors, moist_state, perturbed_state, small_config

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ft,tol", [(np.float64, 1e-13), (np.float32, 1e-3)])
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
        np.testing.assert_array_equal(ro[0], rr[0], err_msg="call %d, centres" % call)
        np.testing.assert_array_equal(ro[1], rr[1], err_msg="call %d, faces" % call)
        o = make_oracle(cfg, ft)
        o.set_precomputed(Yc, Yf)
        o.update_jacobian(Yc, Yf, dtg)
        oc, of = o.ldiv(Rc, Rf)
        errs = field_errors(ro[0], ro[1], oc, of)
        assert all(v <= tol for v in errs.values()), (call, errs)


@pytest.mark.parametrize("ft,tol", [(np.float64, 1e-13), (np.float32, 1e-3)])
def test_noalloc_moist_jacobian_solve_matches_the_allocating_hooks(ft, tol):
    """A moist 0M context: the 19 stored values per level (with the rho q_tot blocks) in the
    static array, bitwise equal to gb_update_jacobian + gb_ldiv, and the oracle's moist ldiv."""
    cfg = small_config(ft=ft, z_elem=40, moist=True)
    p = sim.AtmosCache(cfg)
    dtg = 0.4358665215084590 * cfg.dt
    rng = np.random.default_rng(9)
    Yc, Yf = moist_state(cfg, dtype=ft, w_amp=0.3)
    Rc = (rng.normal(size=Yc.shape) * np.abs(Yc).max(axis=(0, 2, 3), keepdims=True) * 1e-3).astype(ft)
    Rf = (rng.normal(size=Yf.shape) * 0.1).astype(ft)
    Y, R = sim.FieldVector.from_numpy(Yc, Yf), sim.FieldVector.from_numpy(Rc, Rf)
    ref, out = Y.similar(), Y.similar()
    jac = sim.Jacobian(p)
    sim.update_jacobian(jac, Y, p, dtg, 0.0)
    sim.ldiv(ref, jac, R)
    p.call("gb_jacobian_solve_noalloc", out.gb(), Y.gb(), R.gb(), float(dtg))
    ro, rr = out.numpy(), ref.numpy()
    np.testing.assert_array_equal(ro[0], rr[0])
    np.testing.assert_array_equal(ro[1], rr[1])
    o = make_oracle(cfg, ft)
    o.set_precomputed(Yc, Yf)
    o.update_jacobian(Yc, Yf, dtg)
    oc, of = o.ldiv(Rc, Rf)
    errs = moist_field_errors(ro[0], ro[1], oc, of)
    assert all(v <= tol for v in errs.values()), errs


def test_noalloc_rejects_grids_beyond_the_static_scratch():
    cfg = small_config(ft=np.float64, h_elem=30, z_elem=63)   # 86400 columns x 64 faces x 15 x 8 B > 64 MiB
    p = sim.AtmosCache(cfg)
    Y = sim.FieldVector.from_numpy(np.ones((6 * 30 * 30, 4, 16, 63)), np.zeros((6 * 30 * 30, 16, 64)))
    with pytest.raises(N.GBError) as ei:
        p.call("gb_jacobian_solve_noalloc", Y.gb(), Y.gb(), Y.gb(), 1.0)
    assert ei.value.code == N.GB_ERR_ARG and "GB_NOALLOC_SCRATCH_BYTES" in str(ei.value)

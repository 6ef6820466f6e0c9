"""GPU tests of the drop-in boundary's own features, through the C ABI.

* The caller's element layout (gb_config.elem_map / elem_orient): a context built for a
  random element numbering computes, on the state in that numbering, exactly the
  library-order result moved there (bitwise for a renumbering alone; with turned element
  frames the derivatives run in another order, so to FP64 roundoff).
* test_dycore_consistency: with every scratch buffer NaN-filled before each tendency and
  each step (fill_with_nans!, src/utils/debug_utils.jl:58-70) the hooks and the fused step
  give the same bits as without, so nothing reads scratch it did not write first.
* The bounded device wait running out: gb_selftest_bounded_wait waits on a transfer that is
  never issued, with a 1 ms limit; the status reads GB_ERR_TIMEOUT, and the context then
  steps normally.
"""
import numpy as np
import pytest

from gbdycore import _native as N
from gbdycore import layout as LY
from gbdycore import simulation as sim
from helpers import field_errors, perturbed_state, small_config

pytestmark = pytest.mark.gpu


def _steps(cfg, Yc, Yf, n, use_graph=True):
    s = sim.AtmosSimulation(cfg, state=(Yc, Yf))
    s.step(n, use_graph=use_graph)
    s.p.newton_residual()
    return s.Y.numpy()


@pytest.mark.parametrize("rotate", [False, True])
def test_fused_step_in_a_caller_layout(rotate):
    cfg = small_config(ft=np.float64, z_elem=12)
    Yc, Yf = perturbed_state(cfg, w_amp=0.05)
    ref = _steps(cfg, Yc, Yf, 3)
    emap, eori = LY.random_layout(cfg.h_elem, seed=11, rotate=rotate)
    Xc, Xf = LY.to_caller(Yc, Yf, emap, eori)
    out = LY.from_caller(*_steps(cfg.with_(layout=(emap, eori)), Xc, Xf, 3), emap, eori)
    if not rotate:
        np.testing.assert_array_equal(out[0], ref[0])
        np.testing.assert_array_equal(out[1], ref[1])
    else:
        # the turned frames run the derivatives in another order: FP64 roundoff, with u_3's
        # tendency a cancellation of terms ~1e3 times |u_3| (as against the oracle)
        e = field_errors(out[0], out[1], ref[0], ref[1])
        lim = {"rho": 1e-14, "rho_e_tot": 1e-14, "u_1": 1e-12, "u_2": 1e-12, "u_3": 2e-11}
        assert all(e[k] <= lim[k] for k in lim), e


def test_hooks_in_a_permuted_layout_fp32():
    cfg = small_config(ft=np.float32, z_elem=10)
    Yc, Yf = perturbed_state(cfg, dtype=np.float32, w_amp=0.1)
    emap, eori = LY.random_layout(cfg.h_elem, seed=2, rotate=False)
    Xc, Xf = LY.to_caller(Yc, Yf, emap, eori)
    outs = []
    for c, (a, b) in ((cfg, (Yc, Yf)), (cfg.with_(layout=(emap, eori)), (Xc, Xf))):
        p = sim.AtmosCache(c)
        Y = sim.FieldVector.from_numpy(a, b)
        T, Ti = Y.similar(), Y.similar()
        sim.remaining_tendency(T, None, Y, p, 0.0)
        sim.implicit_tendency(Ti, Y, p, 0.0)
        outs.append((T.numpy(), Ti.numpy()))
    for k in range(2):
        got = LY.from_caller(*outs[1][k], emap, eori)
        np.testing.assert_array_equal(got[0], outs[0][k][0])
        np.testing.assert_array_equal(got[1], outs[0][k][1])


@pytest.mark.parametrize("ft", [np.float32, np.float64])
def test_nan_filled_scratch_changes_nothing(ft):
    cfg = small_config(ft=ft, z_elem=10)
    Yc, Yf = perturbed_state(cfg, dtype=ft, w_amp=0.1)
    dbg = cfg.with_(test_dycore_consistency=True)
    for use_graph in (True, False):
        a, b = _steps(cfg, Yc, Yf, 2, use_graph), _steps(dbg, Yc, Yf, 2, use_graph)
        assert np.isfinite(b[0]).all() and np.isfinite(b[1]).all()
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
    res = []
    for c in (cfg, dbg):
        p = sim.AtmosCache(c)
        Y = sim.FieldVector.from_numpy(Yc, Yf)
        T, Ti, corr = Y.similar(), Y.similar(), Y.similar()
        sim.remaining_tendency(T, None, Y, p, 0.0)
        sim.implicit_tendency(Ti, Y, p, 0.0)
        sim.correct_implicit_advection_tendency(corr, Y, p, 0.0)
        res.append([x for F in (T, Ti, corr) for x in F.numpy()])
    for a, b in zip(*res):
        np.testing.assert_array_equal(a, b)


def test_bounded_wait_runs_out_and_the_context_recovers():
    cfg = small_config(ft=np.float32)
    s = sim.AtmosSimulation(cfg, state=perturbed_state(cfg, dtype=np.float32))
    rc = s.p.L.gb_selftest_bounded_wait(s.p.h, 1e-3)
    assert rc == N.GB_ERR_TIMEOUT
    with pytest.raises(N.GBError, match="timed out"):
        sim._check(s.p.h, rc)
    # the status word was cleared: the next steps run and report no failure
    s.step(2)
    r = s.p.newton_residual()
    assert np.isfinite(r).all()
    assert s.p.L.gb_selftest_bounded_wait(s.p.h, 0.0) == N.GB_ERR_ARG

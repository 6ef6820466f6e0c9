"""GPU parity of the moist 0M column hooks (gb_config.moist = 1) against the CPU oracle.

The centre block carries rho q_tot as its fifth component.  Each hook runs through the C ABI:
the implicit tendency (central transport of q_tot, moist pressure from the saturation
adjustment), the post-Newton correction, the Jacobian with kappa_m and the (u_3, rho q_tot),
(rho q_tot, u_3) blocks, and ldiv with the rho q_tot row; the state DSS (bitwise) and the
conservation sums with the water integral.  Tolerances (max-norm error relative
to each component's max magnitude): FP64 <= 2e-12 (measured: the implicit tendency's u_3 row
3e-13 at z_elem 12 and 6e-13 at 63, the pressure-gradient difference of two terms each ~g dz;
every other row and ldiv <= 3e-14); FP32 against the FP32 oracle <= 1e-3 (measured: u_3's
tendency 2.5e-4, the device's hardware exp/log in q_v* against the C library's amplified by the
same cancellation; every other row and ldiv <= 5e-6)."""
import numpy as np
import pytest

from gbdycore import _native as N
from gbdycore import simulation as sim
from helpers import (dss_oracle_on_product_grid, make_oracle, moist_field_errors, moist_state, perturbed_state,
                     rel_err, small_config)

pytestmark = pytest.mark.gpu


def _dev(Yc, Yf):
    return sim.FieldVector.from_numpy(Yc, Yf)


def _assert(errs, tol):
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, "errors above %g: %s (all: %s)" % (tol, bad, errs)


FT_CASES = [(np.float64, 2e-12), (np.float32, 1e-3)]


@pytest.mark.parametrize("ft,tol", FT_CASES)
@pytest.mark.parametrize("z_elem", [12, 63])
def test_moist_implicit_tendency_and_correction(ft, tol, z_elem):
    # z_elem 63: two levels per lane, the production column length
    cfg = small_config(ft=ft, z_elem=z_elem, moist=True)
    Yc, Yf = moist_state(cfg, dtype=ft, w_amp=0.3)
    o = make_oracle(cfg, ft)
    ref = o.implicit_tendency(Yc.copy(), Yf.copy())
    refc = o.correct_implicit(Yc.copy(), Yf.copy())
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf)
    Yt = Y.similar()
    sim.implicit_tendency(Yt, Y, p, 0.0)
    _assert(moist_field_errors(*Yt.numpy(), *ref), tol)
    sim.correct_implicit_advection_tendency(Yt, Y, p, 0.0)
    got = Yt.numpy()
    for c in (3, 4):
        assert rel_err(got[0][:, c], refc[0][:, c]) <= tol, c
    assert np.all(got[0][:, :3] == 0) and np.all(got[1] == 0)


@pytest.mark.parametrize("ft,tol", FT_CASES)
def test_moist_jacobian_and_ldiv(ft, tol):
    cfg = small_config(ft=ft, z_elem=12, moist=True)
    Yc, Yf = moist_state(cfg, dtype=ft, w_amp=0.3)
    dtg = 0.4 * cfg.dt
    o = make_oracle(cfg, ft)
    o.update_jacobian(Yc.copy(), Yf.copy(), dtg)
    rng = np.random.default_rng(21)
    Rc = rng.normal(size=Yc.shape).astype(ft)
    Rf = rng.normal(size=Yf.shape).astype(ft)
    ref = o.ldiv(Rc, Rf)
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf)
    sim.update_jacobian(sim.Jacobian(p), Y, p, dtg, 0.0)
    R = _dev(Rc, Rf)
    dY = R.similar()
    sim.ldiv(dY, sim.Jacobian(p), R)
    _assert(moist_field_errors(*dY.numpy(), *ref), tol)


def test_moist_hooks_without_water_match_the_dry_hooks():
    """rho q_tot = 0: every moist hook reproduces the dry context's (FP64; the moist path forms
    theta_v = T R_m / (Pi R_d) and kappa_m = R_m / cv_m, equal to the dry values up to rounding)."""
    cfg = small_config(z_elem=12)
    Yc, Yf = perturbed_state(cfg, w_amp=0.3)
    Ym = np.ascontiguousarray(np.concatenate([Yc, np.zeros_like(Yc[:, :1])], axis=1))
    pd, pm = sim.AtmosCache(cfg), sim.AtmosCache(cfg.with_(moist=True))
    Yd, Ymd = _dev(Yc, Yf), _dev(Ym, Yf)
    Td, Tm = Yd.similar(), Ymd.similar()
    sim.implicit_tendency(Td, Yd, pd, 0.0)
    sim.implicit_tendency(Tm, Ymd, pm, 0.0)
    a, b = Td.numpy(), Tm.numpy()
    for c in range(4):
        assert rel_err(b[0][:, c], a[0][:, c]) < 1e-13, c
    assert np.all(b[0][:, 4] == 0) and rel_err(b[1], a[1]) < 1e-13
    dtg = 0.4 * cfg.dt
    sim.update_jacobian(sim.Jacobian(pd), Yd, pd, dtg, 0.0)
    sim.update_jacobian(sim.Jacobian(pm), Ymd, pm, dtg, 0.0)
    rng = np.random.default_rng(2)
    Rc, Rf = rng.normal(size=Yc.shape), rng.normal(size=Yf.shape)
    Rm = np.ascontiguousarray(np.concatenate([Rc, np.zeros_like(Rc[:, :1])], axis=1))
    Rd_, Rmd = _dev(Rc, Rf), _dev(Rm, Rf)
    Xd, Xm = Rd_.similar(), Rmd.similar()
    sim.ldiv(Xd, sim.Jacobian(pd), Rd_)
    sim.ldiv(Xm, sim.Jacobian(pm), Rmd)
    a, b = Xd.numpy(), Xm.numpy()
    for c in range(4):
        assert rel_err(b[0][:, c], a[0][:, c]) < 1e-11, c
    assert rel_err(b[1], a[1]) < 1e-11


def test_moist_context_refuses_the_dry_only_entries():
    cfg = small_config(moist=True)
    Yc, Yf = moist_state(cfg)
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf)
    for call in (lambda: sim.remaining_tendency(Y.similar(), None, Y, p, 0.0),
                 lambda: p.call("gb_step", Y.gb(), 0.0, float(cfg.dt), 1, 0),
                 lambda: sim.dss_transpose(Y, p)):
        with pytest.raises(N.GBError) as e:
            call()
        assert e.value.code == N.GB_ERR_ARG


def _assert_u3(errs, tol, tol_u3):
    bad = {k: v for k, v in errs.items() if not v <= (tol_u3 if k == "u_3" else tol)}
    assert not bad, "errors above the bounds: %s (all: %s)" % (bad, errs)


def test_moist_hooks_at_the_production_grid():
    """h_elem 30, z_elem 63 stretched (the headline grid), the moist initial state: the FP64
    implicit tendency and Jacobian solve against the FP64 oracle at 2e-12, u_3's tendency at 1e-11
    (measured 3.8e-12): it is the difference of gravity and the vertical pressure gradient, each
    about g dz, in a hydrostatically balanced state, so that its FP64 roundoff relative to its
    own maximum grows with that cancellation."""
    from gbdycore import config as C
    from gbdycore import setups as S
    from helpers import oracle_geometry
    cfg = C.production_h30().with_(ft=np.float64, moist=True)
    g = oracle_geometry(cfg)
    Yc, Yf = S.moist_initial_state(g, cfg, seed=1, sigma=2.0, dtype=np.float64)
    rng = np.random.default_rng(3)
    Yf = np.ascontiguousarray(rng.normal(0.0, 0.05, size=Yf.shape) * g.dzf[None, None, :])
    o = make_oracle(cfg)
    ref = o.implicit_tendency(Yc.copy(), Yf.copy())
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf)
    Yt = Y.similar()
    sim.implicit_tendency(Yt, Y, p, 0.0)
    _assert_u3(moist_field_errors(*Yt.numpy(), *ref), 2e-12, 1e-11)
    dtg = 0.4358665215084590 * cfg.dt
    o.update_jacobian(Yc.copy(), Yf.copy(), dtg)
    refx = o.ldiv(ref[0], ref[1])
    sim.update_jacobian(sim.Jacobian(p), Y, p, dtg, 0.0)
    X = Y.similar()
    sim.ldiv(X, sim.Jacobian(p), Yt)
    _assert_u3(moist_field_errors(*X.numpy(), *refx), 2e-12, 1e-11)


@pytest.mark.parametrize("ft", [np.float64, np.float32])
def test_moist_state_dss_matches_oracle_bitwise(ft):
    """gb_dss of a moist state: rho q_tot averaged as a scalar with the dry DSS's fixed copy order
    and fused multiply-add recipe, so that on the library's own grid tables the oracle agrees bit
    for bit, rho q_tot included."""
    cfg = small_config(ft=ft, moist=True)
    Yc, Yf = moist_state(cfg)
    rng = np.random.default_rng(2)
    Yc = (Yc * (1 + 1e-3 * rng.normal(size=Yc.shape))).astype(ft)    # break continuity
    Yf = (Yf + 1e-3 * rng.normal(size=Yf.shape)).astype(ft)
    rc, rf = Yc.copy(), Yf.copy()
    dss_oracle_on_product_grid(cfg, ft).dss(rc, rf)
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf)
    sim.dss(Y, p, 0.0)
    gc, gf = Y.numpy()
    np.testing.assert_array_equal(gc, rc)
    np.testing.assert_array_equal(gf, rf)
    assert not np.array_equal(gc[:, 4], Yc[:, 4])


def test_moist_conservation_sums_match_oracle():
    """gb_conservation_sums: the integrals of rho, rho e_tot and rho q_tot against the oracle's
    compensated sums (1e-14); gb_global_sums returns the first two; a dry context reports no water."""
    cfg = small_config(ft=np.float64, moist=True)
    Yc, Yf = moist_state(cfg)
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf)
    s = p.conservation_sums(Y)
    ref = make_oracle(cfg).global_sums(Yc)
    assert s.shape == (3,) and s[2] > 0
    assert np.all(np.abs(s - ref) <= 1e-14 * np.abs(ref)), (s, ref)
    np.testing.assert_array_equal(p.global_sums(Y), s[:2])
    dcfg = cfg.with_(moist=False)
    Dc, Df = perturbed_state(dcfg)
    pd = sim.AtmosCache(dcfg)
    D = _dev(Dc, Df)
    sd = pd.conservation_sums(D)
    assert sd[2] == 0.0
    np.testing.assert_array_equal(sd[:2], pd.global_sums(D))

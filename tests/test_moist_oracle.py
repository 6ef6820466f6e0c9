"""The oracle's moist 0M column operators (CPU only): the saturation adjustment, the transport of
rho q_tot in the implicit tendency and its post-Newton correction, the moist Jacobian blocks and
the Schur solve with the rho q_tot row; the state DSS and the conservation sums with rho q_tot.

Thermodynamics.jl (1.3.0, not vendored) and ClimaParams hold the reference's moist thermodynamics,
so parity with them is unpinned.  Pinned here by properties of the formulation the reference's
Jacobian assumes (manual_sparse_jacobian.jl:646-685): the adjustment returns the equilibrium
whose internal energy is the given one, an unsaturated point keeps all of its water as vapour,
zero water reproduces the dry operators, the (rho q_tot, u_3) block is the exact derivative of
the rho q_tot tendency, the (u_3, rho q_tot) block linearises the pressure gradient, ldiv inverts
the stored Jacobian, and the correction is van Leer minus central for rho q_tot too."""
import numpy as np
import pytest

from helpers import make_oracle, moist_state, oracle_geometry, perturbed_state, rel_err, small_config


def _cfg(**kw):
    return small_config(moist=True, **kw)


def _qsat_np(cfg, T, rho):
    """q_v*(T, rho) restated in numpy from the published formulas (an independent check of the
    C++ restatement)."""
    K, M = cfg.constants, cfg.moist_constants
    lam = np.clip((T - M["T_icenuc"]) / (M["T_freeze"] - M["T_icenuc"]), 0, 1) ** M["pow_icenuc"]
    dcp = lam * (M["cp_v"] - M["cp_l"]) + (1 - lam) * (M["cp_v"] - M["cp_i"])
    L0 = lam * M["LH_v0"] + (1 - lam) * M["LH_s0"]
    ps = M["press_triple"] * (T / M["T_triple"]) ** (dcp / M["R_v"]) * np.exp(
        (L0 - dcp * K["T_0"]) / M["R_v"] * (1 / M["T_triple"] - 1 / T))
    return ps / (rho * M["R_v"] * T), lam


def _eint_np(cfg, T, q, ql, qi):
    K, M = cfg.constants, cfg.moist_constants
    cvv = M["cp_v"] - M["R_v"]
    cvm = K["cv_d"] + (cvv - K["cv_d"]) * q + (M["cp_l"] - cvv) * ql + (M["cp_i"] - cvv) * qi
    ev0, ei0 = M["LH_v0"] - M["R_v"] * K["T_0"], M["LH_s0"] - M["LH_v0"]
    return cvm * (T - K["T_0"]) + (q - ql - qi) * ev0 - qi * ei0 - (1 - q) * K["R_d"] * K["T_0"]


def test_saturation_adjustment_recovers_the_equilibrium():
    """Saturated points from warm (all liquid) through the mixed-phase ramp to cold (all ice):
    the adjustment of e_int(T*, equilibrium at T*) returns T* and its partition."""
    cfg = _cfg()
    o = make_oracle(cfg)
    rng = np.random.default_rng(3)
    T = rng.uniform(215.0, 305.0, 400)
    rho = rng.uniform(0.2, 1.2, 400)
    qs, lam = _qsat_np(cfg, T, rho)
    q = qs * rng.uniform(1.02, 1.6, 400)       # supersaturated at T
    qc = q - qs
    ql, qi = lam * qc, (1 - lam) * qc
    e = _eint_np(cfg, T, q, ql, qi)
    Ta, la, ia = o.sat_adjust(rho, e, q)
    assert np.abs(Ta - T).max() < 1e-9
    assert np.abs(la - ql).max() < 1e-12 and np.abs(ia - qi).max() < 1e-12
    # above freezing all condensate is liquid, at or below T_icenuc all ice
    warm, cold = T > cfg.moist_constants["T_freeze"] + 0.5, T < cfg.moist_constants["T_icenuc"] - 0.5
    assert warm.any() and cold.any()
    assert np.all(ia[warm] == 0) and np.all(la[cold] == 0)


def test_unsaturated_points_keep_their_water_as_vapour():
    cfg = _cfg()
    o = make_oracle(cfg)
    rng = np.random.default_rng(4)
    T = rng.uniform(220.0, 300.0, 200)
    rho = rng.uniform(0.2, 1.2, 200)
    qs, _ = _qsat_np(cfg, T, rho)
    q = qs * rng.uniform(0.0, 0.95, 200)
    e = _eint_np(cfg, T, q, 0.0, 0.0)
    Ta, la, ia = o.sat_adjust(rho, e, q)
    assert np.abs(Ta - T).max() < 1e-10
    assert np.all(la == 0) and np.all(ia == 0)


def test_zero_water_reproduces_the_dry_column_operators():
    cfg = small_config(z_elem=12)
    Yc, Yf = perturbed_state(cfg, w_amp=0.3)
    d, m = make_oracle(cfg), make_oracle(cfg.with_(moist=True))
    Ym = np.ascontiguousarray(np.concatenate([Yc, np.zeros_like(Yc[:, :1])], axis=1))
    for name in ("implicit_tendency", "correct_implicit"):
        a, b = getattr(d, name)(Yc.copy(), Yf.copy()), getattr(m, name)(Ym.copy(), Yf.copy())
        for c in range(4):
            assert rel_err(b[0][:, c], a[0][:, c]) < 1e-13, (name, c)
        assert np.all(b[0][:, 4] == 0)
        assert rel_err(b[1], a[1]) < 1e-13
    dtg = 0.4 * cfg.dt
    d.update_jacobian(Yc.copy(), Yf.copy(), dtg)
    m.update_jacobian(Ym.copy(), Yf.copy(), dtg)
    rng = np.random.default_rng(9)
    Rc, Rf = rng.normal(size=Yc.shape), rng.normal(size=Yf.shape)
    Rm = np.concatenate([Rc, np.zeros_like(Rc[:, :1])], axis=1)
    a, b = d.ldiv(Rc, Rf), m.ldiv(Rm, Rf)
    for c in range(4):
        assert rel_err(b[0][:, c], a[0][:, c]) < 1e-11, c
    assert rel_err(b[1], a[1]) < 1e-11


def test_moist_ldiv_inverts_the_stored_jacobian():
    cfg = _cfg(z_elem=12)
    o = make_oracle(cfg)
    Yc, Yf = moist_state(cfg, w_amp=0.3)
    o.update_jacobian(Yc, Yf, 0.4 * cfg.dt)
    rng = np.random.default_rng(5)
    Rc, Rf = rng.normal(size=Yc.shape), rng.normal(size=Yf.shape)
    Xc, Xf = o.ldiv(Rc, Rf)
    Wc, Wf = o.jac_apply(Xc, Xf)
    assert np.abs(Wc - Rc).max() < 1e-9 * np.abs(Rc).max()
    assert np.abs(Wf - Rf).max() < 1e-6 * np.abs(Rf).max()


def _fd(cfg, o, Yc, Yf, Vc, Vf, dtg, eps=1e-3):
    Tp = o.implicit_tendency(Yc + eps * Vc, Yf + eps * Vf)
    Tm = o.implicit_tendency(Yc - eps * Vc, Yf - eps * Vf)
    o.update_jacobian(Yc, Yf, dtg)
    Wc, Wf = o.jac_apply(Vc, Vf)
    return (Wc + Vc, Wf + Vf), (dtg * (Tp[0] - Tm[0]) / (2 * eps), dtg * (Tp[1] - Tm[1]) / (2 * eps))


def test_rho_q_tot_row_is_exact():
    """(rho q_tot, u_3) = dtγ ᶜadvection_matrix diag(ᶠinterp(q_tot) g³³) is the exact derivative of
    the rho q_tot tendency (linear in u_3)."""
    cfg = _cfg(upwinding="none", z_elem=12)
    o = make_oracle(cfg)
    Yc, Yf = moist_state(cfg, w_amp=0.3)
    rng = np.random.default_rng(7)
    Vc, Vf = np.zeros_like(Yc), np.zeros_like(Yf)
    Vf[:, :, 1:-1] = rng.normal(size=Vf[:, :, 1:-1].shape) * 1e-2 * np.abs(Yf).max()
    got, ref = _fd(cfg, o, Yc, Yf, Vc, Vf, 0.4 * cfg.dt)
    assert np.abs(ref[0][:, 4]).max() > 0
    assert np.linalg.norm(got[0][:, 4] - ref[0][:, 4]) / np.linalg.norm(ref[0][:, 4]) < 1e-9


def test_u3_row_rho_q_tot_column_against_central_differences():
    """(u_3, rho q_tot) = dtγ ᶠp_grad_matrix diag(∂p/∂ρq_tot) (manual_sparse_jacobian.jl:827-831)
    linearises the pressure gradient of an unsaturated column (the formula's own assumption) up
    to vertical truncation error, as the dry columns do (test_oracle_invariants.py)."""
    cfg = _cfg(upwinding="none", z_elem=30)
    o = make_oracle(cfg)
    g = oracle_geometry(cfg)
    Yc, Yf = moist_state(cfg, w_amp=0.0, q0=0.003)
    Vc, Vf = np.zeros_like(Yc), np.zeros_like(Yf)
    # relative to rho q_tot, so that the perturbed columns stay unsaturated and q_tot positive
    Vc[:, 4] = Yc[:, 4] * np.sin(np.pi * g.zc / g.z_max)[None, None, :]
    got, ref = _fd(cfg, o, Yc, Yf, Vc, Vf, 0.4 * cfg.dt)
    gi, ri = got[1][:, :, 1:-1], ref[1][:, :, 1:-1]
    assert np.abs(ri).max() > 0
    assert np.linalg.norm(gi - ri) / np.linalg.norm(ri) < 0.05


def test_moist_correction_conserves_rho_q_tot():
    """The post-Newton correction of rho q_tot (correct_implicit_advection_tendency!,
    implicit_tendency.jl:322-339, van Leer minus central face values of q_tot) is a difference of
    face fluxes with none through the boundaries: nonzero, and its J-weighted column sums
    vanish; with upwinding off it is zero."""
    cfg = _cfg(z_elem=12)
    o = make_oracle(cfg)
    Yc, Yf = moist_state(cfg, w_amp=0.3)
    Tc, _ = o.correct_implicit(Yc.copy(), Yf.copy())
    g = oracle_geometry(cfg)
    J = g.Jh[:, :, None] * (g.rc ** 2 * g.dzc)[None, None, :]
    assert np.abs(Tc[:, 4]).max() > 0
    s = (Tc[:, 4] * J).sum(axis=-1)
    assert np.abs(s).max() < 1e-12 * np.abs(Tc[:, 4] * J).max() * cfg.z_elem
    Tn, _ = make_oracle(cfg.with_(upwinding="none")).correct_implicit(Yc.copy(), Yf.copy())
    assert np.all(Tn == 0)


def test_moist_oracle_refuses_the_dry_only_operators():
    cfg = _cfg()
    o = make_oracle(cfg)
    Yc, Yf = moist_state(cfg)
    with pytest.raises(NotImplementedError):
        o.remaining_tendency(Yc, Yf)
    with pytest.raises(NotImplementedError):
        o.step(Yc, Yf, cfg.dt)


def test_moist_initial_state_carries_the_profile_temperature():
    """gbdycore.setups.moist_initial_state: at rest (K = 0) the adjustment of each point returns
    the profile's temperature where the point is unsaturated, a warmer one (latent heat) where it
    condenses; both kinds of point occur."""
    from gbdycore import setups as S
    cfg = _cfg(z_elem=20)
    g = oracle_geometry(cfg)
    Yc, Yf = S.moist_initial_state(g, cfg, seed=0, sigma=0.0, dtype=np.float64)
    assert Yc.shape == (g.Nh, 5, 16, cfg.z_elem)
    rho, q = Yc[:, 0], Yc[:, 4] / Yc[:, 0]
    eint = Yc[:, 3] / rho - cfg.constants["grav"] * g.zc[None, None, :]
    T, ql, qi = make_oracle(cfg).sat_adjust(rho, eint, q)
    T_prof, _ = S.temperature_pressure(np.broadcast_to(g.zc, T.shape), cfg.constants)
    dry = (ql + qi) == 0
    assert dry.any() and (~dry).any()
    assert np.abs(T[dry] - T_prof[dry]).max() < 1e-9
    assert np.all(T[~dry] > T_prof[~dry])


def _discontinuous_moist(cfg, seed=5):
    """A moist state whose collocated element copies disagree (rho q_tot too)."""
    Yc, Yf = moist_state(cfg)
    rng = np.random.default_rng(seed)
    Yc = Yc * (1 + 1e-3 * rng.normal(size=Yc.shape))
    Yf = Yf + 1e-3 * rng.normal(size=Yf.shape) * np.abs(Yf).max()
    return np.ascontiguousarray(Yc), np.ascontiguousarray(Yf)


def test_moist_state_dss_averages_rho_q_tot_as_a_scalar():
    """dss! of a moist state (constrain_state.jl:59-64): rho, u_h, rho e_tot and the faces as the
    dry DSS does them, rho q_tot exactly as rho (the same weights, copies and summation order)."""
    cfg = _cfg()
    Yc, Yf = _discontinuous_moist(cfg)
    Xc, Xf = Yc.copy(), Yf.copy()
    make_oracle(cfg).dss(Xc, Xf)
    Dc, Df = np.ascontiguousarray(Yc[:, :4]), Yf.copy()
    make_oracle(cfg.with_(moist=False)).dss(Dc, Df)
    assert np.array_equal(Xc[:, :4], Dc) and np.array_equal(Xf, Df)
    Qc = np.ascontiguousarray(Yc[:, [4, 1, 2, 3]])
    make_oracle(cfg.with_(moist=False)).dss(Qc, Yf.copy())
    assert np.array_equal(Xc[:, 4], Qc[:, 0])
    assert not np.array_equal(Xc[:, 4], Yc[:, 4])


def test_moist_conservation_sums_include_the_water():
    """check_conservation's sums (solve.jl:216-265) of a moist state: the integrals of rho and
    rho e_tot as the dry oracle forms them and the integral of rho q_tot with the same weights."""
    cfg = _cfg()
    Yc, Yf = moist_state(cfg)
    s = make_oracle(cfg).global_sums(Yc)
    dry = make_oracle(cfg.with_(moist=False))
    assert s.shape == (3,)
    assert np.array_equal(s[:2], dry.global_sums(np.ascontiguousarray(Yc[:, :4])))
    assert s[2] == dry.global_sums(np.ascontiguousarray(Yc[:, [4, 1, 2, 3]]))[0]
    assert s[2] > 0


def test_check_conservation_budgets():
    """The host side of check_conservation (solve.jl:216-265) on given sums: the energy budget
    relative to the first state's energy, the signed mass change, the water change relative to the
    last state's water, zero water budget for a dry run."""
    from gbdycore.simulation import check_conservation
    first, last = np.array([10.0, 200.0, 0.5]), np.array([10.1, 198.0, 0.4])
    r = check_conservation(first, last, moist=True)
    assert r["energy_conservation"] == pytest.approx(0.01)
    assert r["mass_conservation"] == pytest.approx(0.01)
    assert r["water_conservation"] == pytest.approx(0.25)
    r = check_conservation(first, last, moist=False, energy_surface_change=3.0, energy_radiation_input=1.0)
    assert r["energy_conservation"] == pytest.approx(0.0)
    assert r["water_conservation"] == 0.0

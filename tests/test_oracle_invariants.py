"""The CPU oracle against the reference's own known answers and invariants.

The reference holds no golden vectors for the dry-dycore arithmetic (its
hot-path unit tests are @test_skip placeholders); what it does pin is:
  * the Rayleigh sponge rate  (test/parameterized_tendencies/sponge.jl:46-69),
  * the impenetrable-boundary filter (test/prognostic_equations/advection_tests.jl:45-58),
  * the post-Newton identity corrected + central == upwind
    (test/prognostic_equations/correct_implicit_advection_tests.jl:43-56),
  * mass and energy conservation of the flux-form operators
    (src/simulation/solve.jl:216-265, docs/src/discretization.md:72-123),
  * Jacobian blocks against a differentiated implicit tendency
    (test/implicit/debugging_tools.jl:47-61), restated here as central
    finite differences in FP64,
  * the ARS343 tableau's order conditions (Ascher, Ruuth & Spiteri 1997).
"""
import math

import numpy as np
import pytest

from gbdycore import config as C
from gbdycore.simulation import ars343_tableau
from helpers import make_oracle, oracle_geometry, perturbed_state, small_config


def test_ars343_order_conditions():
    ae, ai, be, bi = ars343_tableau()
    ce, ci = ae.sum(1), ai.sum(1)
    assert np.allclose(ce, ci)                  # stage times agree
    for A, b in ((ae, be), (ai, bi)):
        c = A.sum(1)
        assert abs(b.sum() - 1) < 1e-14
        assert abs(b @ c - 0.5) < 1e-14
        assert abs(b @ c ** 2 - 1 / 3) < 1e-14
        assert abs(b @ A @ c - 1 / 6) < 1e-14
    # coupling conditions of an additive RK method of order 3
    assert abs(be @ ae @ ci - 1 / 6) < 1e-14 and abs(bi @ ai @ ce - 1 / 6) < 1e-14
    assert abs(be @ ai @ ce - 1 / 6) < 1e-14 and abs(bi @ ae @ ci - 1 / 6) < 1e-14
    g = ai[1, 1]
    assert abs(g ** 3 - 3 * g ** 2 + 1.5 * g - 1 / 6) < 1e-14    # L-stability root of ARS(3,4,3)


def _sponge_case(alpha_uh, alpha_w):
    # the reference's test space: cubed sphere radius 10, h_elem 4, z_elem 10, z_max 1, zd 0.5
    cfg = C.DycoreConfig(h_elem=4, z_elem=10, z_max=1.0, z_stretch=False, dt=1.0, nu=0.0, ft=np.float64,
                         sponge_zd=0.5, alpha_uh=alpha_uh, alpha_w=alpha_w, upwinding="none")
    cfg.constants = dict(cfg.constants, radius=10.0)
    return cfg


def test_rayleigh_sponge_known_answers():
    on, off = _sponge_case(1.0, 2.0), _sponge_case(0.0, 0.0)
    g = oracle_geometry(on)
    Nh, Nv = g.Nh, g.Nv
    Yc = np.zeros((Nh, 4, 16, Nv))
    Yc[:, 0] = 1.0
    Yc[:, 1] = 1.0        # u_h = Covariant12Vector(1, 1)
    Yc[:, 2] = 1.0
    Yc[:, 3] = 1.0e5
    Yf = np.ones((Nh, 16, Nv + 1))   # u_3 = Covariant3Vector(1)
    o_on, o_off = make_oracle(on), make_oracle(off)
    a = o_on.remaining_tendency(Yc.copy(), Yf.copy())[0]
    b = o_off.remaining_tendency(Yc.copy(), Yf.copy())[0]
    zc, zf = g.zc, g.zf
    beta_c = np.where(zc > 0.5, 1.0 * np.sin(math.pi / 2 * (zc - 0.5) / 0.5) ** 2, 0.0)
    beta_f = np.where(zf > 0.5, 2.0 * np.sin(math.pi / 2 * (zf - 0.5) / 0.5) ** 2, 0.0)
    scale = np.abs(b[:, 1:3]).max() + 1.0
    assert np.abs((a - b)[:, 1:3] - (-beta_c[None, None, None, :] * 1.0)).max() < 1e-12 * scale
    fa = o_on.implicit_tendency(Yc.copy(), Yf.copy())[1]
    fb = o_off.implicit_tendency(Yc.copy(), Yf.copy())[1]
    expect = -beta_f[None, None, :] * np.ones_like(fa)
    expect[:, :, 0] = expect[:, :, -1] = 0.0   # the boundary faces are filtered to u_3 = 0
    assert np.abs((fa - fb) - expect).max() < 1e-12 * (np.abs(fb).max() + 1.0)


def test_impenetrable_boundary_filter():
    cfg = small_config()
    Yc, Yf = perturbed_state(cfg)
    Yf[:, :, 0] = 3.0
    Yf[:, :, -1] = -2.0
    o = make_oracle(cfg)
    o.set_precomputed(Yc, Yf)
    assert np.all(Yf[:, :, 0] == 0) and np.all(Yf[:, :, -1] == 0)
    assert np.abs(Yf[:, :, 1:-1]).max() > 0


def _column_thermo(cfg, Yc, Yf, g):
    c = cfg.constants
    r2 = ((g.R + g.zc) / g.R) ** 2
    gu = g.gup[:, :, :, None] / r2[None, None, None, :]
    u1, u2 = Yc[:, 1], Yc[:, 2]
    c1 = gu[:, :, 0] * u1 + gu[:, :, 1] * u2
    c2 = gu[:, :, 1] * u1 + gu[:, :, 2] * u2
    u3c = Yf / g.dzf[None, None, :] ** 2
    kv = 0.5 * (Yf[:, :, :-1] * u3c[:, :, :-1] + Yf[:, :, 1:] * u3c[:, :, 1:])
    K = 0.5 * (u1 * c1 + u2 * c2 + kv)
    e_tot = Yc[:, 3] / Yc[:, 0]
    T = np.maximum(c["T_min_sgs"], c["T_0"] + (e_tot - K - c["grav"] * g.zc - (-c["R_d"] * c["T_0"])) / c["cv_d"])
    h = e_tot + c["R_d"] * T
    return h, u3c


def _vertical_transport(cfg, Yc, h, u3c, g, upwind):
    Nv = g.Nv
    J = g.Jh[:, :, None] * ((g.R + g.zc) / g.R)[None, None, :] ** 2 * g.dzc[None, None, :]
    rJ = Yc[:, 0] * J
    F = np.zeros(u3c.shape)
    for k in range(1, Nv):
        rb = 0.5 * (rJ[:, :, k - 1] + rJ[:, :, k])
        u = u3c[:, :, k]
        if not upwind:
            face = u * 0.5 * (h[:, :, k - 1] + h[:, :, k])
        else:
            def lim(am, a0, ap):
                da = 0.5 * (ap - am)
                mn, mx = np.minimum(np.minimum(am, a0), ap), np.maximum(np.maximum(am, a0), ap)
                return np.copysign(np.minimum(np.abs(da), np.minimum(2 * (a0 - mn), 2 * (mx - a0))), da)
            cr = 1 - np.abs(u) * cfg.dt
            if k == 1 or k == Nv - 1:
                up = np.where(u >= 0, h[:, :, k - 1], h[:, :, k])
            else:
                pos = h[:, :, k - 1] + lim(h[:, :, k - 2], h[:, :, k - 1], h[:, :, k]) * cr / 2
                neg = h[:, :, k] - lim(h[:, :, k - 1], h[:, :, k], h[:, :, k + 1]) * cr / 2
                up = np.where(u >= 0, pos, neg)
            face = u * up
        F[:, :, k] = rb * face
    return -(F[:, :, 1:] - F[:, :, :-1]) / J


def test_post_newton_identity():
    cfg = small_config(z_elem=10)
    g = oracle_geometry(cfg)
    Yc, Yf = perturbed_state(cfg, w_amp=0.5)
    o = make_oracle(cfg)
    corr = o.correct_implicit(Yc.copy(), Yf.copy())[0][:, 3]
    h, u3c = _column_thermo(cfg, Yc, Yf, g)
    central = _vertical_transport(cfg, Yc, h, u3c, g, upwind=False)
    upwind = _vertical_transport(cfg, Yc, h, u3c, g, upwind=True)
    scale = np.abs(upwind).max()
    assert scale > 0 and np.abs(corr).max() > 1e-6 * scale
    assert np.abs(corr + central - upwind).max() < 1e-10 * scale


@pytest.mark.parametrize("upwinding", ["vanleer", "none"])
def test_mass_and_energy_conservation(upwinding):
    cfg = small_config(upwinding=upwinding)
    o = make_oracle(cfg)
    Yc, Yf = perturbed_state(cfg)
    o.dss(Yc, Yf)
    s0 = o.global_sums(Yc)
    o.step(Yc, Yf, cfg.dt, 3)
    s1 = o.global_sums(Yc)
    assert np.isfinite(Yc).all()
    assert abs(s1[0] - s0[0]) <= 1e-13 * abs(s0[0])
    assert abs(s1[1] - s0[1]) <= 1e-12 * abs(s0[1])


def test_ldiv_inverts_the_stored_jacobian():
    cfg = small_config()
    o = make_oracle(cfg)
    Yc, Yf = perturbed_state(cfg)
    o.update_jacobian(Yc, Yf, 0.4 * cfg.dt)
    rng = np.random.default_rng(5)
    Rc, Rf = rng.normal(size=Yc.shape), rng.normal(size=Yf.shape)
    Xc, Xf = o.ldiv(Rc, Rf)
    Wc, Wf = o.jac_apply(Xc, Xf)
    # the acoustic Schur system has entries up to (c dt gamma / dz)^2 ~ 1e5, so the
    # attainable residual is eps * |W| |x|; 1e-6 of |R| is ~1e3 eps of that bound
    assert np.abs(Wc - Rc).max() < 1e-9 * np.abs(Rc).max()
    assert np.abs(Wf - Rf).max() < 1e-6 * np.abs(Rf).max()


def _fd_vs_manual(cfg, Yc, Yf, Vc, Vf, row, dtg, eps=1e-3):
    o = make_oracle(cfg)
    o.set_precomputed(Yc, Yf)
    Tp = o.implicit_tendency(Yc + eps * Vc, Yf + eps * Vf)
    Tm = o.implicit_tendency(Yc - eps * Vc, Yf - eps * Vf)
    o.update_jacobian(Yc, Yf, dtg)
    Wc, Wf = o.jac_apply(Vc, Vf)
    if row == "rho":
        got, ref = Wc[:, 0] + Vc[:, 0], dtg * (Tp[0] - Tm[0])[:, 0] / (2 * eps)
    else:
        got, ref = (Wf + Vf)[:, :, 1:-1], dtg * (Tp[1] - Tm[1])[:, :, 1:-1] / (2 * eps)
    assert np.abs(ref).max() > 0
    return np.linalg.norm(got - ref) / np.linalg.norm(ref)


def test_jacobian_mass_row_is_exact():
    """(rho, u_3) = dtγ ᶜadvection_matrix diag(g³³) is the exact derivative of the mass tendency."""
    cfg = small_config(upwinding="none")
    Yc, Yf = perturbed_state(cfg, w_amp=0.3)
    rng = np.random.default_rng(7)
    Vc, Vf = np.zeros_like(Yc), np.zeros_like(Yf)
    Vf[:, :, 1:-1] = rng.normal(size=Vf[:, :, 1:-1].shape) * 1e-2 * np.abs(Yf).max()
    assert _fd_vs_manual(cfg, Yc, Yf, Vc, Vf, "rho", 0.4 * cfg.dt) < 1e-9


@pytest.mark.parametrize("col,tol", [("rho", 0.1), ("rhoe", 0.02), ("u3", 0.03)])
def test_jacobian_momentum_row_against_central_differences(col, tol):
    """The u_3 row linearises the Exner-form pressure gradient through continuous
    identities (manual_sparse_jacobian.jl:789-815), so it equals the derivative of
    the discrete tendency only up to vertical truncation error: compared with
    smooth perturbations, as the reference's AD comparison tool does (not asserted there)."""
    cfg = small_config(upwinding="none", z_elem=30)
    g = oracle_geometry(cfg)
    Yc, Yf = perturbed_state(cfg, w_amp=0.3 if col == "u3" else 0.0)
    Vc, Vf = np.zeros_like(Yc), np.zeros_like(Yf)
    prof = np.sin(np.pi * g.zc / g.z_max)[None, None, :]
    if col == "rho":
        Vc[:, 0] = 1e-3 * Yc[:, 0] * prof
    elif col == "rhoe":
        Vc[:, 3] = 1e-3 * np.abs(Yc[:, 3]).max() * prof
    else:
        Vf[:, :, 1:-1] = 0.1 * g.dzf[1:-1] * np.sin(np.pi * g.zf[1:-1] / g.z_max)
    assert _fd_vs_manual(cfg, Yc, Yf, Vc, Vf, "u3", 0.4 * cfg.dt) < tol


def test_oracle_is_deterministic():
    cfg = small_config()
    o = make_oracle(cfg)
    a = perturbed_state(cfg)
    b = (a[0].copy(), a[1].copy())
    o.step(a[0], a[1], cfg.dt, 2)
    o.step(b[0], b[1], cfg.dt, 2)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_step_meets_the_reference_conservation_bounds():
    """check_conservation (solve.jl:216-265) over three oracle steps of the dry dycore, held to the
    bounds the reference's CI asserts (.buildkite/ci_driver.jl:175-187): the energy budget within
    100 eps, the mass budget within 250 eps (FP64)."""
    from gbdycore.simulation import check_conservation
    cfg = small_config(ft=np.float64)
    Yc, Yf = perturbed_state(cfg)
    o = make_oracle(cfg)
    s0 = np.append(o.global_sums(Yc), 0.0)
    o.step(Yc, Yf, cfg.dt, 3)
    s1 = np.append(o.global_sums(Yc), 0.0)
    r = check_conservation(s0, s1, moist=False)
    eps = np.finfo(np.float64).eps
    # the reference's `x ≈ 0 atol = a`: |x| <= a (the energy budget divides by the signed ∫ρe_tot)
    assert abs(r["energy_conservation"]) <= 100 * eps and abs(r["mass_conservation"]) <= 250 * eps, r

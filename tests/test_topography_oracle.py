"""The oracle's dry step over terrain-following levels (CPU only): the per-point metric enters
every operator, the impenetrable filter, the Jacobian (with its (rho, u_h) and
(rho e_tot, u_h) blocks) and the DSS of the Laplacians' covariant 3-vector.

Pinned by properties that hold for the reference's formulation whatever ClimaCore's
arithmetic order: a flat surface reproduces the flat-geometry oracle, the flux-form
tendencies conserve mass and energy, the filter zeroes the contravariant u^3 on both
boundary faces, the Jacobian's mass row is exact against central differences in every
direction it claims (u_3 and u_h), ldiv inverts the stored Jacobian, and the C123 DSS is a
projection."""
import numpy as np
import pytest

import oracle as O
import topography as T
from geometry import OracleGeometry
from gbdycore import config as C
from gbdycore import setups as S


def _grid(h=3, z=8, zs=None, warp=None):
    cfg = C.DycoreConfig(h_elem=h, z_elem=z, z_max=30000.0, z_stretch=True, dz_bottom=300.0, dt=200.0,
                         ft=np.float64)
    g = OracleGeometry(cfg.h_elem, cfg.z_elem, cfg.z_max, cfg.z_stretch, cfg.dz_bottom)
    if zs is not None:
        g.terrain = T.oracle_terrain(g, zs(g), warp or T.LinearWarp())
    return cfg, g


def _hill(g):
    return T.smooth_surface(g.xyz)


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_flat_surface_reproduces_the_flat_oracle():
    cfg, g0 = _grid()
    _, g1 = _grid(zs=lambda g: np.zeros((g.Nh, 16)))
    p = cfg.oracle_params(dss_stage1=False)
    o0, o1 = O.Oracle(g0, p), O.Oracle(g1, p)
    Yc, Yf = S.workload_state(g0, cfg, "plain")
    a, b = o0.remaining_tendency(Yc.copy(), Yf.copy()), o1.remaining_tendency(Yc.copy(), Yf.copy())
    for c in range(4):
        assert _rel(b[0][:, c], a[0][:, c]) < 1e-13
    assert _rel(b[1], a[1]) < 1e-13
    r0c, r0f = Yc.copy(), Yf.copy()
    r1c, r1f = Yc.copy(), Yf.copy()
    o0.step(r0c, r0f, cfg.dt, 2)
    o1.step(r1c, r1f, cfg.dt, 2)
    for c in range(4):
        assert _rel(r1c[:, c], r0c[:, c]) < 1e-12
    assert _rel(r1f, r0f) < 1e-10  # u_3 ~ 1e-3 of its scale: the metric's roundoff, relatively


@pytest.mark.parametrize("warp", [T.LinearWarp(), T.SLEVEWarp()])
def test_tendencies_conserve_mass_and_energy_over_terrain(warp):
    cfg, g = _grid(4, 10, _hill, warp)
    o = O.Oracle(g, cfg.oracle_params(dss_stage1=False))
    Yc, Yf = S.workload_state(g, cfg, "plain")
    WJ = g.W[None, :, None] * g.terrain["Jc"]
    for Tc, _ in (o.remaining_tendency(Yc.copy(), Yf.copy()), o.implicit_tendency(Yc.copy(), Yf.copy())):
        for c in (0, 3):
            assert abs((Tc[:, c] * WJ).sum()) <= 1e-14 * (np.abs(Tc[:, c]) * WJ).sum()
    s0 = o.global_sums(Yc)
    o.step(Yc, Yf, cfg.dt, 3)
    assert np.isfinite(Yc).all() and np.isfinite(Yf).all()
    assert np.all(np.abs(o.global_sums(Yc) - s0) <= 1e-13 * np.abs(s0))


def test_filter_zeroes_contravariant_u3_on_both_faces():
    cfg, g = _grid(3, 8, _hill)
    o = O.Oracle(g, cfg.oracle_params(dss_stage1=False))
    Yc, Yf = S.workload_state(g, cfg, "plain")
    Yf[:] = 1.0
    o.set_precomputed(Yc, Yf)
    gu, gf = g.terrain["guc"], g.terrain["guf"]
    for k, v in ((0, 0), (-1, -1)):
        ct3 = gu[..., v, 3] * Yc[:, 1, :, v] + gu[..., v, 4] * Yc[:, 2, :, v]
        u3 = ct3 + gf[..., k, 5] * Yf[..., k]
        assert np.abs(u3).max() <= 1e-13 * np.abs(ct3).max()
    assert np.abs(Yf[..., 0]).max() > 0   # the terrain makes it nonzero


def test_ldiv_inverts_the_stored_jacobian_over_terrain():
    cfg, g = _grid(3, 8, _hill)
    o = O.Oracle(g, cfg.oracle_params(dss_stage1=False))
    Yc, Yf = S.workload_state(g, cfg, "plain")
    o.update_jacobian(Yc.copy(), Yf.copy(), 50.0)
    rng = np.random.default_rng(5)
    Rc = rng.standard_normal(Yc.shape) * np.abs(Yc).max(axis=(0, 2, 3), keepdims=True)
    Rf = rng.standard_normal(Yf.shape) * 10.0
    Xc, Xf = o.ldiv(Rc, Rf)
    Oc, Of = o.jac_apply(Xc, Xf)
    # the bounds of the flat-geometry check (test_oracle_invariants): the acoustic Schur system's
    # entries reach (c dtγ / dz)^2, so the attainable face residual is ~1e3 eps of |W| |x|
    for c in range(4):
        assert _rel(Oc[:, c], Rc[:, c]) < 1e-9
    assert _rel(Of, Rf) < 1e-6
    # the (rho, u_h) blocks take part: zeroing R_uh changes the rho rows of the solution
    Rc2 = Rc.copy()
    Rc2[:, 1:3] = 0.0
    assert _rel(o.ldiv(Rc2, Rf)[0][:, 0], Xc[:, 0]) > 1e-8


@pytest.mark.parametrize("comp", ["u3", "uh"])
def test_jacobian_mass_row_is_exact_over_terrain(comp):
    """The mass tendency is linear in u_3 and (through u_h^3) in u_h away from the two levels
    the impenetrable filter reads: the stored (rho, u_3) and (rho, u_h) blocks times a
    direction equal the central difference of dtγ T_rho."""
    cfg, g = _grid(3, 8, _hill)
    o = O.Oracle(g, cfg.oracle_params(dss_stage1=False))
    Yc, Yf = S.workload_state(g, cfg, "plain")
    Yf[..., 1:-1] = np.random.default_rng(1).standard_normal(Yf[..., 1:-1].shape) * 5.0
    dtg = 40.0
    o.update_jacobian(Yc.copy(), Yf.copy(), dtg)
    rng = np.random.default_rng(2)
    Vc, Vf = np.zeros_like(Yc), np.zeros_like(Yf)
    if comp == "u3":
        Vf[..., 1:-1] = rng.standard_normal(Vf[..., 1:-1].shape)
    else:
        Vc[:, 1:3, :, 1:-1] = rng.standard_normal(Vc[:, 1:3, :, 1:-1].shape) * np.abs(Yc[:, 1:3]).max()
    Oc, _ = o.jac_apply(Vc, Vf)
    h = 1e-3
    Tp, _ = o.implicit_tendency(Yc + h * Vc, Yf + h * Vf)
    Tm, _ = o.implicit_tendency(Yc - h * Vc, Yf - h * Vf)
    fd = dtg * (Tp[:, 0] - Tm[:, 0]) / (2 * h) - Vc[:, 0]
    assert _rel(Oc[:, 0], fd) < 1e-9


def test_c123_dss_is_a_projection_and_reduces_to_the_flat_form():
    """The DSS of the Laplacians' covariant 3-vector: idempotent over terrain, equal to the flat
    form (Cartesian horizontal vector, scalar third component) over a flat surface, and the
    collocated copies of a node describe one Cartesian vector after it."""
    cfg, g = _grid(3, 6, _hill)
    o = O.Oracle(g, cfg.oracle_params(dss_stage1=False))
    rng = np.random.default_rng(3)
    X = rng.standard_normal((g.Nh, 4, 16, g.Nv))
    A = X.copy()
    o.dss_c123(A)
    B = A.copy()
    o.dss_c123(B)
    assert _rel(B, A) < 2e-12
    Ecn = g.terrain["Ecn"].reshape(g.Nh, 16, g.Nv, 3, 3)
    V = np.einsum("eInv,envId->envd", A[:, 1:4], Ecn)      # Cartesian vector per copy
    key = np.round(g.xyz.reshape(-1, 3) * 1e9).astype(np.int64)
    _, inv = np.unique(key, axis=0, return_inverse=True)
    Vn = V.reshape(-1, g.Nv, 3)
    for u in np.unique(inv)[:50]:
        idx = np.nonzero(inv.reshape(-1) == u)[0]
        assert np.abs(Vn[idx] - Vn[idx[0]]).max() <= 1e-12 * np.abs(Vn).max()
    _, g0 = _grid(3, 6)
    _, gz = _grid(3, 6, lambda g: np.zeros((g.Nh, 16)))
    o0, oz = O.Oracle(g0, cfg.oracle_params()), O.Oracle(gz, cfg.oracle_params())
    F0, Fz = X.copy(), X.copy()
    o0.dss_c123(F0)
    oz.dss_c123(Fz)
    assert _rel(Fz, F0) < 2e-12

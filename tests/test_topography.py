"""Surface-elevation profiles and terrain-following warps of the oracle (the first piece of
the topography extension), pinned to the reference's known answers in test/topography.jl,
and the warps' properties on the production grid (CPU only)."""
import numpy as np
import pytest

import topography as T
from geometry import OracleGeometry, vertical_faces


def test_dcmip200_on_the_cubed_sphere():
    # test/topography.jl:11-22: extrema (0, 2000), the peak on the equator at -90 longitude
    g = OracleGeometry(4, 2)
    lat, lon = np.degrees(g.lat), np.degrees(g.lon)
    z = T.dcmip200(lat, lon)
    assert z.min() == 0.0 and abs(z.max() - 2000.0) < 1e-9
    k = np.unravel_index(np.argmax(z), z.shape)
    assert abs(lat[k]) < 1e-9 and abs(lon[k] + 90.0) < 1e-9


def test_hughes2023_on_the_cubed_sphere():
    # test/topography.jl:24-34: within [0, 2000], no NaN
    g = OracleGeometry(6, 2)
    z = T.hughes2023(np.degrees(g.lat), np.degrees(g.lon))
    assert np.all(np.isfinite(z)) and z.min() >= 0.0 and z.max() <= 2000.0


def test_cosine_known_answers():
    # test/topography.jl:36-60
    t3 = T.CosineTopography(dim=3, h_max=100.0, lam=1000.0)
    assert t3(0.0, 0.0) == 100.0
    assert abs(t3(500.0, 0.0) + 100.0) <= np.finfo(np.float64).eps
    t2 = T.CosineTopography(dim=2, h_max=50.0, lam=2000.0)
    assert t2(0.0) == 50.0
    assert abs(t2(1000.0) + 50.0) <= np.finfo(np.float64).eps


def test_agnesi_and_schar_known_answers():
    # test/topography.jl:62-91
    a = T.AgnesiTopography(h_max=1000.0, x_center=500.0, a=100.0)
    assert a(500.0) == 1000.0 and a(600.0) == 500.0 and a(0.0) < 50.0
    s = T.ScharTopography(h_max=500.0, x_center=1000.0, lam=200.0, a=100.0)
    assert s(1000.0) == 500.0
    assert abs(s(1100.0)) <= 1e-6
    assert np.all(s(np.arange(0.0, 2001.0, 100.0)) >= 0.0)


def test_warp_defaults_and_parameters():
    # test/topography.jl:93-101 and the defaults at src/topography/topography.jl:304-307
    assert T.SLEVEWarp() == T.SLEVEWarp(eta=0.7, s=10.0)
    w = T.SLEVEWarp(eta=0.8, s=12.0)
    assert w.eta == 0.8 and w.s == 12.0


@pytest.mark.parametrize("warp", [T.LinearWarp(), T.SLEVEWarp()])
def test_warped_production_columns(warp):
    """Over the DCMIP200 mountain on the production levels (63, tanh-stretched from 30 m):
    the bottom face follows the surface, the top stays at z_top, levels stay ordered, and a
    flat surface leaves the levels unchanged."""
    zf = vertical_faces(63, 30000.0, True, 30.0)
    g = OracleGeometry(4, 2)
    zs = T.dcmip200(np.degrees(g.lat), np.degrees(g.lon))
    Z = T.warped_faces(zf, zs, warp)
    assert Z.shape == zs.shape + (64,)
    np.testing.assert_allclose(Z[..., 0], zs, rtol=0, atol=1e-9)
    np.testing.assert_allclose(Z[..., -1], 30000.0, rtol=0, atol=1e-9)
    assert np.all(np.diff(Z, axis=-1) > 0)
    np.testing.assert_allclose(T.warped_faces(zf, np.zeros(3), warp), np.broadcast_to(zf, (3, 64)), atol=1e-9)


def test_sleve_flat_above_eta_and_refuses_high_terrain():
    zf = np.linspace(0.0, 1000.0, 11)
    Z = T.warped_faces(zf, np.array([100.0]), T.SLEVEWarp(eta=0.5, s=2.0))[0]
    np.testing.assert_array_equal(Z[zf / 1000.0 > 0.5], zf[zf / 1000.0 > 0.5])
    assert np.all(Z[zf / 1000.0 < 0.5] > zf[zf / 1000.0 < 0.5])
    with pytest.raises(ValueError):
        T.warped_faces(zf, np.array([2500.0]), T.SLEVEWarp(eta=0.5, s=2.0))


# ---------------------------------------------------------------- terrain-following geometry
def _grid(h=4, z=8):
    g = OracleGeometry(h, z, 30000.0, True, 300.0)
    return g, T.dcmip200(np.degrees(g.lat), np.degrees(g.lon))


def test_flat_surface_reproduces_the_flat_geometry():
    g, _ = _grid(2, 4)
    G = T.warped_geometry(g, np.zeros((g.Nh, 16)), T.LinearWarp())
    Jc = g.Jh[:, :, None] * (g.rc ** 2 * g.dzc)[None, None, :]
    Jf = g.Jh[:, :, None] * (g.rf ** 2 * g.dzf)[None, None, :]
    np.testing.assert_allclose(G["Jc"], Jc, rtol=1e-13)
    np.testing.assert_allclose(G["Jf"], Jf, rtol=1e-13)
    gu = G["gup_f"]
    np.testing.assert_allclose(gu[..., 2, 2], np.broadcast_to(1 / g.dzf ** 2, gu.shape[:3]), rtol=1e-12)
    assert np.abs(gu[..., 2, :2]).max() < 1e-14 * np.abs(gu[..., 2, 2]).max()
    scale = np.abs(gu[..., 0, 0]).max()
    for (a, b), c in (((0, 0), 0), ((0, 1), 1), ((1, 1), 2)):
        np.testing.assert_allclose(gu[..., a, b], g.gup[:, :, None, c] / (g.rf ** 2)[None, None, :],
                                   rtol=1e-12, atol=1e-13 * scale)


@pytest.mark.parametrize("warp", [T.LinearWarp(), T.SLEVEWarp()])
def test_warped_jacobian_and_column_volume(warp):
    g, zs = _grid()
    G = T.warped_geometry(g, zs, warp)
    R = g.R
    dzc = G["zf"][..., 1:] - G["zf"][..., :-1]
    # E_3 is radial, so J = dz r^2 J_h whatever the slopes
    np.testing.assert_allclose(G["Jc"], dzc * ((R + G["zc"]) / R) ** 2 * g.Jh[:, :, None], rtol=1e-12)
    # the column integral of r^2 dz from the surface to the top (midpoint rule)
    vol = (G["Jc"] / g.Jh[:, :, None]).sum(axis=-1)
    exact = ((R + 30000.0) ** 3 - (R + zs) ** 3) / (3 * R * R)
    np.testing.assert_allclose(vol, exact, rtol=1e-6)


def test_terrain_following_flow_has_no_contravariant_u3_at_the_surface():
    # a velocity in the tangent plane of the bottom face (spanned by E_1, E_2) has u^3 = 0:
    # the impenetrable condition u_3 = -(g^31 u_1 + g^32 u_2) / g^33 of a sloping surface
    g, zs = _grid()
    G = T.warped_geometry(g, zs, T.LinearWarp())
    E = G["Ef"][:, :, 0]                                          # [Nh, 16, 3, 3]
    rng = np.random.default_rng(3)
    a, b = rng.standard_normal((2,) + E.shape[:2])
    v = a[..., None] * E[..., 0, :] + b[..., None] * E[..., 1, :]
    u = np.einsum("enik,enk->eni", E, v)                           # covariant components
    u3 = np.einsum("enj,enj->en", G["gup_f"][:, :, 0, 2, :], u)
    scale = np.abs(np.einsum("enj,enj->en", G["gup_f"][:, :, 0, 2, :], np.abs(u))).max()
    assert np.abs(u3).max() <= 1e-12 * scale
    assert np.abs(zs).max() > 1000.0                              # the mountain is in the grid


def test_linear_warp_slopes_decay_linearly():
    g, zs = _grid()
    G = T.warped_geometry(g, zs, T.LinearWarp())
    zz = zs.reshape(g.Nh, 4, 4)
    ds1 = np.einsum("ik,ejk->eji", g.D, zz).reshape(g.Nh, 16)
    for k in (0, 3, 8):
        slope = np.einsum("enk,enk->en", G["Ef"][:, :, k, 0, :], g.xyz)   # E_1 . x_hat = dz/dxi^1
        np.testing.assert_allclose(slope, (1 - g.zf[k] / 30000.0) * ds1, atol=1e-9 * np.abs(ds1).max())


def test_impenetrable_u3_over_terrain():
    # set_velocity_at_surface!/top! (src/cache/precomputed_quantities.jl:473-547)
    g, zs = _grid()
    rng = np.random.default_rng(5)
    shape = (g.Nh, 16, g.Nv)
    rho, u1, u2 = np.ones(shape), rng.standard_normal(shape), rng.standard_normal(shape)
    flat = T.warped_geometry(g, np.zeros_like(zs), T.LinearWarp())
    assert np.abs(T.impenetrable_u3(flat, rho, u1, u2)).max() < 1e-12     # no terrain: u_3 = 0
    G = T.warped_geometry(g, zs, T.LinearWarp())
    u3 = T.impenetrable_u3(G, rho, u1, u2)
    # linear in u_h, nonzero over the mountain
    np.testing.assert_allclose(T.impenetrable_u3(G, rho, 2 * u1, 2 * u2), 2 * u3, rtol=1e-14, atol=1e-300)
    assert np.abs(u3[..., 0]).max() > 0
    # u^3 = u_h^3 + g^33 u_3 vanishes on the bottom face (u_h^3 extrapolated from the first centre)
    uh3 = G["gup_c"][..., 0, 2, 0] * u1[..., 0] + G["gup_c"][..., 0, 2, 1] * u2[..., 0]
    np.testing.assert_allclose(uh3 + G["gup_f"][..., 0, 2, 2] * u3[..., 0], 0, atol=1e-12 * np.abs(uh3).max())


def test_impenetrable_u3_zeroes_contravariant_u3_on_both_faces():
    # u^3 = ᶠwinterp(rho J, u_h^3) + g^33 u_3 must vanish on the bottom and the top face for any
    # rho and u_h over DCMIP200 terrain; the weights are checked to drop out only at those faces
    g, zs = _grid()
    rng = np.random.default_rng(9)
    shape = (g.Nh, 16, g.Nv)
    rho = np.exp(rng.normal(size=shape))
    u1, u2 = rng.standard_normal(shape), rng.standard_normal(shape)
    for warp in (T.LinearWarp(), T.SLEVEWarp()):
        G = T.warped_geometry(g, zs, warp)
        u3 = T.impenetrable_u3(G, rho, u1, u2)
        uh3 = G["gup_c"][..., 2, 0] * u1 + G["gup_c"][..., 2, 1] * u2
        uh3f = T.winterp_faces(rho * G["Jc"], uh3)
        for side, k in ((0, 0), (1, -1)):
            contra = uh3f[..., k] + G["gup_f"][..., k, 2, 2] * u3[..., side]
            assert np.abs(contra).max() <= 1e-12 * np.abs(uh3).max(), (warp, side)
        assert np.abs(u3).max() > 0
        # interior faces: the weights matter (a uniform weight gives another value)
        plain = T.winterp_faces(np.ones_like(rho), uh3)
        assert np.abs(plain[..., 1:-1] - uh3f[..., 1:-1]).max() > 1e-6 * np.abs(uh3).max()
        np.testing.assert_array_equal(plain[..., [0, -1]], uh3f[..., [0, -1]])

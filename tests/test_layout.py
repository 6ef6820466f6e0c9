"""The caller's element layout (gb_config.elem_map / elem_orient, gb_match_elements) on
the host: the library's geometry tables and DSS plan built in a permuted, rotated-frame
layout are the library-order ones moved to the caller's (element, node) and turned to the
caller's covariant basis; the matcher recovers the layout from node positions alone.
ClimaCore numbers elements along a space-filling curve (src/simulation/grids.jl:74-75)
with per-element frames, which is why the drop-in boundary needs this (CPU only)."""
import ctypes

import numpy as np
import pytest

from gbdycore import _native as N
from gbdycore import config as C
from gbdycore import layout as LY
from gbdycore.simulation import Geometry


def _cfg(h=3):
    return C.DycoreConfig(h_elem=h, z_elem=6, z_stretch=True, dz_bottom=300.0, ft=np.float64)


@pytest.mark.parametrize("rotate", [False, True])
def test_geometry_in_a_caller_layout(rotate):
    cfg = _cfg()
    emap, eori = LY.random_layout(cfg.h_elem, seed=3, rotate=rotate)
    g0, g1 = Geometry(cfg), Geometry(cfg.with_(layout=(emap, eori)))
    nodes = LY.NODE_OF[eori]
    # positions and J_h: the library's, moved (exactly)
    np.testing.assert_array_equal(g1.xyz, g0.xyz[emap[:, None], nodes])
    np.testing.assert_array_equal(g1.Jh, g0.Jh[emap[:, None], nodes])
    # covariant basis on the caller's frame: e'_k = sum_m R_km e_m
    e0 = g0.ecov[emap[:, None], nodes]                                   # [Nh, 16, 2, 3]
    R = LY.ROT[eori]
    np.testing.assert_array_equal(g1.ecov, np.einsum("ekm,enmd->enkd", R, e0))
    # the contravariant metric follows: g'^{-1} = R g^{-1} R^T
    def full(gu):
        return np.stack([np.stack([gu[..., 0], gu[..., 1]], -1), np.stack([gu[..., 1], gu[..., 2]], -1)], -2)
    G0 = full(g0.gup[emap[:, None], nodes])
    G1 = np.einsum("ekm,enml,ejl->enkj", R, G0, R)
    np.testing.assert_allclose(full(g1.gup), G1, rtol=1e-13, atol=0)
    # DSS: the same groups of physical nodes, each in the library's order
    np.testing.assert_array_equal(g1.dss_off, g0.dss_off)
    inv = np.empty(g1.Nh, np.int64)
    inv[emap] = np.arange(g1.Nh)
    lib_of = emap[g1.dss_copy // 16] * 16 + nodes[g1.dss_copy // 16, g1.dss_copy % 16]
    np.testing.assert_array_equal(lib_of, g0.dss_copy)


def test_layout_maps_invert():
    cfg = _cfg(2)
    emap, eori = LY.random_layout(cfg.h_elem, seed=1)
    rng = np.random.default_rng(0)
    Yc, Yf = rng.normal(size=(24, 4, 16, 5)), rng.normal(size=(24, 16, 6))
    Xc, Xf = LY.to_caller(Yc, Yf, emap, eori)
    Zc, Zf = LY.from_caller(Xc, Xf, emap, eori)
    np.testing.assert_array_equal(Zc, Yc)
    np.testing.assert_array_equal(Zf, Yf)
    # covariant components: u'_k = u . e'_k on the caller's basis
    g0 = Geometry(cfg)
    g1 = Geometry(cfg.with_(layout=(emap, eori)))
    gu = g0.gup
    # the physical horizontal vector of a library node: u^i e_i with u^i = g^ij u_j
    def vec(g, c):
        u1, u2 = c[:, 1, :, 0], c[:, 2, :, 0]
        a1 = g.gup[..., 0] * u1 + g.gup[..., 1] * u2
        a2 = g.gup[..., 1] * u1 + g.gup[..., 2] * u2
        return a1[..., None] * g.ecov[:, :, 0] + a2[..., None] * g.ecov[:, :, 1]
    v0 = vec(g0, Yc)
    v1 = vec(g1, Xc)
    nodes = LY.NODE_OF[eori]
    np.testing.assert_allclose(v1, v0[emap[:, None], nodes], rtol=1e-12, atol=1e-12 * np.abs(v0).max())
    del gu


def test_match_elements_recovers_the_layout():
    cfg = _cfg(4)
    emap, eori = LY.random_layout(cfg.h_elem, seed=7)
    g1 = Geometry(cfg.with_(layout=(emap, eori)))
    # positions at another radius, with roundoff noise: still matched
    xyz = g1.xyz * 6.4e6 * (1 + 1e-13 * np.random.default_rng(0).normal(size=g1.xyz.shape))
    m, o = N.match_elements(cfg, xyz)
    np.testing.assert_array_equal(m, emap)
    np.testing.assert_array_equal(o, eori)
    # the library's own order
    m, o = N.match_elements(cfg, Geometry(cfg).xyz)
    np.testing.assert_array_equal(m, np.arange(len(m)))
    assert not o.any()


def test_match_elements_refuses_mirrored_frames_and_duplicates():
    cfg = _cfg(2)
    xyz = Geometry(cfg).xyz.copy()
    bad = xyz.copy()
    e = 5
    bad[e] = bad[e].reshape(4, 4, 3).transpose(1, 0, 2).reshape(16, 3)     # i <-> j: a mirrored frame
    with pytest.raises(N.GBError):
        N.match_elements(cfg, bad)
    dup = xyz.copy()
    dup[1] = dup[0]
    with pytest.raises(N.GBError):
        N.match_elements(cfg, dup)
    with pytest.raises(N.GBError):
        N.match_elements(cfg.with_(h_elem=3), np.resize(xyz, (54, 16, 3)))


def test_invalid_layouts_are_rejected():
    L = N.load()
    cfg = _cfg(2)
    Nh = 24
    for emap, eori in [(np.zeros(Nh), np.zeros(Nh)), (np.arange(Nh), np.full(Nh, 4)),
                       (np.arange(Nh) + 1, np.zeros(Nh))]:
        c = N.make_config(cfg.with_(layout=(emap, eori)))
        n = ctypes.c_size_t()
        assert L.gb_sizes(ctypes.byref(c), ctypes.byref(n), None, None, None) == N.GB_ERR_ARG
    c = N.make_config(cfg.with_(layout=(np.arange(Nh), np.zeros(Nh))))
    c.elem_orient = None
    assert L.gb_sizes(ctypes.byref(c), None, None, None, None) == N.GB_ERR_ARG

"""Terrain-following configurations at the C ABI (no GPU needed): gb_sizes validates the
surface and the warp, and the host's centre heights are the oracle's."""
import ctypes

import numpy as np
import pytest

import topography as T
from geometry import OracleGeometry
from gbdycore import _native as N
from gbdycore import simulation as sim
from helpers import small_config


def _sizes(cfg):
    c = N.make_config(cfg)
    return N.load().gb_sizes(ctypes.byref(c), None, None, None, None)


def test_terrain_config_validation():
    cfg = small_config(h_elem=2, z_elem=6)
    Nh = 6 * 2 * 2
    hill = np.full((Nh, 16), 1500.0)
    assert _sizes(cfg.with_(z_surface=hill)) == N.GB_OK
    assert _sizes(cfg.with_(z_surface=hill, warp="sleve")) == N.GB_OK
    # levels that cross (a surface at z_max leaves the linear warp's layers no thickness)
    assert _sizes(cfg.with_(z_surface=np.full((Nh, 16), cfg.z_max))) == N.GB_ERR_ARG
    # SLEVE needs s z_top above the highest surface (topography.jl:295-297)
    assert _sizes(cfg.with_(z_surface=hill, warp="sleve", sleve_s=0.01)) == N.GB_ERR_ARG
    bad = hill.copy()
    bad[3, 5] = np.nan
    assert _sizes(cfg.with_(z_surface=bad)) == N.GB_ERR_ARG
    # the Held-Suarez forcing is not built over terrain
    assert _sizes(cfg.with_(z_surface=hill, held_suarez=True)) == N.GB_ERR_ARG


@pytest.mark.parametrize("warp", ["linear", "sleve"])
def test_centre_heights_match_the_oracle(warp):
    cfg = small_config(h_elem=3, z_elem=8)
    g = OracleGeometry(cfg.h_elem, cfg.z_elem, cfg.z_max, cfg.z_stretch, cfg.dz_bottom)
    zs = T.dcmip200_nodes(g.xyz)
    G = T.warped_geometry(g, zs, T.LinearWarp() if warp == "linear" else T.SLEVEWarp())
    zc = sim.terrain_centre_heights(cfg.with_(z_surface=zs, warp=warp), g.zf)
    assert np.abs(zc - G["zc"]).max() < 1e-9

"""Product grid (C++, libgbdycore) against the independent oracle grid (numpy)."""
import math

import numpy as np
import pytest

from gbdycore import config as C
from gbdycore.simulation import Geometry
from helpers import oracle_geometry


@pytest.mark.parametrize("cfg", [C.plain_h6(), C.production_h30().with_(h_elem=4), C.differentiation_h16().with_(h_elem=2)])
def test_product_geometry_matches_oracle(cfg):
    g, o = Geometry(cfg), oracle_geometry(cfg)
    for k in ["xyz", "ecov", "Jh", "gup", "fh0", "zf"]:
        a, b = getattr(g, k), getattr(o, k)
        assert np.abs(a - b).max() <= 1e-14 * max(np.abs(b).max(), 1.0), k
    assert np.array_equal(g.dss_off, o.dss_off)
    assert np.array_equal(g.dss_copy, o.dss_copy)


def test_sphere_area_and_node_count():
    o = oracle_geometry(C.plain_h6())
    area = (o.W[None, :] * o.Jh).sum()
    assert abs(area / (4 * math.pi * o.R ** 2) - 1) < 1e-7
    M = 3 * o.h
    assert o.unique_nodes == 6 * M * M + 2
    sizes = np.bincount(np.diff(o.dss_off))
    assert sizes[3] == 8            # the cube corners
    assert sizes.sum() == len(o.dss_off) - 1


def test_stretched_levels():
    cfg = C.production_h30()
    g = Geometry(cfg)
    assert abs(g.zf[1] - cfg.dz_bottom) < 1e-6 * cfg.dz_bottom
    assert g.zf[-1] == cfg.z_max and np.all(np.diff(g.zf) > 0)

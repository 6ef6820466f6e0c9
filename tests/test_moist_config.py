"""Moist 0M configurations at the C ABI (no GPU needed): gb_sizes reports the five-component
centre block and validates the moist constants; moist 0M over terrain, with the Held-Suarez
forcing or with the batched columns is refused."""
import ctypes

import numpy as np

from gbdycore import _native as N
from gbdycore import config as C
from helpers import small_config


def _sizes(cfg):
    c = N.make_config(cfg)
    nc, nf = ctypes.c_size_t(), ctypes.c_size_t()
    rc = N.load().gb_sizes(ctypes.byref(c), ctypes.byref(nc), ctypes.byref(nf), None, None)
    return rc, nc.value, nf.value


def test_moist_sizes_carry_rho_q_tot():
    cfg = small_config(h_elem=2, z_elem=6)
    Nh = 6 * 2 * 2
    rc, nc, nf = _sizes(cfg)
    assert rc == N.GB_OK and nc == Nh * 4 * 16 * 6 and nf == Nh * 16 * 7
    rc, nc, nf = _sizes(cfg.with_(moist=True))
    assert rc == N.GB_OK and nc == Nh * 5 * 16 * 6 and nf == Nh * 16 * 7


def test_moist_constants_are_validated():
    cfg = small_config(h_elem=2, z_elem=6, moist=True)
    for key, bad in (("R_v", 0.0), ("LH_s0", 1.0e6), ("T_icenuc", 300.0), ("pow_icenuc", 0.0), ("press_triple", -1.0)):
        m = dict(C.MOIST)
        m[key] = bad
        assert _sizes(cfg.with_(moist_constants=m))[0] == N.GB_ERR_ARG, key
    for it in (0, 101):
        assert _sizes(cfg.with_(sa_iters=it))[0] == N.GB_ERR_ARG, it
    assert _sizes(cfg.with_(sa_iters=1))[0] == N.GB_OK


def test_moist_refuses_terrain_and_held_suarez():
    cfg = small_config(h_elem=2, z_elem=6, moist=True)
    hill = np.full((6 * 4, 16), 1000.0)
    assert _sizes(cfg.with_(z_surface=hill))[0] == N.GB_ERR_ARG
    assert _sizes(cfg.with_(held_suarez=True))[0] == N.GB_ERR_ARG


def test_batched_columns_refuse_moist():
    cfg = small_config(h_elem=2, z_elem=6, moist=True)
    c = N.make_config(cfg)
    z = (ctypes.c_int * 2)(8, 10)
    h = ctypes.c_void_p()
    L = N.load()
    assert L.gb_columns_create(ctypes.byref(c), 2, z, ctypes.byref(h)) == N.GB_ERR_ARG
    assert not h.value

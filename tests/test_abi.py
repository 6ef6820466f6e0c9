"""The C-ABI library builds, loads and exports every symbol include/gbdycore.h declares (no GPU needed)."""
import ctypes
import os
import re

import numpy as np

from gbdycore import _native as N
from gbdycore import config as C
from conftest import ROOT


def header_symbols():
    src = open(os.path.join(ROOT, "include", "gbdycore.h")).read()
    return sorted(set(re.findall(r"^int\s+(gb_\w+)\s*\(", src, flags=re.M)))


def test_header_declares_the_bound_symbols():
    assert header_symbols() == sorted(N.SYMBOLS)


def test_library_loads_and_exports_every_symbol():
    L = N.load()
    for s in header_symbols():
        assert hasattr(L, s), s
        assert ctypes.cast(getattr(L, s), ctypes.c_void_p).value


def test_invalid_configs_are_rejected():
    L = N.load()
    base = C.plain_h6()
    for bad in [dict(h_elem=0), dict(z_elem=1), dict(z_elem=500), dict(ft=np.float16), dict(z_stretch=True, dz_bottom=1e5)]:
        cfg = base.with_(**bad) if "ft" not in bad else base
        c = N.make_config(cfg)
        if "ft" in bad:
            c.ft_bytes = 2
        n = ctypes.c_size_t()
        assert L.gb_sizes(ctypes.byref(c), ctypes.byref(n), None, None, None) == N.GB_ERR_ARG
        h = ctypes.c_void_p()
        assert L.gb_ctx_create(ctypes.byref(c), ctypes.byref(h)) == N.GB_ERR_ARG
        assert not h.value


def test_null_context_is_rejected():
    L = N.load()
    fv = N.GBFieldVec(None, None)
    assert L.gb_dss(None, fv) == N.GB_ERR_ARG
    assert L.gb_step(None, fv, 0.0, 1.0, 1, 0) == N.GB_ERR_ARG
    assert L.gb_ctx_destroy(None) == N.GB_ERR_ARG


def test_sizes():
    L = N.load()
    cfg = C.production_h30()
    c = N.make_config(cfg)
    nc, nf = ctypes.c_size_t(), ctypes.c_size_t()
    ng, ncp = ctypes.c_int(), ctypes.c_int()
    assert L.gb_sizes(ctypes.byref(c), ctypes.byref(nc), ctypes.byref(nf), ctypes.byref(ng), ctypes.byref(ncp)) == 0
    Nh = 6 * 30 * 30
    assert nc.value == Nh * 4 * 16 * 63 and nf.value == Nh * 16 * 64
    # every element boundary node is shared: 12 per element
    assert ncp.value == Nh * 12

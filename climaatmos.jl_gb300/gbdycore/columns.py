"""Batched standalone columns of uneven height (``gb_columns_*`` of the C ABI).

A batch of independent dry ``ColumnGrid`` columns (src/simulation/grids.jl:93-127,
flat column metric), each with its own ``z_elem``, solved on the GPU by Newton on
the implicit stage equation ``U = U^ + dtgamma T_imp(U)`` — the column part of the
IMEX step (implicit_tendency! residual, update_jacobian! blocks and the
BlockArrowheadSolve of manual_sparse_jacobian.jl:580-583), as
``NewtonsMethod(max_iters = n, update_j = UpdateEvery(NewNewtonIteration))``
drives it (src/simulation/integrator.jl:63-120).

State layout (``C`` = total centres): ``c`` is ``[4, C]`` (rho, u_1, u_2,
rho e_tot), column ``k`` at ``offsets[k] .. offsets[k] + z_elem[k]``; ``f`` is
``[C + ncols]`` (u_3), column ``k`` at ``offsets[k] + k .. offsets[k] + k + z_elem[k]``.
"""
import ctypes

import numpy as np

from . import _native as N
from .setups import temperature_pressure
from .simulation import FieldVector

MODES = {"graph": N.GB_COLUMNS_GRAPH, "persistent": N.GB_COLUMNS_PERSISTENT, "per_height": N.GB_COLUMNS_PER_HEIGHT}


def _check(h, rc):
    if rc != N.GB_OK:
        msg = ""
        if h:
            buf = ctypes.create_string_buffer(512)
            N.load().gb_columns_last_error(h, buf, 512)
            msg = buf.value.decode(errors="replace")
        raise N.GBError(rc, msg or "call failed")


def offsets(z_elem):
    """Centre offset of every column (its faces start at offset + column index)."""
    z = np.asarray(z_elem, dtype=np.int64)
    return np.concatenate([[0], np.cumsum(z)[:-1]]).astype(np.int64)


def column_faces(cfg, z):
    """Face heights of a column of ``z`` levels (uniform or tanh-stretched like the library)."""
    if not cfg.z_stretch:
        return cfg.z_max * np.arange(z + 1) / z
    target = cfg.dz_bottom / cfg.z_max
    first = lambda g: 1.0 + np.tanh(g * (1.0 / z - 1.0)) / np.tanh(g)
    lo, hi = 1e-8, 50.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if first(mid) > target:
            lo = mid
        else:
            hi = mid
    g = 0.5 * (lo + hi)
    zf = cfg.z_max * (1.0 + np.tanh(g * (np.arange(z + 1) / z - 1.0)) / np.tanh(g))
    zf[0], zf[-1] = 0.0, cfg.z_max
    return zf


def batch_state(cfg, z_elem, seed=2, w_sigma=0.5, rhoe_rel=0.005, dtype=None):
    """Balanced lapse-rate columns with a seeded vertical-velocity perturbation
    w ~ N(0, w_sigma) m/s on the interior faces (u_3 = w dz_f, the covariant
    component on the flat column) and rho e_tot scaled by 1 + rhoe_rel N(0, 1).
    Returns (c [4, C], f [C + ncols]) as numpy arrays."""
    c = cfg.constants
    dtype = np.dtype(dtype or cfg.ft)
    z_elem = np.asarray(z_elem, dtype=np.int64)
    off = offsets(z_elem)
    C = int(z_elem.sum())
    Yc = np.zeros((4, C))
    Yf = np.zeros(C + len(z_elem))
    rng = np.random.default_rng(seed + 1000)
    for k, z in enumerate(z_elem):
        zf = column_faces(cfg, int(z))
        zc = 0.5 * (zf[1:] + zf[:-1])
        T, p = temperature_pressure(zc, c)
        rho = p / (c["R_d"] * T)
        eint = c["cv_d"] * (T - c["T_0"]) - c["R_d"] * c["T_0"]
        rhoe = rho * (eint + c["grav"] * zc) * (1.0 + rhoe_rel * rng.standard_normal(z))
        s = slice(off[k], off[k] + z)
        Yc[0, s] = rho
        Yc[3, s] = rhoe
        dzf = np.empty(z + 1)
        dzf[0], dzf[-1] = zf[1] - zf[0], zf[-1] - zf[-2]
        dzf[1:-1] = 0.5 * (zf[2:] - zf[:-2])
        w = np.zeros(z + 1)
        w[1:-1] = w_sigma * rng.standard_normal(z - 1)
        Yf[off[k] + k: off[k] + k + z + 1] = w * dzf
    return Yc.astype(dtype), Yf.astype(dtype)


def batch_heights(ncols, lo=30, hi=127, seed=2):
    """z_elem drawn uniformly from {lo .. hi} with the given seed."""
    return np.random.default_rng(seed).integers(lo, hi + 1, size=ncols).astype(np.int32)


class ColumnBatch:
    """A batch of standalone columns on the GPU (one gb_columns handle)."""

    def __init__(self, cfg, z_elem, device="cuda"):
        import torch
        self.cfg = cfg
        self.z_elem = np.ascontiguousarray(z_elem, dtype=np.int32)
        self.ncols = len(self.z_elem)
        self.dtype = torch.float32 if np.dtype(cfg.ft) == np.float32 else torch.float64
        self.device = device
        L = N.load()
        c = N.make_config(cfg)
        h = ctypes.c_void_p()
        _check(None, L.gb_columns_create(ctypes.byref(c), self.ncols,
                                         self.z_elem.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), ctypes.byref(h)))
        self.h = h.value
        nc, nf = ctypes.c_longlong(), ctypes.c_longlong()
        _check(self.h, L.gb_columns_size(self.h, ctypes.byref(nc), ctypes.byref(nf)))
        self.n_centre, self.n_face = nc.value, nf.value
        self.offsets = offsets(self.z_elem)
        self.stream = torch.cuda.current_stream()
        _check(self.h, L.gb_columns_set_stream(self.h, ctypes.c_void_p(self.stream.cuda_stream)))

    def __del__(self):
        try:
            if getattr(self, "h", None):
                N.load().gb_columns_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def state(self, Yc, Yf):
        import torch
        return FieldVector(torch.from_numpy(np.ascontiguousarray(Yc)).to(self.device, self.dtype),
                           torch.from_numpy(np.ascontiguousarray(Yf)).to(self.device, self.dtype))

    def solve(self, U, Uhat, dtgamma, newton_iters=2, mode="graph", residual=True):
        """Newton iterations in place on U; returns the [iters, 3] FP64 squared
        residual sums (rho, rho e_tot, u_3) when ``residual``."""
        out = np.zeros((newton_iters, 3)) if residual else None
        ptr = out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if residual else None
        _check(self.h, N.load().gb_columns_solve(self.h, U.gb(), Uhat.gb(), float(dtgamma), int(newton_iters),
                                                 MODES[mode], ptr))
        return out

    def autotune(self, U, Uhat, dtgamma, newton_iters=2, reps=3):
        """Times the persistent variants on this data and keeps the fastest; returns (choice, ms[variants])."""
        ms = np.zeros(N.GB_COLUMNS_VARIANTS)
        ch = ctypes.c_int()
        _check(self.h, N.load().gb_columns_autotune(self.h, U.gb(), Uhat.gb(), float(dtgamma), int(newton_iters),
                                                    int(reps), ctypes.byref(ch),
                                                    ms.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return ch.value, ms

    def set_variant(self, v):
        _check(self.h, N.load().gb_columns_set_variant(self.h, int(v)))

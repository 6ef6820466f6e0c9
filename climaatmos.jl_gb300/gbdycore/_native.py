"""ctypes binding of the C ABI in include/gbdycore.h (libgbdycore.so).

This is the Python counterpart of the ``ccall((:gb_*, libgbdycore), ...)``
stubs of the Julia shim.  Loading fails loudly if the library has not been
built; there is no CPU fallback.
"""
import ctypes
import os

from . import build as _build

_c_int, _c_double, _vp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p

GB_OK, GB_ERR_ARG, GB_ERR_CUDA, GB_ERR_NOMEM, GB_ERR_NONFINITE, GB_ERR_TIMEOUT, GB_ERR_STATE = 0, -1, -2, -3, -4, -5, -6
STATUS_NAMES = {0: "GB_OK", -1: "GB_ERR_ARG", -2: "GB_ERR_CUDA", -3: "GB_ERR_NOMEM", -4: "GB_ERR_NONFINITE",
                -5: "GB_ERR_TIMEOUT", -6: "GB_ERR_STATE"}

# Every symbol the header declares (checked by the CPU test suite).
SYMBOLS = [
    "gb_sizes", "gb_geometry_export", "gb_ctx_create", "gb_ctx_destroy", "gb_set_stream", "gb_last_error",
    "gb_set_precomputed_quantities", "gb_remaining_tendency", "gb_implicit_tendency", "gb_update_jacobian",
    "gb_ldiv", "gb_correct_implicit_advection_tendency", "gb_dss", "gb_step", "gb_global_sums",
    "gb_conservation_sums",    "gb_newton_residual", "gb_time_kernel", "gb_jacobian_solve_noalloc", "gb_match_elements",
    "gb_selftest_bounded_wait",
    "gb_dss_transpose", "gb_remaining_tendency_vjp", "gb_implicit_stage", "gb_implicit_stage_vjp", "gb_step_vjp",
    "gb_adjoint_forward", "gb_adjoint_reverse", "gb_adjoint_set_record_segments",
    "gb_columns_create", "gb_columns_destroy", "gb_columns_set_stream", "gb_columns_size", "gb_columns_solve",
    "gb_columns_autotune", "gb_columns_set_variant", "gb_columns_last_error",
]
GB_COLUMNS_GRAPH, GB_COLUMNS_PERSISTENT, GB_COLUMNS_PER_HEIGHT = 0, 1, 2
GB_COLUMNS_VARIANTS = 5
GB_NOALLOC_SCRATCH_BYTES = 64 << 20


class GBConfig(ctypes.Structure):
    _fields_ = [("h_elem", _c_int), ("z_elem", _c_int), ("ft_bytes", _c_int), ("z_stretch", _c_int),
                ("z_max", _c_double), ("dz_bottom", _c_double), ("dt", _c_double),
                ("nu_v", _c_double), ("nu_s", _c_double), ("div_damp", _c_double),
                ("sponge_zd", _c_double), ("alpha_uh", _c_double), ("alpha_w", _c_double),
                ("upwinding", _c_int)] + [(n, _c_double) for n in (
                    "grav", "omega", "R_d", "cp_d", "cv_d", "T_0", "p_ref", "T_min_ref", "T_surf_ref",
                    "T_min_sgs", "radius")] + [("held_suarez", _c_int)] + [(n, _c_double) for n in (
                    "hs_day", "hs_sigma_b", "hs_dT_y", "hs_T_equator", "hs_dtheta_z", "hs_T_min",
                    "hs_p_ref_theta", "hs_MSLP")] + [
                    ("elem_map", ctypes.POINTER(_c_int)), ("elem_orient", ctypes.POINTER(_c_int)),
                    ("test_dycore_consistency", _c_int),
                    ("z_surface", ctypes.POINTER(_c_double)), ("warp", _c_int),
                    ("sleve_eta", _c_double), ("sleve_s", _c_double),
                    ("moist", _c_int)] + [(n, _c_double) for n in (
                    "R_v", "cp_v", "cp_l", "cp_i", "LH_v0", "LH_s0", "T_triple", "press_triple", "T_freeze",
                    "T_icenuc", "pow_icenuc")] + [("sa_iters", _c_int)]


class GBFieldVec(ctypes.Structure):
    _fields_ = [("c", _vp), ("f", _vp)]


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class GBGeometryHost(ctypes.Structure):
    _fields_ = [("xyz", _dp), ("ecov", _dp), ("Jh", _dp), ("gup", _dp), ("fh0", _dp), ("zf", _dp),
                ("dss_off", _ip), ("dss_copy", _ip), ("econ", _dp), ("dss_w", _dp)]


class GBError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS_NAMES.get(code, code), msg))
        self.code = code


_lib = None


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load libgbdycore.so (building it with nvcc first if it is missing or stale)."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build_if_missing else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError("libgbdycore.so is not built (run __graft_entry__.build())")
    L = ctypes.CDLL(path)
    fv = GBFieldVec
    cfgp = ctypes.POINTER(GBConfig)
    L.gb_sizes.argtypes = [cfgp, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t), _ip, _ip]
    L.gb_geometry_export.argtypes = [cfgp, ctypes.POINTER(GBGeometryHost)]
    L.gb_ctx_create.argtypes = [cfgp, ctypes.POINTER(_vp)]
    L.gb_ctx_destroy.argtypes = [_vp]
    L.gb_set_stream.argtypes = [_vp, _vp]
    L.gb_last_error.argtypes = [_vp, ctypes.c_char_p, ctypes.c_size_t]
    L.gb_set_precomputed_quantities.argtypes = [_vp, fv, _c_double]
    L.gb_remaining_tendency.argtypes = [_vp, fv, fv, _c_double]
    L.gb_implicit_tendency.argtypes = [_vp, fv, fv, _c_double]
    L.gb_update_jacobian.argtypes = [_vp, fv, _c_double, _c_double]
    L.gb_ldiv.argtypes = [_vp, fv, fv]
    L.gb_correct_implicit_advection_tendency.argtypes = [_vp, fv, fv, _c_double]
    L.gb_dss.argtypes = [_vp, fv]
    L.gb_step.argtypes = [_vp, fv, _c_double, _c_double, _c_int, _c_int]
    L.gb_global_sums.argtypes = [_vp, fv, _dp]
    L.gb_conservation_sums.argtypes = [_vp, fv, _dp]
    L.gb_newton_residual.argtypes = [_vp, _dp]
    L.gb_time_kernel.argtypes = [_vp, _c_int, fv, _c_int, _dp]
    L.gb_jacobian_solve_noalloc.argtypes = [_vp, fv, fv, fv, _c_double]
    L.gb_match_elements.argtypes = [cfgp, _dp, _ip, _ip]
    L.gb_selftest_bounded_wait.argtypes = [_vp, _c_double]
    L.gb_dss_transpose.argtypes = [_vp, fv]
    L.gb_remaining_tendency_vjp.argtypes = [_vp, fv, fv, fv, _c_double, _dp]
    L.gb_implicit_stage.argtypes = [_vp, fv, fv, fv, _c_double]
    L.gb_implicit_stage_vjp.argtypes = [_vp, fv, fv, fv, fv, _c_double, _dp]
    L.gb_step_vjp.argtypes = [_vp, fv, fv, _c_double, _c_double, _dp]
    L.gb_adjoint_forward.argtypes = [_vp, fv, _c_double, _c_double, _c_int, _c_int]
    L.gb_adjoint_reverse.argtypes = [_vp, fv, _dp, ctypes.POINTER(ctypes.c_size_t)]
    L.gb_adjoint_set_record_segments.argtypes = [_vp, _c_int]
    _llp = ctypes.POINTER(ctypes.c_longlong)
    L.gb_columns_create.argtypes = [cfgp, _c_int, _ip, ctypes.POINTER(_vp)]
    L.gb_columns_destroy.argtypes = [_vp]
    L.gb_columns_set_stream.argtypes = [_vp, _vp]
    L.gb_columns_size.argtypes = [_vp, _llp, _llp]
    L.gb_columns_solve.argtypes = [_vp, fv, fv, _c_double, _c_int, _c_int, _dp]
    L.gb_columns_autotune.argtypes = [_vp, fv, fv, _c_double, _c_int, _c_int, _ip, _dp]
    L.gb_columns_set_variant.argtypes = [_vp, _c_int]
    L.gb_columns_last_error.argtypes = [_vp, ctypes.c_char_p, ctypes.c_size_t]
    for s in SYMBOLS:
        getattr(L, s).restype = _c_int
    _lib = L
    return L


def make_config(cfg):
    """gb_config from a gbdycore.config.DycoreConfig."""
    import numpy as np
    c = GBConfig()
    c.h_elem, c.z_elem = cfg.h_elem, cfg.z_elem
    c.ft_bytes = np.dtype(cfg.ft).itemsize
    c.z_stretch = 1 if cfg.z_stretch else 0
    c.z_max, c.dz_bottom, c.dt = cfg.z_max, cfg.dz_bottom, cfg.dt
    c.nu_v, c.nu_s, c.div_damp = cfg.nu, cfg.nu_s, cfg.divergence_damping
    c.sponge_zd, c.alpha_uh, c.alpha_w = cfg.sponge_zd, cfg.alpha_uh, cfg.alpha_w
    c.upwinding = 1 if cfg.upwinding == "vanleer" else 0
    for k, v in cfg.constants.items():
        setattr(c, k, float(v))
    c.held_suarez = 1 if cfg.held_suarez else 0
    for k, v in cfg.hs.items():
        setattr(c, "hs_" + k, float(v))
    c.test_dycore_consistency = 1 if getattr(cfg, "test_dycore_consistency", False) else 0
    keep = []
    layout = getattr(cfg, "layout", None)
    if layout is not None:
        emap = np.ascontiguousarray(layout[0], dtype=np.int32)
        eori = np.ascontiguousarray(layout[1], dtype=np.int32)
        c.elem_map = emap.ctypes.data_as(ctypes.POINTER(_c_int))
        c.elem_orient = eori.ctypes.data_as(ctypes.POINTER(_c_int))
        keep += [emap, eori]
    zs = getattr(cfg, "z_surface", None)
    if zs is not None:
        z = np.ascontiguousarray(zs, dtype=np.float64).reshape(-1)
        c.z_surface = z.ctypes.data_as(ctypes.POINTER(_c_double))
        keep.append(z)
    c.warp = 1 if getattr(cfg, "warp", "linear") == "sleve" else 0
    c.sleve_eta, c.sleve_s = float(getattr(cfg, "sleve_eta", 0.7)), float(getattr(cfg, "sleve_s", 10.0))
    c.moist = 1 if getattr(cfg, "moist", False) else 0
    for k, v in getattr(cfg, "moist_constants", {}).items():
        setattr(c, k, float(v))
    c.sa_iters = int(getattr(cfg, "sa_iters", 16))
    c._keep = tuple(keep)   # the arrays live as long as the struct
    return c


def match_elements(cfg, xyz):
    """(elem_map, elem_orient) of the caller's layout from its node positions [Nh, 16, 3]
    (gb_match_elements); raises GBError if the positions are not a rotated-frame equiangular
    cubed sphere at cfg.h_elem."""
    import numpy as np
    L = load()
    c = make_config(cfg.with_(layout=None) if hasattr(cfg, "with_") else cfg)
    Nh = 6 * cfg.h_elem ** 2
    x = np.ascontiguousarray(xyz, dtype=np.float64).reshape(Nh, 16, 3)
    emap, eori = np.zeros(Nh, np.int32), np.zeros(Nh, np.int32)
    ip = ctypes.POINTER(_c_int)
    rc = L.gb_match_elements(ctypes.byref(c), x.ctypes.data_as(_dp), emap.ctypes.data_as(ip), eori.ctypes.data_as(ip))
    if rc != GB_OK:
        raise GBError(rc, "gb_match_elements: the node positions are not those of a cubed sphere at h_elem=%d"
                      % cfg.h_elem)
    return emap, eori

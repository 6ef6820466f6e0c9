"""ctypes front end of the CPU oracle (``dycore_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``, as the reference results to compare with and as
the timed CPU port.  The
product (``climaatmos.jl_gb300``) never imports it.

Parity status: restated from the reference's call sites and documentation; the
ClimaCore / ClimaTimeSteppers arithmetic it replaces cannot run here (no Julia),
so agreement with ClimaCore itself is unpinned.  It is pinned by the
reference's invariants (see ``tests/test_oracle_invariants.py``).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
# ORACLE_VARIANT selects a precision-study build of dycore_oracle.cpp: "store32" (ORACLE_STORE32:
# every field the step stores is rounded to FP32, the arithmetic stays in the oracle's type) or
# "phid" (ORACLE_PHID: g z - Phi_r formed as a deviation from per-level reference values, the
# same mathematics without the O(1e5) cancellation); unset, the oracle is the default build.
VARIANT = os.environ.get("ORACLE_VARIANT", "")
_FLAGS = {"": [], "store32": ["-DORACLE_STORE32"], "phid": ["-DORACLE_PHID"]}
if VARIANT not in _FLAGS:
    raise ValueError("ORACLE_VARIANT must be unset, 'store32' or 'phid'")
LIB = os.path.join(BUILD, "liboracle_%s.so" % VARIANT if VARIANT else "liboracle.so")
SRC = os.path.join(HERE, "dycore_oracle.cpp")


def build(force=False):
    """Compile the oracle with g++ (OpenMP) into oracle/_build/liboracle.so (or the
    precision-study variant)."""
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["g++", "-O3", "-fopenmp", "-shared", "-fPIC", "-std=c++17", "-ffp-contract=off", SRC, "-o", LIB + ".tmp"]
    cmd += _FLAGS[VARIANT]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


class _Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in (
        "grav", "omega", "R_d", "cp_d", "cv_d", "T_0", "p_ref", "T_min_ref", "T_surf_ref", "T_min_sgs", "radius",
        "nu_v", "nu_s", "div_damp", "sponge_zd", "alpha_uh", "alpha_w", "z_max", "dt_model")] + [
        ("upwinding", ctypes.c_int), ("dss_stage1", ctypes.c_int), ("held_suarez", ctypes.c_int)] + [
        (n, ctypes.c_double) for n in ("hs_day", "hs_sigma_b", "hs_dT_y", "hs_T_equator", "hs_dtheta_z",
                                       "hs_T_min", "hs_p_ref_theta", "hs_MSLP")] + [
        ("moist", ctypes.c_int)] + [
        (n, ctypes.c_double) for n in ("R_v", "cp_v", "cp_l", "cp_i", "LH_v0", "LH_s0", "T_triple", "press_triple",
                                       "T_freeze", "T_icenuc", "pow_icenuc")] + [
        ("sa_iters", ctypes.c_int)]


_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class _Geom(ctypes.Structure):
    _fields_ = [("Nh", ctypes.c_int), ("Nv", ctypes.c_int), ("ngroups", ctypes.c_int)] + [
        (n, _dp) for n in ("W", "D", "Jh", "gup", "gdn", "sinlat", "fh0", "ecov", "econ", "zf")] + [
        ("dss_off", _ip), ("dss_copy", _ip), ("dss_w", _dp)] + [
        ("t_" + n, _dp) for n in ("zc", "zf", "Jc", "Jf", "guc", "guf", "gdc", "f3c", "f12f", "Ecc", "Ecn")]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        v = ctypes.c_void_p
        _lib.oracle_create.restype = v
        _lib.oracle_create.argtypes = [ctypes.POINTER(_Geom), ctypes.POINTER(_Params), ctypes.c_int]
        _lib.oracle_destroy.argtypes = [v]
        for name in ("oracle_remaining_tendency", "oracle_implicit_tendency", "oracle_correct_implicit", "oracle_ldiv",
                     "oracle_jac_apply"):
            getattr(_lib, name).argtypes = [v, v, v, v, v]
        _lib.oracle_set_precomputed.argtypes = [v, v, v]
        _lib.oracle_pressure.argtypes = [v, v, v, v]
        _lib.oracle_dss.argtypes = [v, v, v]
        _lib.oracle_dss_c123.argtypes = [v, v]
        _lib.oracle_laplacians.argtypes = [v, v, v]
        _lib.oracle_update_jacobian.argtypes = [v, v, v, ctypes.c_double]
        _lib.oracle_step.argtypes = [v, v, v, ctypes.c_double, ctypes.c_int]
        _lib.oracle_global_sums.argtypes = [v, v, _dp]
        _lib.oracle_sat_adjust.argtypes = [v, ctypes.c_int] + [_dp] * 6
        _lib.oracle_set_threads.argtypes = [ctypes.c_int]
        _lib.oracle_max_threads.restype = ctypes.c_int
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Oracle:
    """FP64 (or FP32) CPU restatement of the dry IMEX step on one grid.

    ``params`` is a dict with the keys of ``_Params``; state arrays use the
    C-ABI layout: centre ``[Nh, 4, 16, Nv]`` (rho, u_1, u_2, rho e_tot) and
    face ``[Nh, 16, Nv + 1]`` (u_3).  With ``params["moist"] = 1`` (moist 0M) the centre
    block is ``[Nh, 5, 16, Nv]`` (rho q_tot last) and only the column operators are
    available: set_precomputed, pressure, implicit_tendency, update_jacobian, ldiv,
    jac_apply and correct_implicit.
    """

    def __init__(self, geom, params, dtype=np.float64):
        self.geom = geom
        self.dtype = np.dtype(dtype)
        L = lib()
        self._keep = []

        def arr(x, t=np.float64):
            a = np.ascontiguousarray(x, dtype=t)
            self._keep.append(a)
            return a.ctypes.data_as(_ip if t == np.int32 else _dp)

        g = _Geom()
        g.Nh, g.Nv, g.ngroups = geom.Nh, geom.Nv, len(geom.dss_off) - 1
        g.W = arr(geom.W)
        g.D = arr(geom.D.reshape(-1))
        g.Jh = arr(geom.Jh)
        g.gup = arr(geom.gup)
        g.gdn = arr(geom.gdn)
        g.sinlat = arr(geom.sinlat)
        g.fh0 = arr(geom.fh0)
        g.ecov = arr(geom.ecov)
        g.econ = arr(geom.econ)
        g.zf = arr(geom.zf)
        g.dss_off = arr(geom.dss_off, np.int32)
        g.dss_copy = arr(geom.dss_copy, np.int32)
        g.dss_w = arr(geom.dss_w)
        # terrain-following geometry: a dict of per-point arrays (topography.oracle_terrain)
        terrain = getattr(geom, "terrain", None)
        if terrain is not None:
            for k in ("zc", "zf", "Jc", "Jf", "guc", "guf", "gdc", "f3c", "f12f", "Ecc", "Ecn"):
                setattr(g, "t_" + k, arr(terrain[k]))
        p = _Params()
        for k, _ in _Params._fields_:
            setattr(p, k, params.get(k, 0))
        self._g, self._p = g, p
        self.moist = bool(params.get("moist", 0))
        if self.moist and terrain is not None:
            raise NotImplementedError("moist 0M over terrain-following levels is not restated")
        self.nfc = 5 if self.moist else 4
        self.h = L.oracle_create(ctypes.byref(g), ctypes.byref(p), self.dtype.itemsize)
        self.Nh, self.Nv = geom.Nh, geom.Nv

    def __del__(self):
        try:
            lib().oracle_destroy(self.h)
        except Exception:
            pass

    def zeros(self):
        return (np.zeros((self.Nh, self.nfc, 16, self.Nv), self.dtype),
                np.zeros((self.Nh, 16, self.Nv + 1), self.dtype))

    def _dry_only(self, what):
        if self.moist:
            raise NotImplementedError(what + " is restated for dry air only (moist 0M: the column operators)")

    def _chk(self, *a):
        for x in a:
            assert x.dtype == self.dtype and x.flags.c_contiguous

    def set_precomputed(self, Yc, Yf):
        self._chk(Yc, Yf)
        lib().oracle_set_precomputed(self.h, _ptr(Yc), _ptr(Yf))

    def pressure(self, Yc, Yf):
        """The precomputed pressure at Y, [Nh, 16, Nv]."""
        Yc = np.ascontiguousarray(Yc, self.dtype)
        Yf = np.ascontiguousarray(Yf, self.dtype)
        p = np.zeros((self.Nh, 16, self.Nv), self.dtype)
        lib().oracle_pressure(self.h, _ptr(Yc), _ptr(Yf), _ptr(p))
        return p

    def remaining_tendency(self, Yc, Yf):
        self._dry_only('remaining_tendency')
        Tc, Tf = self.zeros()
        self._chk(Yc, Yf)
        lib().oracle_remaining_tendency(self.h, _ptr(Tc), _ptr(Tf), _ptr(Yc), _ptr(Yf))
        return Tc, Tf

    def implicit_tendency(self, Yc, Yf):
        Tc, Tf = self.zeros()
        self._chk(Yc, Yf)
        lib().oracle_implicit_tendency(self.h, _ptr(Tc), _ptr(Tf), _ptr(Yc), _ptr(Yf))
        return Tc, Tf

    def correct_implicit(self, Yc, Yf):
        Tc, Tf = self.zeros()
        self._chk(Yc, Yf)
        lib().oracle_correct_implicit(self.h, _ptr(Tc), _ptr(Tf), _ptr(Yc), _ptr(Yf))
        return Tc, Tf

    def update_jacobian(self, Yc, Yf, dtg):
        self._chk(Yc, Yf)
        lib().oracle_update_jacobian(self.h, _ptr(Yc), _ptr(Yf), float(dtg))

    def ldiv(self, Rc, Rf):
        Xc, Xf = self.zeros()
        Rc = np.ascontiguousarray(Rc, self.dtype)
        Rf = np.ascontiguousarray(Rf, self.dtype)
        lib().oracle_ldiv(self.h, _ptr(Xc), _ptr(Xf), _ptr(Rc), _ptr(Rf))
        return Xc, Xf

    def jac_apply(self, Vc, Vf):
        """W V with the blocks of the last update_jacobian."""
        Oc, Of = self.zeros()
        Vc = np.ascontiguousarray(Vc, self.dtype)
        Vf = np.ascontiguousarray(Vf, self.dtype)
        lib().oracle_jac_apply(self.h, _ptr(Oc), _ptr(Of), _ptr(Vc), _ptr(Vf))
        return Oc, Of

    def dss(self, Yc, Yf):
        self._chk(Yc, Yf)
        lib().oracle_dss(self.h, _ptr(Yc), _ptr(Yf))

    def dss_c123(self, C):
        """In place: the DSS of a centre block [Nh, 4, 16, Nv] whose comp 0 is a scalar and
        comps 1-3 one covariant 3-vector (the block of the Laplacians)."""
        self._dry_only('dss_c123')
        self._chk(C)
        lib().oracle_dss_c123(self.h, _ptr(C))

    def laplacians(self, X):
        """Per level, after the DSS: the scalar Laplacian wdiv(grad f) of comp 0 and the vector
        Laplacian of the covariant (comp 1, comp 2); X and the result are [Nh, 4, 16, Nv]."""
        self._dry_only('laplacians')
        X = np.ascontiguousarray(X, self.dtype)
        O = np.zeros_like(X)
        lib().oracle_laplacians(self.h, _ptr(X), _ptr(O))
        return O

    def step(self, Yc, Yf, dt, nsteps=1):
        self._dry_only('step')
        self._chk(Yc, Yf)
        lib().oracle_step(self.h, _ptr(Yc), _ptr(Yf), float(dt), int(nsteps))

    def sat_adjust(self, rho, eint, q):
        """The saturation adjustment (moist oracles): (T, q_liq, q_ice) of each point of the
        equal-shaped arrays rho, e_int, q_tot, in the oracle's precision."""
        if not self.moist:
            raise NotImplementedError("the saturation adjustment belongs to a moist oracle")
        a = [np.ascontiguousarray(x, np.float64).ravel() for x in np.broadcast_arrays(rho, eint, q)]
        out = [np.zeros_like(a[0]) for _ in range(3)]
        lib().oracle_sat_adjust(self.h, a[0].size, *[x.ctypes.data_as(_dp) for x in a + out])
        shape = np.broadcast(rho, eint, q).shape
        return tuple(x.reshape(shape) for x in out)

    def global_sums(self, Yc):
        """∫ρ dV, ∫ρe_tot dV and, for a moist oracle, ∫ρq_tot dV (compensated FP64)."""
        out = np.zeros(3 if self.moist else 2)
        lib().oracle_global_sums(self.h, _ptr(Yc), out.ctypes.data_as(_dp))
        return out


def set_threads(n):
    lib().oracle_set_threads(int(n))


def max_threads():
    return lib().oracle_max_threads()

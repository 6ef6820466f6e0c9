"""Shared test helpers: oracle construction and field comparisons."""
import numpy as np

from geometry import OracleGeometry
import oracle as O
from gbdycore import config as C
from gbdycore import setups as S

_GEO = {}


def oracle_geometry(cfg):
    key = (cfg.h_elem, cfg.z_elem, cfg.z_max, cfg.z_stretch, cfg.dz_bottom, cfg.constants["radius"])
    if key not in _GEO:
        _GEO[key] = OracleGeometry(cfg.h_elem, cfg.z_elem, cfg.z_max, cfg.z_stretch, cfg.dz_bottom,
                                   radius=cfg.constants["radius"], omega=cfg.constants["omega"])
    return _GEO[key]


def make_oracle(cfg, dtype=np.float64, dss_stage1=True):
    cfg64 = cfg.with_(ft=np.float64)
    return O.Oracle(oracle_geometry(cfg64), cfg64.oracle_params(dss_stage1=dss_stage1), dtype)


def dss_oracle_on_product_grid(cfg, dtype=np.float64):
    """An oracle whose DSS plan and bases are the library's own (gb_geometry_export), so
    that a DSS comparison sees the summation and nothing of the two grids' last-bit
    differences (the grids themselves agree to 1e-14, test_geometry.py)."""
    import copy
    from gbdycore.simulation import Geometry
    cfg64 = cfg.with_(ft=np.float64)
    g = copy.copy(oracle_geometry(cfg64))
    pg = Geometry(cfg64)
    g.ecov, g.econ = pg.ecov, pg.econ
    g.dss_off, g.dss_copy, g.dss_w = pg.dss_off, pg.dss_copy, pg.dss_w
    return O.Oracle(g, cfg64.oracle_params(), dtype)


def state(cfg, workload="plain", dtype=np.float64, geom=None):
    g = geom or oracle_geometry(cfg)
    Yc, Yf = S.workload_state(g, cfg, workload)
    return Yc.astype(dtype), Yf.astype(dtype)


def perturbed_state(cfg, seed=11, dtype=np.float64, w_amp=0.05):
    """Balanced state plus nonzero u_3 (interior faces), so every operator is exercised."""
    Yc, Yf = state(cfg, dtype=np.float64)
    rng = np.random.default_rng(seed)
    g = oracle_geometry(cfg)
    w = rng.normal(0, w_amp, size=Yf.shape)
    Yf = w * g.dzf[None, None, :]
    Yf[:, :, 0] = 0
    Yf[:, :, -1] = 0
    Yc = Yc.copy()
    Yc[:, 3] *= 1 + 1e-3 * rng.normal(size=Yc[:, 3].shape)
    make_oracle(cfg).dss(Yc, Yf)        # continuous, as every stage state of the step is
    return Yc.astype(dtype), Yf.astype(dtype)


def small_config(ft=np.float64, **kw):
    base = dict(h_elem=3, z_elem=8, z_max=30000.0, z_stretch=True, dz_bottom=300.0, dt=300.0, ft=ft)
    base.update(kw)
    return C.DycoreConfig(**base)


def rel_err(a, b):
    """max-norm relative error per component (normalised by the component's max magnitude)."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def field_errors(Xc, Xf, Rc, Rf):
    names = ["rho", "u_1", "u_2", "rho_e_tot"]
    out = {names[c]: rel_err(Xc[:, c], Rc[:, c]) for c in range(4)}
    out["u_3"] = rel_err(Xf, Rf)
    return out


def moist_state(cfg, seed=11, dtype=np.float64, w_amp=0.05, q0=0.018, H=2500.0):
    """Moist 0M state [Nh, 5, 16, Nv] (rho q_tot last) and faces: the perturbed dry state with
    q_tot = q0 exp(-z / H) (x (1 + 5 % noise)) and rho e_tot raised by
    rho q_tot ((cv_v - cv_d)(T - T_0) + e_int_v0 + R_d T_0), so that the all-vapour temperature
    is the dry state's T.  With q0 = 0.018 the lowest kilometres and the mixed-phase levels are
    supersaturated there (the saturation adjustment condenses); q0 = 0.003 keeps every point
    unsaturated."""
    Yc, Yf = perturbed_state(cfg.with_(moist=False), seed, np.float64, w_amp)
    dry = make_oracle(cfg.with_(moist=False))
    p = dry.pressure(Yc, Yf)
    K, M = cfg.constants, cfg.moist_constants
    rho = Yc[:, 0]
    T = p / (rho * K["R_d"])
    g = oracle_geometry(cfg)
    rng = np.random.default_rng(seed + 100)
    q = q0 * np.exp(-g.zc / H)[None, None, :] * (1 + 0.05 * rng.normal(size=rho.shape))
    cvv = M["cp_v"] - M["R_v"]
    ev0 = M["LH_v0"] - M["R_v"] * K["T_0"]
    Ym = np.concatenate([Yc, (rho * q)[:, None]], axis=1)
    Ym[:, 3] += rho * q * ((cvv - K["cv_d"]) * (T - K["T_0"]) + ev0 + K["R_d"] * K["T_0"])
    return np.ascontiguousarray(Ym.astype(dtype)), Yf.astype(dtype)


def moist_field_errors(Xc, Xf, Rc, Rf):
    out = field_errors(Xc, Xf, Rc, Rf)
    out["rho_q_tot"] = rel_err(Xc[:, 4], Rc[:, 4])
    return out

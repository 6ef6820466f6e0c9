"""Initial states of the dry dynamical-core workloads.

Host-side counterpart of ``Setups.initial_state`` (src/setups/Setups.jl:313):
``center_initial_condition`` -> ``physical_state(; T, p, u, v)`` ->
``grid_scale_center_variables`` (src/setups/common/prognostic_variables.jl:43-61),
which stores ``rho``, the covariant ``u_h = C12(UVVector(u, v))`` and
``rho e_tot = rho (e_kin + e_pot + e_int(T))``; ``u_3 = 0`` on faces
(prognostic_variables.jl:280-287).

The temperature profile is T(z) = max(300 - 6.5e-3 z, 200) K with p_surf = 1e5 Pa
in hydrostatic balance (power law below the tropopause, exponential above).
Horizontal-velocity perturbations are drawn per unique node and level with the
given seed, so collocated element copies carry the same physical wind.
"""
import math

import numpy as np

T_SURF, LAPSE, T_STRAT, P_SURF = 300.0, 6.5e-3, 200.0, 1.0e5


def temperature_pressure(z, c):
    g, Rd = c["grav"], c["R_d"]
    z = np.asarray(z, dtype=np.float64)
    zt = (T_SURF - T_STRAT) / LAPSE
    T = np.maximum(T_SURF - LAPSE * z, T_STRAT)
    expo = g / (Rd * LAPSE)
    pt = P_SURF * (T_STRAT / T_SURF) ** expo
    p = np.where(z <= zt, P_SURF * (np.maximum(T_SURF - LAPSE * z, 1e-9) / T_SURF) ** expo,
                 pt * np.exp(-g * (z - zt) / (Rd * T_STRAT)))
    return T, p


def _unique_node_index(xyz):
    key = np.round(xyz.reshape(-1, 3) * 1e9).astype(np.int64)
    _, inv = np.unique(key, axis=0, return_inverse=True)
    return inv.reshape(xyz.shape[:-1]), int(inv.max()) + 1


def _east_north(xyz):
    x, y, z = (np.where(np.abs(xyz[..., d]) < 1e-12, 0.0, xyz[..., d]) for d in range(3))
    lon = np.arctan2(y, x)
    coslat = np.sqrt(x * x + y * y)
    E = np.stack([-np.sin(lon), np.cos(lon), np.zeros_like(lon)], axis=-1)
    N = np.stack([-z * np.cos(lon), -z * np.sin(lon), coslat], axis=-1)
    return E, N


def initial_state(geom, cfg, seed=0, sigma=1.0, bump=None, dtype=None):
    """Return (Yc, Yf) in the C-ABI layout for the balanced lapse-rate state.

    ``geom`` provides ``xyz[Nh,16,3]`` (unit sphere), ``ecov[Nh,16,2,3]``
    (covariant basis at the surface radius), ``zc[Nv]``, ``R``.  ``bump`` is
    ``(amplitude, radius_m, lat_deg, lon_deg)`` for a Gaussian rho e_tot bump.
    """
    c = cfg.constants
    dtype = np.dtype(dtype or cfg.ft)
    Nh, Nv = geom.Nh, geom.Nv
    zc = np.asarray(geom.zc, dtype=np.float64)
    terrain = getattr(geom, "terrain", None)
    if terrain is not None:
        # terrain-following levels: the same profile at each point's own height
        zc = np.asarray(terrain["zc"], dtype=np.float64)        # [Nh,16,Nv]
    else:
        zc = np.broadcast_to(zc, (Nh, 16, Nv))
    T, p = temperature_pressure(zc, c)
    rho = p / (c["R_d"] * T)                                   # [Nh,16,Nv]
    rc = (geom.R + zc) / geom.R
    uidx, nu = _unique_node_index(geom.xyz)
    rng = np.random.default_rng(seed)
    uv = rng.normal(0.0, sigma, size=(nu, Nv, 2))
    u = uv[uidx][..., 0]                                       # [Nh,16,Nv]
    v = uv[uidx][..., 1]
    E, N = _east_north(geom.xyz)
    ecov = geom.ecov
    # covariant components u_i = e_i(z) . (u E + v N), e_i(z) = r(z) e_i(R)
    eE = np.einsum("enik,enk->eni", ecov, E)                   # [Nh,16,2]
    eN = np.einsum("enik,enk->eni", ecov, N)
    u1 = (eE[..., 0, None] * u + eN[..., 0, None] * v) * rc
    u2 = (eE[..., 1, None] * u + eN[..., 1, None] * v) * rc
    K = 0.5 * (u * u + v * v)
    eint = c["cv_d"] * (T - c["T_0"]) - c["R_d"] * c["T_0"]
    rhoe = rho * (eint + c["grav"] * zc + K)
    if bump is not None:
        amp, rad, lat0, lon0 = bump
        la, lo = math.radians(lat0), math.radians(lon0)
        X0 = np.array([math.cos(la) * math.cos(lo), math.cos(la) * math.sin(lo), math.sin(la)])
        d = geom.R * np.arccos(np.clip(geom.xyz @ X0, -1.0, 1.0))   # [Nh,16]
        rhoe = rhoe * (1.0 + amp * np.exp(-(d / rad) ** 2))[..., None]
    Yc = np.empty((Nh, 4, 16, Nv), dtype=np.float64)
    Yc[:, 0] = rho
    Yc[:, 1] = u1
    Yc[:, 2] = u2
    Yc[:, 3] = rhoe
    Yf = np.zeros((Nh, 16, Nv + 1), dtype=np.float64)
    return np.ascontiguousarray(Yc.astype(dtype)), np.ascontiguousarray(Yf.astype(dtype))


def workload_state(geom, cfg, name):
    """Initial state of a named workload: 'plain' (seed 0), 'production' (seed 1 + bump), 'precision' (seed 4)."""
    if name == "plain":
        return initial_state(geom, cfg, seed=0, sigma=1.0)
    if name == "production":
        return initial_state(geom, cfg, seed=1, sigma=2.0, bump=(0.01, 500e3, 40.0, 0.0))
    if name == "precision":
        return initial_state(geom, cfg, seed=4, sigma=1.0)
    if name == "differentiation":
        return initial_state(geom, cfg, seed=3, sigma=1.0)
    raise ValueError(name)


def moist_initial_state(geom, cfg, seed=0, sigma=1.0, q0=0.018, scale_height=2500.0, dtype=None):
    """Moist 0M counterpart of ``initial_state``: (Yc [Nh,5,16,Nv], Yf) with rho q_tot last.

    The same temperature profile and winds, specific humidity q_tot = q0 exp(-z / H) with 5 %
    noise per unique node and level, rho = p / (R_m T) with the all-vapour R_m, and
    rho e_tot = rho (e_int(T, q_tot) + g z + K) with the all-vapour internal energy
    cv_m (T - T_0) + q_tot e_int_v0 - (1 - q_tot) R_d T_0 (the saturation adjustment condenses
    where q_tot exceeds saturation: the lowest kilometres and the mixed-phase levels).
    """
    c, m = cfg.constants, cfg.moist_constants
    dtype = np.dtype(dtype or cfg.ft)
    Yc, Yf = initial_state(geom, cfg, seed=seed, sigma=sigma, dtype=np.float64)
    Nh, Nv = geom.Nh, geom.Nv
    zc = np.broadcast_to(np.asarray(geom.zc, dtype=np.float64), (Nh, 16, Nv))
    T, p = temperature_pressure(zc, c)
    uidx, nu = _unique_node_index(geom.xyz)
    noise = np.random.default_rng(seed + 1000).normal(0.0, 0.05, size=(nu, Nv))[uidx]
    q = q0 * np.exp(-zc / scale_height) * (1.0 + noise)
    Rm = c["R_d"] * (1.0 - q) + m["R_v"] * q
    rho_d = Yc[:, 0]
    rho = p / (Rm * T)
    cvv = m["cp_v"] - m["R_v"]
    ev0 = m["LH_v0"] - m["R_v"] * c["T_0"]
    e_dry = c["cv_d"] * (T - c["T_0"]) - c["R_d"] * c["T_0"]
    e_moist = (c["cv_d"] + (cvv - c["cv_d"]) * q) * (T - c["T_0"]) + q * ev0 - (1.0 - q) * c["R_d"] * c["T_0"]
    # rho e_tot / rho of the dry state is e_int + g z + K: replace its e_int
    spec = Yc[:, 3] / rho_d - e_dry + e_moist
    out = np.empty((Nh, 5, 16, Nv), dtype=np.float64)
    out[:, 0] = rho
    out[:, 1:3] = Yc[:, 1:3]
    out[:, 3] = rho * spec
    out[:, 4] = rho * q
    return np.ascontiguousarray(out.astype(dtype)), np.ascontiguousarray(Yf.astype(dtype))

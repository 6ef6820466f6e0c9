"""Held-Suarez forcing of the explicit tendency (rad: held_suarez).

Reference: src/parameterized_tendencies/radiation/held_suarez.jl:98-296 (compute_dRhoT,
compute_sigma, height_factor, the rho e_tot relaxation times cv_d and the
boundary-layer drag k_f = 1/day), applied in remaining_tendency!
(src/prognostic_equations/remaining_tendency.jl:154-172).  Flat surface: the
surface pressure is MSLP, so sigma = p / MSLP.

CPU: the oracle's forcing equals a numpy restatement of those formulas (the
difference of the oracle's remaining tendency with and without the forcing);
invalid parameters are rejected at the C ABI.  GPU: the remaining tendency and
the fused IMEX step with the forcing on against the oracle, and the pullbacks of
the tendency and of one step against central differences (FP64).
"""
import ctypes

import numpy as np
import pytest

from gbdycore import _native as N
from gbdycore import config as C
from helpers import field_errors, make_oracle, oracle_geometry, perturbed_state, small_config


def hs_config(ft=np.float64, **kw):
    # a deeper model top than the small test grid so that sigma spans the boundary layer
    return small_config(ft=ft, held_suarez=True, **kw)


def held_suarez_restated(cfg, Yc, p, sinlat):
    """-(cv_d k_T rho (p / (rho R_d) - T_eq)) for rho e_tot and -k_f hf u_h (numpy, FP64)."""
    c, h = cfg.constants, cfg.hs
    rho = Yc[:, 0]
    s2 = (sinlat ** 2)[:, :, None]
    c2 = 1.0 - s2
    sig = p / h["MSLP"]
    hf = np.maximum(0.0, (sig - h["sigma_b"]) / (1.0 - h["sigma_b"]))
    ka, ks, kf = 1.0 / (40.0 * h["day"]), 1.0 / (4.0 * h["day"]), 1.0 / h["day"]
    kT = ka + (ks - ka) * hf * c2 ** 2
    pr = p / h["p_ref_theta"]
    kappa = c["R_d"] / c["cp_d"]
    Teq = np.maximum(h["T_min"], (h["T_equator"] - h["dT_y"] * s2 - h["dtheta_z"] * np.log(pr) * c2) * pr ** kappa)
    d = np.zeros_like(Yc)
    d[:, 3] = -kT * rho * (p / (rho * c["R_d"]) - Teq) * c["cv_d"]
    d[:, 1] = -kf * hf * Yc[:, 1]
    d[:, 2] = -kf * hf * Yc[:, 2]
    return d, sig


def test_oracle_forcing_matches_restatement():
    cfg = hs_config()
    Yc, Yf = perturbed_state(cfg)
    on = make_oracle(cfg)
    off = make_oracle(cfg.with_(held_suarez=False))
    Ton, Tfon = on.remaining_tendency(Yc.copy(), Yf.copy())
    Toff, Tfoff = off.remaining_tendency(Yc.copy(), Yf.copy())
    p = on.pressure(Yc, Yf)
    g = oracle_geometry(cfg)
    d, sig = held_suarez_restated(cfg, Yc, p, np.asarray(g.sinlat).reshape(cfg_nh(cfg), 16))
    # both regimes of the boundary-layer weight occur on this grid
    assert (sig > cfg.hs["sigma_b"]).any() and (sig < cfg.hs["sigma_b"]).any()
    assert np.abs(Tfon - Tfoff).max() == 0
    assert np.abs(Ton[:, 0] - Toff[:, 0]).max() == 0
    for comp in (1, 2, 3):
        got = Ton[:, comp] - Toff[:, comp]
        scale = np.abs(d[:, comp]).max()
        assert scale > 0
        assert np.abs(got - d[:, comp]).max() <= 1e-10 * max(scale, np.abs(Ton[:, comp]).max()), comp


def cfg_nh(cfg):
    return 6 * cfg.h_elem * cfg.h_elem


def test_invalid_held_suarez_parameters_are_rejected():
    L = N.load()
    for bad in [dict(sigma_b=1.0), dict(day=0.0), dict(MSLP=-1.0)]:
        hs = dict(C.HELD_SUAREZ)
        hs.update(bad)
        c = N.make_config(C.plain_h6().with_(held_suarez=True, hs=hs))
        n = ctypes.c_size_t()
        assert L.gb_sizes(ctypes.byref(c), ctypes.byref(n), None, None, None) == N.GB_ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("ft,tol", [(np.float64, 1e-11), (np.float32, 1e-4)])
def test_gpu_remaining_tendency_with_forcing(ft, tol):
    from gbdycore import simulation as sim
    cfg = hs_config(ft=ft)
    Yc, Yf = perturbed_state(cfg, dtype=ft)
    ref = make_oracle(cfg, ft).remaining_tendency(Yc.copy(), Yf.copy())
    p = sim.AtmosCache(cfg)
    Y = sim.FieldVector.from_numpy(Yc, Yf)
    Yt = Y.similar()
    sim.remaining_tendency(Yt, None, Y, p, 0.0)
    Xc, Xf = Yt.numpy()
    e = field_errors(Xc, Xf, ref[0], ref[1])
    assert all(v <= tol for v in e.values()), e


@pytest.mark.gpu
def test_gpu_fused_step_with_forcing_fp64():
    from gbdycore import simulation as sim
    cfg = hs_config(ft=np.float64)
    Yc, Yf = perturbed_state(cfg, w_amp=0.05)
    o = make_oracle(cfg, np.float64, dss_stage1=False)
    rc, rf = Yc.copy(), Yf.copy()
    o.step(rc, rf, cfg.dt, 3)
    s = sim.AtmosSimulation(cfg, state=(Yc, Yf))
    s.step(3, use_graph=True)
    Xc, Xf = s.Y.numpy()
    e = field_errors(Xc, Xf, rc, rf)
    assert all(v <= 1e-10 for v in e.values()), e
    # and the forcing changed the answer
    o2 = make_oracle(cfg.with_(held_suarez=False), np.float64, dss_stage1=False)
    r2c, r2f = Yc.copy(), Yf.copy()
    o2.step(r2c, r2f, cfg.dt, 3)
    assert np.abs(r2c - rc).max() > 0


def _fv(Yc, Yf):
    from gbdycore import simulation as sim
    return sim.FieldVector.from_numpy(np.ascontiguousarray(Yc), np.ascontiguousarray(Yf))


def _dot(A, B):
    return float((A.c * B.c).sum().item() + (A.f * B.f).sum().item())


def _direction(Yc, Yf, seed):
    rng = np.random.default_rng(seed)
    dc = rng.standard_normal(Yc.shape)
    for c in range(4):
        dc[:, c] *= np.sqrt(np.mean(Yc[:, c] ** 2))
    df = rng.standard_normal(Yf.shape) * np.sqrt(np.mean(Yf ** 2))
    return dc, df


def _cotangent(Xc, Xf, seed):
    rng = np.random.default_rng(seed)
    return _fv(rng.standard_normal(Xc.shape) / np.maximum(np.abs(Xc).max(axis=(0, 2, 3), keepdims=True), 1e-30),
               rng.standard_normal(Xf.shape) / max(np.abs(Xf).max(), 1e-30))


H = 1.0e-6


@pytest.mark.gpu
def test_gpu_remaining_tendency_vjp_with_forcing():
    """<Tb, (T(Y + h d) - T(Y - h d)) / 2h> == <T^T Tb, d> with the forcing on (FP64)."""
    from gbdycore import simulation as sim
    cfg = hs_config(ft=np.float64)
    Yc, Yf = perturbed_state(cfg)
    p = sim.AtmosCache(cfg)
    Y = _fv(Yc, Yf)
    T = Y.similar()
    sim.remaining_tendency(T, None, Y, p, 0.0)
    Tb = _cotangent(*T.numpy(), seed=2)
    Yb = Y.similar()
    sim.remaining_tendency_vjp(Yb, Tb, Y, p, 0.0)
    for seed in (3, 4):
        dc, df = _direction(Yc, Yf, seed)
        Tp, Tm = Y.similar(), Y.similar()
        sim.remaining_tendency(Tp, None, _fv(Yc + H * dc, Yf + H * df), p, 0.0)
        sim.remaining_tendency(Tm, None, _fv(Yc - H * dc, Yf - H * df), p, 0.0)
        fd = (_dot(Tb, Tp) - _dot(Tb, Tm)) / (2 * H)
        got = _dot(Yb, _fv(dc, df))
        assert abs(got - fd) <= 1e-6 * abs(fd), (got, fd)


@pytest.mark.gpu
def test_gpu_step_vjp_with_forcing():
    from gbdycore import simulation as sim
    cfg = hs_config(ft=np.float64)
    Yc, Yf = perturbed_state(cfg, w_amp=0.05)
    p = sim.AtmosCache(cfg)
    Y = _fv(Yc, Yf)

    def step(X):
        Z = X.copy()
        p.call("gb_step", Z.gb(), 0.0, float(cfg.dt), 1, 0)
        return Z

    Yb = _cotangent(*step(Y).numpy(), seed=8)
    Ybar = Yb.copy()
    sim.step_vjp(Ybar, Y, p, 0.0, cfg.dt)
    for seed in (9, 10):
        dc, df = _direction(Yc, Yf, seed)
        fd = (_dot(Yb, step(_fv(Yc + H * dc, Yf + H * df))) - _dot(Yb, step(_fv(Yc - H * dc, Yf - H * df)))) / (2 * H)
        got = _dot(Ybar, _fv(dc, df))
        assert abs(got - fd) <= 1e-6 * abs(fd), (got, fd)

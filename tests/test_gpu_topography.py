"""GPU parity over terrain-following levels: the terrain slab kernels, the column stage with
the column's own metric, the impenetrable filter u_3 = -u_h^3 / g^33 and the compensated
sums, through the C ABI, against the CPU oracle's terrain path (tests/test_topography_oracle.py
pins that path by conservation, the filter, the exact mass-row Jacobian and the flat limit).

Tolerances (max-norm error relative to each component's max magnitude): FP64 tendencies
<= 1e-12; FP64 steps as the flat steps on the small grids (rho, rho e_tot 1e-14, u_h 1e-12,
u_3 2e-11: the conditioning of u_3's tendency, see test_gpu_parity.py); FP32 tendencies
against the FP32 oracle <= 1e-4; FP32 steps against the FP64 oracle as the flat FP32 runs
(rho, rho e_tot 1e-5; u_h 1e-3; u_3 1e-2)."""
import copy

import numpy as np
import pytest

import oracle as O
import topography as T
from gbdycore import _native as N
from gbdycore import setups as S
from gbdycore import simulation as sim
from helpers import field_errors, oracle_geometry, small_config

pytestmark = pytest.mark.gpu

WARPS = {"linear": T.LinearWarp(), "sleve": T.SLEVEWarp()}


def _setup(ft=np.float64, h=3, z=8, warp="linear", surface=None, seed=7):
    cfg = small_config(ft=ft, h_elem=h, z_elem=z)
    g = copy.copy(oracle_geometry(cfg.with_(ft=np.float64)))
    zs = T.smooth_surface(g.xyz) if surface is None else surface(g)
    g.terrain = T.oracle_terrain(g, zs, WARPS[warp])
    cfgt = cfg.with_(z_surface=zs, warp=warp)
    o = O.Oracle(g, cfg.with_(ft=np.float64).oracle_params(dss_stage1=False))
    Yc, Yf = S.workload_state(g, cfg.with_(ft=np.float64), "plain")
    rng = np.random.default_rng(seed)
    dzf = g.terrain["Jf"] / (g.Jh[..., None] * ((g.R + g.terrain["zf"]) / g.R) ** 2)
    Yf = rng.normal(0, 0.05, size=Yf.shape) * dzf
    Yc[:, 3] *= 1 + 1e-3 * rng.normal(size=Yc[:, 3].shape)
    o.dss(Yc, Yf)
    return cfgt, g, o, Yc, Yf


def _dev(Yc, Yf, ft):
    return sim.FieldVector.from_numpy(np.ascontiguousarray(Yc, ft), np.ascontiguousarray(Yf, ft))


def _assert(errs, tol):
    tol = tol if isinstance(tol, dict) else {k: tol for k in errs}
    bad = {k: v for k, v in errs.items() if not v <= tol[k]}
    assert not bad, (bad, errs)


@pytest.mark.parametrize("ft,tol", [(np.float64, 1e-12), (np.float32, 1e-4)])
@pytest.mark.parametrize("warp", ["linear", "sleve"])
def test_terrain_remaining_tendency(ft, tol, warp):
    cfg, g, o, Yc, Yf = _setup(ft, warp=warp)
    ref = O.Oracle(g, cfg.with_(ft=np.float64).oracle_params(dss_stage1=False), ft).remaining_tendency(
        Yc.astype(ft), Yf.astype(ft))
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf, ft)
    Yt = Y.similar()
    sim.remaining_tendency(Yt, None, Y, p, 0.0)
    Tc, Tf = Yt.numpy()
    _assert(field_errors(Tc, Tf, ref[0], ref[1]), tol)


def test_terrain_filter_and_global_sums():
    cfg, g, o, Yc, Yf = _setup()
    Rc, Rf = Yc.copy(), Yf.copy()
    o.set_precomputed(Rc, Rf)
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf, np.float64)
    sim.set_precomputed_quantities(Y, p, 0.0)
    _, Gf = Y.numpy()
    for k in (0, -1):
        # -CT3(u_h) / g^33 from the closed-form metric here; the oracle forms the metric from
        # Cartesian basis vectors, where x_hat . e_a rounds to ~1e-16 |e_a| ~ 1e-10 against
        # slopes of ~1e3: its g^3a carry ~1e-13, and CT3(u_h) = g^31 u_1 + g^32 u_2 partly cancels
        assert np.abs(Gf[..., k] - Rf[..., k]).max() <= 1e-11 * np.abs(Rf[..., k]).max()
    assert np.abs(Rf[..., 0]).max() > 0
    assert np.array_equal(Gf[..., 1:-1], Yf[..., 1:-1])
    s = p.global_sums(Y)
    r = o.global_sums(Yc)
    assert np.all(np.abs(s - r) <= 1e-13 * np.abs(r))


@pytest.mark.parametrize("warp", ["linear", "sleve"])
def test_terrain_step_fp64_matches_oracle(warp):
    cfg, g, o, Yc, Yf = _setup(warp=warp)
    rc, rf = Yc.copy(), Yf.copy()
    o.step(rc, rf, cfg.dt, 3)
    s = sim.AtmosSimulation(cfg, state=(Yc, Yf))
    s.step(3, use_graph=True)
    Gc, Gf = s.Y.numpy()
    _assert(field_errors(Gc, Gf, rc, rf), {"rho": 1e-14, "rho_e_tot": 1e-14, "u_1": 1e-12, "u_2": 1e-12, "u_3": 2e-11})
    assert np.abs(Gf[..., 0]).max() > 0   # the filter's value over the terrain, not zero


def test_terrain_fp32_step_against_fp64_oracle():
    cfg, g, o, Yc, Yf = _setup(np.float32, h=4, z=10)
    rc, rf = Yc.copy(), Yf.copy()
    o.step(rc, rf, cfg.dt, 2)
    s = sim.AtmosSimulation(cfg, state=(Yc.astype(np.float32), Yf.astype(np.float32)))
    s.step(2, use_graph=True)
    Gc, Gf = s.Y.numpy()
    _assert(field_errors(Gc, Gf, rc, rf), {"rho": 1e-5, "rho_e_tot": 1e-5, "u_1": 1e-3, "u_2": 1e-3, "u_3": 1e-2})


def test_terrain_step_production_levels_fp32():
    """The production column (63 levels stretched from 30 m): the slabs exceed the default
    48 KB of dynamic shared memory and the column stage takes its 32-lane form."""
    cfg, g, o, Yc, Yf = _setup(np.float32, h=2, z=63)
    cfg = cfg.with_(dz_bottom=30.0)
    g = copy.copy(oracle_geometry(cfg.with_(ft=np.float64, z_surface=None)))
    g.terrain = T.oracle_terrain(g, cfg.z_surface, WARPS["linear"])
    o = O.Oracle(g, cfg.with_(ft=np.float64).oracle_params(dss_stage1=False))
    Yc, Yf = S.workload_state(g, cfg.with_(ft=np.float64), "plain")
    rc, rf = Yc.copy(), Yf.copy()
    o.step(rc, rf, cfg.dt, 2)
    s = sim.AtmosSimulation(cfg, state=(Yc.astype(np.float32), Yf.astype(np.float32)))
    s.step(2, use_graph=True)
    Gc, Gf = s.Y.numpy()
    _assert(field_errors(Gc, Gf, rc, rf), {"rho": 1e-5, "rho_e_tot": 1e-5, "u_1": 1e-3, "u_2": 1e-3, "u_3": 1e-2})


def test_flat_surface_terrain_context_matches_the_flat_step():
    """z_s = 0 through the terrain kernels equals the flat kernels (independent of the oracle)."""
    cfg, g, o, Yc, Yf = _setup(surface=lambda g: np.zeros((g.Nh, 16)))
    flat = cfg.with_(z_surface=None)
    a = sim.AtmosSimulation(cfg, state=(Yc, Yf))
    b = sim.AtmosSimulation(flat, state=(Yc, Yf))
    a.step(2)
    b.step(2)
    Ac, Af = a.Y.numpy()
    Bc, Bf = b.Y.numpy()
    _assert(field_errors(Ac, Af, Bc, Bf), {"rho": 1e-14, "rho_e_tot": 1e-14, "u_1": 1e-12, "u_2": 1e-12, "u_3": 2e-11})


@pytest.mark.parametrize("ft,tol", [(np.float64, 1e-12), (np.float32, 1e-4)])
def test_terrain_implicit_tendency_and_correction(ft, tol):
    cfg, g, o, Yc, Yf = _setup(ft, z=12)
    o32 = O.Oracle(g, cfg.with_(ft=np.float64).oracle_params(dss_stage1=False), ft)
    ref = o32.implicit_tendency(Yc.astype(ft), Yf.astype(ft))
    refc = o32.correct_implicit(Yc.astype(ft), Yf.astype(ft))
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf, ft)
    Yt = Y.similar()
    sim.implicit_tendency(Yt, Y, p, 0.0)
    e = field_errors(*Yt.numpy(), ref[0], ref[1])
    # u_3's tendency is the near-cancellation of gravity and the pressure gradient (FP32: 1e-3)
    _assert({k: v for k, v in e.items() if k in ("rho", "rho_e_tot")}, tol)
    assert e["u_3"] <= (tol if ft == np.float64 else 1e-3), e
    sim.correct_implicit_advection_tendency(Yt, Y, p, 0.0)
    e = field_errors(*Yt.numpy(), refc[0], refc[1])
    assert e["rho_e_tot"] <= tol, e


def test_terrain_jacobian_and_ldiv_with_the_uh_blocks():
    """update_jacobian + ldiv over terrain with a residual whose u_h part is nonzero: the
    (rho, u_h) and (rho e_tot, u_h) blocks (manual_sparse_jacobian.jl:150-187, 745-786) enter
    the scalar rows' right-hand sides."""
    cfg, g, o, Yc, Yf = _setup(z=40)   # two levels per lane
    dtg = 0.4358665215084590 * cfg.dt
    o.set_precomputed(Yc, Yf)
    o.update_jacobian(Yc, Yf, dtg)
    rng = np.random.default_rng(3)
    Rc = rng.normal(size=Yc.shape) * np.abs(Yc).max(axis=(0, 2, 3), keepdims=True) * 1e-3
    Rf = rng.normal(size=Yf.shape) * 0.1
    ref = o.ldiv(Rc, Rf)
    ref0 = o.ldiv(np.concatenate([Rc[:, :1], 0 * Rc[:, 1:3], Rc[:, 3:]], axis=1), Rf)
    assert np.abs(ref[0][:, 0] - ref0[0][:, 0]).max() > 1e-6 * np.abs(ref[0][:, 0]).max()
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf, np.float64)
    jac = sim.Jacobian(p)
    sim.update_jacobian(jac, Y, p, dtg, 0.0)
    dY = Y.similar()
    sim.ldiv(dY, jac, _dev(Rc, Rf, np.float64))
    _assert(field_errors(*dY.numpy(), ref[0], ref[1]), 1e-12)


def test_terrain_hook_loop_matches_fused_step():
    """The ClimaTimeSteppers stage loop through the hooks (stage states DSSed, the filter at
    every cache!) against the fused step over terrain."""
    cfg, g, o, Yc, Yf = _setup()
    a = sim.AtmosSimulation(cfg, state=(Yc, Yf))
    a.step(2, use_graph=False)
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf, np.float64)
    for k in range(2):
        sim.ars343_step_via_hooks(Y, p, k * cfg.dt, cfg.dt)
    _assert(field_errors(*Y.numpy(), *a.Y.numpy()), {"rho": 1e-14, "rho_e_tot": 1e-14, "u_1": 1e-12, "u_2": 1e-12, "u_3": 2e-11})


@pytest.mark.parametrize("rotate", [False, True])
def test_terrain_step_in_a_caller_layout(rotate):
    """Over terrain in the caller's element order and frames (the surface given in that layout):
    the library-order result moved there, bitwise for a renumbering alone."""
    from gbdycore import layout as LY
    cfg, g, o, Yc, Yf = _setup()
    a = sim.AtmosSimulation(cfg, state=(Yc, Yf))
    a.step(2)
    ref = a.Y.numpy()
    emap, eori = LY.random_layout(cfg.h_elem, seed=5, rotate=rotate)
    zs = np.asarray(cfg.z_surface)[emap[:, None], LY.NODE_OF[eori & 3]]
    Xc, Xf = LY.to_caller(Yc, Yf, emap, eori)
    b = sim.AtmosSimulation(cfg.with_(layout=(emap, eori), z_surface=zs), state=(Xc, Xf))
    b.step(2)
    out = LY.from_caller(*b.Y.numpy(), emap, eori)
    if not rotate:
        np.testing.assert_array_equal(out[0], ref[0])
        np.testing.assert_array_equal(out[1], ref[1])
    else:
        _assert(field_errors(out[0], out[1], ref[0], ref[1]),
                {"rho": 1e-14, "rho_e_tot": 1e-14, "u_1": 1e-12, "u_2": 1e-12, "u_3": 2e-11})


def test_terrain_production_step_matches_oracle():
    """The production grid (h_elem 30, z_elem 63 stretched from 30 m, dt 120 s, the workload's
    perturbed state) over the DCMIP-2-0-0 mountain: one FP64 step against the FP64 oracle within
    the 1e-12 target per field, and the FP32 step against the FP64 oracle."""
    from gbdycore import config as C
    O.set_threads(O.max_threads())
    base = C.production_h30()
    g = copy.copy(oracle_geometry(base.with_(ft=np.float64)))
    zs = T.dcmip200_nodes(g.xyz)
    g.terrain = T.oracle_terrain(g, zs, T.LinearWarp())
    cfg64 = base.with_(ft=np.float64, z_surface=zs)
    Yc, Yf = S.workload_state(g, cfg64, "production")
    o = O.Oracle(g, cfg64.oracle_params(dss_stage1=False))
    r1 = (Yc.copy(), Yf.copy())
    o.step(*r1, cfg64.dt, 1)
    del o
    s = sim.AtmosSimulation(cfg64, state=(Yc, Yf))
    s.step(1)
    e = field_errors(*s.Y.numpy(), *r1)
    print("terrain, FP64 vs oracle, 1 step:", e)
    _assert(e, {"rho": 1e-12, "rho_e_tot": 1e-12, "u_1": 1e-12, "u_2": 1e-12, "u_3": 2e-12})
    s32 = sim.AtmosSimulation(cfg64.with_(ft=np.float32), state=(Yc.astype(np.float32), Yf.astype(np.float32)))
    s32.step(1)
    e = field_errors(*s32.Y.numpy(), *r1)
    print("terrain, FP32 vs FP64 oracle, 1 step:", e)
    _assert(e, {"rho": 2e-6, "rho_e_tot": 3e-6, "u_1": 1e-4, "u_2": 1e-4, "u_3": 1e-3})


def test_terrain_context_refuses_what_is_not_built():
    cfg, g, o, Yc, Yf = _setup()
    p = sim.AtmosCache(cfg)
    Y = _dev(Yc, Yf, np.float64)
    Yt = Y.similar()
    for call in (lambda: p.call("gb_jacobian_solve_noalloc", Yt.gb(), Y.gb(), Y.gb(), 10.0),
                 lambda: p.call("gb_step_vjp", Yt.gb(), Y.gb(), 0.0, float(cfg.dt), None)):
        with pytest.raises(N.GBError) as ei:
            call()
        assert ei.value.code == N.GB_ERR_ARG and "terrain" in str(ei.value)

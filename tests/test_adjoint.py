"""Reverse mode (the pullback of the differentiable step) against central finite differences.

Each reverse kernel is checked by the dot-product identity
    <ybar, (f(x + h d) - f(x - h d)) / 2h>  ==  <f_vjp(ybar), d>
on the FP64 forward of the same library (which matches the FP64 oracle to
1e-10), for the layers of the step and for the whole checkpointed trajectory,
including the derivatives with respect to the hyperdiffusivity nu and the
Rayleigh sponge rate (config: sponge above 15 km with rate 1e-3 s^-1).
"""
import numpy as np
import pytest

from helpers import perturbed_state, small_config

RATE = 1.0e-3
GAMMA = 0.4358665215084590
H = 1.0e-6  # relative finite-difference step (directions are scaled to the fields)
HP = 1.0e-4  # relative step for the scalar parameters (the losses are O(1e7): a smaller step drowns in round-off)
# Over several steps the van Leer limiter's min/max branches make the map piecewise smooth; a
# smaller state step keeps the central differences from straddling a branch switch.
HT = 1.0e-8


def adj_config(**kw):
    base = dict(sponge_zd=15000.0, alpha_uh=RATE, alpha_w=RATE)
    base.update(kw)
    return small_config(np.float64, **base)


def _sim():
    from gbdycore import simulation as sim
    return sim


def _fv(Yc, Yf):
    return _sim().FieldVector.from_numpy(np.ascontiguousarray(Yc), np.ascontiguousarray(Yf))


def _dot(A, B):
    return float((A.c * B.c).sum().item() + (A.f * B.f).sum().item())


def _scaled(shape_c, shape_f, ref_c, ref_f, seed, comp_axis=1):
    """Random direction with each component scaled to the RMS of the reference field."""
    rng = np.random.default_rng(seed)
    dc = rng.standard_normal(shape_c)
    for c in range(shape_c[comp_axis]):
        s = np.sqrt(np.mean(ref_c[:, c] ** 2)) if ref_c is not None else 1.0
        dc[:, c] *= s if s > 0 else 1.0
    sf = np.sqrt(np.mean(ref_f ** 2)) if ref_f is not None else 1.0
    df = rng.standard_normal(shape_f) * (sf if sf > 0 else 1.0)
    return dc, df


def _axpy(Yc, Yf, a, dc, df):
    return _fv(Yc + a * dc, Yf + a * df)


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


@pytest.fixture(scope="module")
def setup():
    cfg = adj_config()
    Yc, Yf = perturbed_state(cfg, w_amp=0.05, dtype=np.float64)
    return cfg, Yc, Yf


@pytest.mark.gpu
def test_dss_transpose(setup):
    sim = _sim()
    cfg, Yc, Yf = setup
    p = sim.AtmosCache(cfg)
    rng = np.random.default_rng(1)
    X = _fv(rng.standard_normal(Yc.shape), rng.standard_normal(Yf.shape))
    Y = _fv(rng.standard_normal(Yc.shape), rng.standard_normal(Yf.shape))
    DX = X.copy()
    sim.dss(DX, p, 0.0)
    DtY = Y.copy()
    sim.dss_transpose(DtY, p)
    assert rel(_dot(DX, Y), _dot(X, DtY)) < 1e-13


@pytest.mark.gpu
def test_remaining_tendency_vjp(setup):
    sim = _sim()
    cfg, Yc, Yf = setup
    p = sim.AtmosCache(cfg)
    Y = _fv(Yc, Yf)
    T = Y.similar()
    sim.remaining_tendency(T, None, Y, p, 0.0)
    Tn = T.numpy()
    rng = np.random.default_rng(2)
    Tb = _fv(rng.standard_normal(Yc.shape) / np.maximum(np.abs(Tn[0]).max(axis=(0, 2, 3), keepdims=True), 1e-30),
             rng.standard_normal(Yf.shape) / max(np.abs(Tn[1]).max(), 1e-30))
    Yb = Y.similar()
    dpar = sim.remaining_tendency_vjp(Yb, Tb, Y, p, 0.0)
    for seed in (3, 4):
        dc, df = _scaled(Yc.shape, Yf.shape, Yc, Yf, seed)
        Tp, Tm = Y.similar(), Y.similar()
        sim.remaining_tendency(Tp, None, _axpy(Yc, Yf, H, dc, df), p, 0.0)
        sim.remaining_tendency(Tm, None, _axpy(Yc, Yf, -H, dc, df), p, 0.0)
        fd = (_dot(Tb, Tp) - _dot(Tb, Tm)) / (2 * H)
        assert rel(_dot(Yb, _fv(dc, df)), fd) < 1e-6
    # parameters: nu (nu_s follows) and the sponge rate
    for k, mk in ((0, lambda c, s: c.with_(nu=c.nu * s)),
                  (1, lambda c, s: c.with_(alpha_uh=RATE * s, alpha_w=RATE * s))):
        vals = []
        for s in (1 + HP, 1 - HP):
            q = sim.AtmosCache(mk(cfg, s))
            Tq = Y.similar()
            sim.remaining_tendency(Tq, None, Y, q, 0.0)
            vals.append(_dot(Tb, Tq))
        scale = cfg.nu if k == 0 else RATE
        fd = (vals[0] - vals[1]) / (2 * HP * scale)
        assert rel(dpar[k], fd) < 1e-6, (k, dpar[k], fd)


@pytest.mark.gpu
def test_implicit_stage_vjp(setup):
    sim = _sim()
    cfg, Yc, Yf = setup
    p = sim.AtmosCache(cfg)
    dtg = GAMMA * cfg.dt
    Uh = _fv(Yc, Yf)

    def run(X, q=p):
        U, Ti = X.similar(), sim.reduced_like(X)
        sim.implicit_stage(U, Ti, X, q, dtg)
        return U, Ti

    U, Ti = run(Uh)
    rng = np.random.default_rng(5)
    Un, Tin = U.numpy(), Ti.numpy()
    Ub = _fv(rng.standard_normal(Yc.shape) / np.maximum(np.abs(Un[0]).max(axis=(0, 2, 3), keepdims=True), 1e-30),
             rng.standard_normal(Yf.shape) / max(np.abs(Un[1]).max(), 1e-30))
    Tib = _fv(rng.standard_normal(Tin[0].shape) / np.maximum(np.abs(Tin[0]).max(axis=(0, 2, 3), keepdims=True), 1e-30),
              rng.standard_normal(Yf.shape) / max(np.abs(Tin[1]).max(), 1e-30))
    Uhb = Uh.similar()
    dpar = sim.implicit_stage_vjp(Uhb, Ub, Tib, Uh, p, dtg)

    def J(X, q=p):
        Uo, To = run(X, q)
        return _dot(Ub, Uo) + _dot(Tib, To)

    for seed in (6, 7):
        dc, df = _scaled(Yc.shape, Yf.shape, Yc, Yf, seed)
        fd = (J(_axpy(Yc, Yf, H, dc, df)) - J(_axpy(Yc, Yf, -H, dc, df))) / (2 * H)
        assert rel(_dot(Uhb, _fv(dc, df)), fd) < 1e-6
    # the sponge acts on the top levels only, so J's change with the rate is small against J
    # itself and a central difference at a small step is round-off bound (measured: 1.6e-6 at
    # a 1e-4 relative step, 2.1e-5 at 1e-5); larger steps with Richardson extrapolation,
    # (4 D(h) - D(2h)) / 3, remove the h^2 truncation term instead
    def D(hp):
        vals = [J(Uh, sim.AtmosCache(cfg.with_(alpha_uh=RATE * s, alpha_w=RATE * s))) for s in (1 + hp, 1 - hp)]
        return (vals[0] - vals[1]) / (2 * hp * RATE)
    fd = (4 * D(1e-3) - D(2e-3)) / 3
    assert rel(dpar[1], fd) < 1e-6, (dpar[1], fd)
    assert dpar[0] == 0.0


@pytest.mark.gpu
def test_step_vjp(setup):
    sim = _sim()
    cfg, Yc, Yf = setup
    p = sim.AtmosCache(cfg)
    Y = _fv(Yc, Yf)

    def step(X, q=p):
        Z = X.copy()
        q.call("gb_step", Z.gb(), 0.0, float(cfg.dt), 1, 0)
        return Z

    Y1 = step(Y).numpy()
    rng = np.random.default_rng(8)
    Yb = _fv(rng.standard_normal(Yc.shape) / np.maximum(np.abs(Y1[0]).max(axis=(0, 2, 3), keepdims=True), 1e-30),
             rng.standard_normal(Yf.shape) / max(np.abs(Y1[1]).max(), 1e-30))
    Ybar = Yb.copy()
    dpar = sim.step_vjp(Ybar, Y, p, 0.0, cfg.dt)
    for seed in (9, 10):
        dc, df = _scaled(Yc.shape, Yf.shape, Yc, Yf, seed)
        fd = (_dot(Yb, step(_axpy(Yc, Yf, H, dc, df))) - _dot(Yb, step(_axpy(Yc, Yf, -H, dc, df)))) / (2 * H)
        assert rel(_dot(Ybar, _fv(dc, df)), fd) < 1e-6
    for k, mk, scale in ((0, lambda s: cfg.with_(nu=cfg.nu * s), cfg.nu),
                         (1, lambda s: cfg.with_(alpha_uh=RATE * s, alpha_w=RATE * s), RATE)):
        vals = [_dot(Yb, step(Y, sim.AtmosCache(mk(s)))) for s in (1 + HP, 1 - HP)]
        assert rel(dpar[k], (vals[0] - vals[1]) / (2 * HP * scale)) < 1e-6, (k, dpar[k])


@pytest.mark.gpu
def test_trajectory_gradient_checkpointed(setup):
    """J = 1/2 |rho e_tot(t_N) - target|^2 over 3 steps: the checkpointed pullback
    (every 2 steps) against FD in random directions and in (nu, rate), and equal
    to the pullback without intermediate checkpoints."""
    import torch
    sim = _sim()
    cfg, Yc, Yf = setup
    p = sim.AtmosCache(cfg)
    nsteps = 3
    rng = np.random.default_rng(11)
    target = _fv(Yc * (1 + 1e-3 * rng.standard_normal(Yc.shape)), Yf)

    def forward(X, q=p):
        Z = X.copy()
        q.call("gb_step", Z.gb(), 0.0, float(cfg.dt), nsteps, 0)
        return Z

    def loss_and_grad(YN):
        d = (YN.c[:, 3] - target.c[:, 3])
        G = YN.similar()
        G.c[:, 3] = d
        return 0.5 * float((d * d).sum().item()), G

    Y0 = _fv(Yc, Yf)
    J0, G2, dnu2, dal2, peak = sim.gradient(p, Y0, nsteps, loss_and_grad, checkpoint_every=2)
    _, G3, dnu3, dal3, _ = sim.gradient(p, Y0, nsteps, loss_and_grad, checkpoint_every=3)
    assert torch.equal(G2.c, G3.c) and torch.equal(G2.f, G3.f) and dnu2 == dnu3 and dal2 == dal3
    assert peak > 0
    # keeping the stage data of more trailing segments (less recomputation) changes nothing
    for every, keep in ((1, 2), (1, 3), (2, 2)):
        _, Gk, dnuk, dalk, peak_k = sim.gradient(p, Y0, nsteps, loss_and_grad, checkpoint_every=every,
                                                 record_segments=keep)
        assert torch.equal(Gk.c, G2.c) and torch.equal(Gk.f, G2.f) and dnuk == dnu2 and dalk == dal2, (every, keep)
    p.call("gb_adjoint_set_record_segments", 1)
    for seed in (12, 13, 14):
        dc, df = _scaled(Yc.shape, Yf.shape, Yc, Yf, seed)
        fd = (loss_and_grad(forward(_axpy(Yc, Yf, HT, dc, df)))[0] -
              loss_and_grad(forward(_axpy(Yc, Yf, -HT, dc, df)))[0]) / (2 * HT)
        assert rel(_dot(G2, _fv(dc, df)), fd) < 1e-5, (seed, _dot(G2, _fv(dc, df)), fd)
    for val, mk, scale in ((dnu2, lambda s: cfg.with_(nu=cfg.nu * s), cfg.nu),
                           (dal2, lambda s: cfg.with_(alpha_uh=RATE * s, alpha_w=RATE * s), RATE)):
        vals = [loss_and_grad(forward(Y0, sim.AtmosCache(mk(s))))[0] for s in (1 + HP, 1 - HP)]
        assert rel(val, (vals[0] - vals[1]) / (2 * HP * scale)) < 1e-5


@pytest.mark.gpu
def test_step_vjp_deterministic_with_separate_blocks(setup):
    """Repeated pullbacks into freshly allocated (separate c and f) cotangents agree bitwise."""
    import torch
    sim = _sim()
    cfg, Yc, Yf = setup
    p = sim.AtmosCache(cfg)
    Y = _fv(Yc, Yf)
    rng = np.random.default_rng(8)
    Wb = _fv(rng.standard_normal(Yc.shape), rng.standard_normal(Yf.shape))
    outs = []
    for _ in range(8):
        pad = torch.empty(int(rng.integers(1, 4096)), dtype=torch.float64, device="cuda")  # vary the placement
        G = Wb.copy()
        sim.step_vjp(G, Y, p, 0.0, cfg.dt)
        outs.append(G)
        del pad
    for G in outs[1:]:
        assert torch.equal(G.c, outs[0].c) and torch.equal(G.f, outs[0].f)


@pytest.mark.gpu
def test_step_vjp_tall_columns():
    """z_elem = 70: the slab kernels' second level sweep, pass B^T reading the Laplacians and
    the cotangent from global memory (FP64 slabs too tall to stage) and the 4-levels-per-lane
    column pullback.  Without the van Leer limiter: at this height its min/max branches sit
    close enough to the state that central differences straddle them (the limiter's own
    pullback is covered at smaller heights)."""
    sim = _sim()
    cfg = adj_config(z_elem=70, upwinding="none")
    Yc, Yf = perturbed_state(cfg, w_amp=0.05, dtype=np.float64)
    p = sim.AtmosCache(cfg)
    Y = _fv(Yc, Yf)

    def step(X):
        Z = X.copy()
        p.call("gb_step", Z.gb(), 0.0, float(cfg.dt), 1, 0)
        return Z

    Y1 = step(Y).numpy()
    rng = np.random.default_rng(21)
    Yb = _fv(rng.standard_normal(Yc.shape) / np.maximum(np.abs(Y1[0]).max(axis=(0, 2, 3), keepdims=True), 1e-30),
             rng.standard_normal(Yf.shape) / max(np.abs(Y1[1]).max(), 1e-30))
    Ybar = Yb.copy()
    sim.step_vjp(Ybar, Y, p, 0.0, cfg.dt)
    dc, df = _scaled(Yc.shape, Yf.shape, Yc, Yf, 22)
    fd = (_dot(Yb, step(_axpy(Yc, Yf, H, dc, df))) - _dot(Yb, step(_axpy(Yc, Yf, -H, dc, df)))) / (2 * H)
    assert rel(_dot(Ybar, _fv(dc, df)), fd) < 1e-6


@pytest.mark.gpu
def test_remaining_tendency_vjp_at_zero_hyperdiffusion(setup):
    """nu = 0: d/dnu from the direct form (the transposes carry no nu then)."""
    sim = _sim()
    cfg0, Yc, Yf = setup
    nu0 = cfg0.nu
    cfg = cfg0.with_(nu=0.0)
    p = sim.AtmosCache(cfg)
    Y = _fv(Yc, Yf)
    T = Y.similar()
    sim.remaining_tendency(T, None, Y, p, 0.0)
    rng = np.random.default_rng(23)
    Tn = sim.AtmosCache(cfg0)
    T0 = Y.similar()
    sim.remaining_tendency(T0, None, Y, Tn, 0.0)
    T0n = T0.numpy()
    Tb = _fv(rng.standard_normal(Yc.shape) / np.maximum(np.abs(T0n[0]).max(axis=(0, 2, 3), keepdims=True), 1e-30),
             rng.standard_normal(Yf.shape) / max(np.abs(T0n[1]).max(), 1e-30))
    Yb = Y.similar()
    dpar = sim.remaining_tendency_vjp(Yb, Tb, Y, p, 0.0)
    vals = []
    for s in (1.0, -1.0):
        q = sim.AtmosCache(cfg.with_(nu=s * HP * nu0))
        Tq = Y.similar()
        sim.remaining_tendency(Tq, None, Y, q, 0.0)
        vals.append(_dot(Tb, Tq))
    fd = (vals[0] - vals[1]) / (2 * HP * nu0)
    assert rel(dpar[0], fd) < 1e-6, (dpar[0], fd)


@pytest.mark.gpu
@pytest.mark.parametrize("z_elem", [8, 45])
def test_step_vjp_fp32_agrees_with_fp64(z_elem):
    """The FP32 pullback (the production precision) against the FP64 one: <Ybar, d> for the same
    state, cotangent and direction agree to FP32 accuracy of the tangent map (z_elem = 45: the
    32-lane column pullback that FP32 runs at six CTAs per SM)."""
    sim = _sim()
    cfg64 = adj_config(z_elem=z_elem)
    Yc, Yf = perturbed_state(cfg64, w_amp=0.05, dtype=np.float64)
    dc, df = _scaled(Yc.shape, Yf.shape, Yc, Yf, 31)
    rng = np.random.default_rng(30)
    bc = rng.standard_normal(Yc.shape)
    bf = rng.standard_normal(Yf.shape)
    out = {}
    for ft in (np.float64, np.float32):
        cfg = cfg64.with_(ft=ft)
        p = sim.AtmosCache(cfg)
        Y = sim.FieldVector.from_numpy(Yc.astype(ft), Yf.astype(ft))
        Z = Y.copy()
        p.call("gb_step", Z.gb(), 0.0, float(cfg.dt), 1, 0)
        Zc, Zf = Z.numpy()
        scale_c = np.maximum(np.abs(Zc.astype(np.float64)).max(axis=(0, 2, 3), keepdims=True), 1e-30)
        Yb = sim.FieldVector.from_numpy((bc / scale_c).astype(ft), (bf / max(np.abs(Zf).max(), 1e-30)).astype(ft))
        dpar = sim.step_vjp(Yb, Y, p, 0.0, cfg.dt)
        Ybc, Ybf = Yb.numpy()
        out[ft] = (float((Ybc.astype(np.float64) * dc).sum() + (Ybf.astype(np.float64) * df).sum()), dpar)
    (g64, p64), (g32, p32) = out[np.float64], out[np.float32]
    assert rel(g32, g64) < 1e-3, (g32, g64)
    assert rel(p32[0], p64[0]) < 1e-3 and rel(p32[1], p64[1]) < 1e-3, (p32, p64)

"""Batched standalone columns of uneven height: the GPU Newton solve against the oracle.

The reference drives the column solve through NewtonsMethod (src/simulation/integrator.jl:63-120)
on ColumnGrid columns (src/simulation/grids.jl:93-127); the oracle repeats the
dycore_oracle.cpp implicit-stage iteration per column (column_oracle.py).
"""
import numpy as np
import pytest

from gbdycore import config as C
from gbdycore import columns as CB
import column_oracle

GAMMA = 0.4358665215084590
DTG = GAMMA * 120.0
# every height class: 4/8/16/32 lanes x 4 levels and 8/16/32 lanes x 2 levels, both sides of each edge
EDGE_HEIGHTS = [2, 3, 7, 14, 15, 16, 30, 31, 32, 47, 62, 63, 64, 90, 126, 127]


def cfg_for(ft):
    return C.DycoreConfig(h_elem=1, z_elem=10, z_max=30000.0, z_stretch=False, ft=ft, dt=120.0)


def heights(n_random=40, seed=5):
    rng = np.random.default_rng(seed)
    return np.array(EDGE_HEIGHTS + list(rng.integers(2, 128, n_random)), dtype=np.int32)


def oracle_solve(cfg, z, Yc, Yf, iters):
    return column_oracle.newton(cfg.with_(ft=np.float64), z, Yc, Yf, Yc, Yf, DTG, iters, CB.column_faces)


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


# ---------------------------------------------------------------- CPU
def test_heights_seeded_and_in_range():
    z = CB.batch_heights(20000)
    assert z.min() >= 30 and z.max() <= 127 and len(np.unique(z)) == 98
    assert np.array_equal(z, CB.batch_heights(20000))


def test_batch_state_layout():
    cfg = cfg_for(np.float64)
    z = np.array([3, 5, 2], dtype=np.int32)
    Yc, Yf = CB.batch_state(cfg, z)
    assert Yc.shape == (4, 10) and Yf.shape == (13,)
    off = CB.offsets(z)
    assert list(off) == [0, 3, 8]
    for k, n in enumerate(z):
        f = Yf[off[k] + k: off[k] + k + n + 1]
        assert f[0] == 0 and f[-1] == 0
        assert np.all(Yc[0, off[k]: off[k] + n] > 0)
    assert np.all(Yc[1:3] == 0)
    Yc2, Yf2 = CB.batch_state(cfg, z)
    assert np.array_equal(Yc, Yc2) and np.array_equal(Yf, Yf2)


def test_oracle_column_newton_converges():
    cfg = cfg_for(np.float64)
    z = np.array([5, 9, 17, 30, 5, 40], dtype=np.int32)
    Yc, Yf = CB.batch_state(cfg, z)
    _, _, rn = oracle_solve(cfg, z, Yc, Yf, 3)
    # the manual Jacobian is approximate (manual_sparse_jacobian.jl), so Newton
    # converges linearly: measured factors ~1e-7 (rho), ~1e-6 (rho e_tot), ~5e-3 (u_3)
    assert np.all(rn[0] > 0)
    assert np.all(rn[1] < 1e-2 * rn[0])
    assert np.all(rn[2] < 1e-1 * rn[1])


def test_oracle_column_matches_full_oracle_column():
    """A standalone column solves like the same column inside the sphere oracle
    when the horizontal metric is flat: compare two packings of one batch."""
    cfg = cfg_for(np.float64)
    z = np.array([8] * 20, dtype=np.int32)
    Yc, Yf = CB.batch_state(cfg, z)
    a = oracle_solve(cfg, z, Yc, Yf, 2)
    perm = np.arange(20)[::-1]
    off = CB.offsets(z)
    Pc = np.concatenate([Yc[:, off[k]: off[k] + 8] for k in perm], axis=1)
    Pf = np.concatenate([Yf[off[k] + k: off[k] + k + 9] for k in perm])
    b = oracle_solve(cfg, z, Pc, Pf, 2)
    for j, k in enumerate(perm):
        assert np.array_equal(a[0][:, off[k]: off[k] + 8], b[0][:, off[j]: off[j] + 8])


# ---------------------------------------------------------------- GPU
def _gpu(cfg, z, Yc, Yf, iters=2, mode="graph", variant=None):
    import torch
    B = CB.ColumnBatch(cfg, z)
    if variant is not None:
        B.set_variant(variant)
    Uh = B.state(Yc, Yf)
    U = Uh.copy()
    rn = B.solve(U, Uh, DTG, iters, mode)
    torch.cuda.synchronize()
    return U.numpy(), rn, B


@pytest.mark.gpu
@pytest.mark.parametrize("iters", [1, 2])
def test_gpu_fp64_matches_oracle(iters):
    cfg = cfg_for(np.float64)
    z = heights()
    Yc, Yf = CB.batch_state(cfg, z)
    (gc, gf), rn, _ = _gpu(cfg, z, Yc, Yf, iters)
    oc, of, orn = oracle_solve(cfg, z, Yc, Yf, iters)
    assert rel(gc[0], oc[0]) < 1e-12
    assert rel(gc[3], oc[3]) < 1e-12
    assert rel(gf, of) < 1e-10
    np.testing.assert_allclose(rn, orn, rtol=1e-7)


@pytest.mark.gpu
def test_gpu_fp32_against_fp64_oracle():
    cfg = cfg_for(np.float32)
    z = heights()
    Yc, Yf = CB.batch_state(cfg_for(np.float64), z)
    (gc, gf), rn, _ = _gpu(cfg, z, Yc.astype(np.float32), Yf.astype(np.float32))
    oc, of, orn = oracle_solve(cfg, z, Yc, Yf, 2)
    assert rel(gc[0], oc[0]) < 1e-5
    assert rel(gc[3], oc[3]) < 1e-5
    assert rel(gf, of) < 2e-3  # u_3 after the solve: cancellation of O(1e5) hydrostatic terms in FP32
    assert np.all(rn[1] < 1e-1 * rn[0])
    # first-iteration residual sums of squares (compensated FP32 pairs per column, reduced in
    # FP32 TwoSum arithmetic) against the FP64 oracle's
    np.testing.assert_allclose(rn[0], orn[0], rtol=5e-2)


@pytest.mark.gpu
def test_gpu_modes_and_variants_agree():
    cfg = cfg_for(np.float64)
    z = heights(60, seed=9)
    Yc, Yf = CB.batch_state(cfg, z)
    (ac, af), _, _ = _gpu(cfg, z, Yc, Yf, mode="graph")
    (bc, bf), _, _ = _gpu(cfg, z, Yc, Yf, mode="persistent")
    assert np.array_equal(ac, bc) and np.array_equal(af, bf)
    (cc, cf), _, _ = _gpu(cfg, z, Yc, Yf, mode="per_height")
    assert rel(cc[3], ac[3]) < 1e-13 and rel(cf, af) < 1e-11
    for v in range(5):
        (vc, vf), _, _ = _gpu(cfg, z, Yc, Yf, mode="graph", variant=v)
        assert rel(vc[3], ac[3]) < 1e-13 and rel(vf, af) < 1e-11


@pytest.mark.gpu
def test_gpu_graph_replay_and_autotune():
    import torch
    cfg = cfg_for(np.float32)
    z = heights(200, seed=3)
    Yc, Yf = CB.batch_state(cfg, z)
    B = CB.ColumnBatch(cfg, z)
    Uh = B.state(Yc, Yf)
    U0 = Uh.copy()
    choice, ms = B.autotune(U0, Uh, DTG, 2, reps=2)
    assert 0 <= choice < 5 and np.all(ms > 0) and ms[choice] == ms.min()
    assert torch.equal(U0.c, Uh.c) and torch.equal(U0.f, Uh.f)  # left unchanged
    outs = []
    U = Uh.copy()
    for _ in range(2):  # same buffers: the second solve replays the captured graph
        U.assign_(Uh)
        B.solve(U, Uh, DTG, 2, "graph")
        outs.append(U.numpy())
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


@pytest.mark.gpu
def test_gpu_invalid_arguments():
    from gbdycore import _native as N
    cfg = cfg_for(np.float32)
    z = np.array([10, 20], dtype=np.int32)
    Yc, Yf = CB.batch_state(cfg, z)
    B = CB.ColumnBatch(cfg, z)
    U = B.state(Yc, Yf)
    with pytest.raises(N.GBError) as e:
        B.solve(U, U.copy(), DTG, 0)
    assert e.value.code == N.GB_ERR_ARG
    with pytest.raises(N.GBError):
        CB.ColumnBatch(cfg, np.array([10, 128], dtype=np.int32))

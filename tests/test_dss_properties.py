"""Properties of the oracle's direct stiffness summation (the weighted DSS of
src/prognostic_equations/constrain_state.jl:59-64) on random fields: a projection
(DSS(DSS(x)) = DSS(x)), linear, leaving continuous fields unchanged, and equalising every
collocated copy (the pullback's DSS transpose relies on the first).  CPU only; uses hypothesis
where it is installed."""
import numpy as np
import pytest

from helpers import make_oracle, small_config

hyp = pytest.importorskip("hypothesis")
st = pytest.importorskip("hypothesis.strategies")

CFG = small_config(h_elem=2, z_elem=3)
O = make_oracle(CFG)
NH, NV = 6 * CFG.h_elem ** 2, CFG.z_elem


def _random(seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal((NH, 4, 16, NV)), rng.standard_normal((NH, 16, NV + 1))


def _dss(c, f):
    c, f = c.copy(), f.copy()
    O.dss(c, f)
    return c, f


def _close(a, b, tol=1e-13):
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1.0)


@hyp.settings(max_examples=15, deadline=None)
@hyp.given(st.integers(0, 2 ** 31 - 1))
def test_dss_is_a_projection(seed):
    c1, f1 = _dss(*_random(seed))
    c2, f2 = _dss(c1, f1)
    assert _close(c2, c1) and _close(f2, f1)


@hyp.settings(max_examples=15, deadline=None)
@hyp.given(st.integers(0, 2 ** 31 - 1), st.floats(-3.0, 3.0), st.floats(-3.0, 3.0))
def test_dss_is_linear(seed, a, b):
    x, y = _random(seed), _random(seed + 1)
    lc, lf = _dss(a * x[0] + b * y[0], a * x[1] + b * y[1])
    xc, xf = _dss(*x)
    yc, yf = _dss(*y)
    assert _close(lc, a * xc + b * yc, 1e-12) and _close(lf, a * xf + b * yf, 1e-12)


def test_dss_equalises_collocated_scalars():
    # rho, rho e_tot and u_3 are scalars: after the DSS every copy of a node holds the same value
    g = O.geom
    c, f = _dss(*_random(7))
    key = np.round(g.xyz.reshape(-1, 3) * 1e9).astype(np.int64)
    _, inv = np.unique(key, axis=0, return_inverse=True)
    inv = inv.reshape(NH, 16)
    for field in (c[:, 0], c[:, 3]):
        for u in range(inv.max() + 1):
            vals = field[inv == u]          # [copies, Nv]
            assert np.abs(vals - vals[0]).max() <= 1e-14 * max(np.abs(vals).max(), 1.0)
    for u in range(inv.max() + 1):
        vals = f[inv == u]
        assert np.abs(vals - vals[0]).max() <= 1e-14 * max(np.abs(vals).max(), 1.0)

"""Analytic pins of the spectral-element operators, independent of any restatement choice.

The oracle's horizontal Laplacians (the operators of prep_hyperdiffusion_tendency!,
src/prognostic_equations/hyperdiffusion.jl:140-147, with the DSS of
remaining_tendency.jl:18-21) are applied to spherical harmonics: the restriction to the
sphere of a harmonic polynomial of degree l, and the gradient and rotational vector fields
made from it.  On a sphere of radius a each is an eigenfunction with eigenvalue
-l (l + 1) / a^2 (for the vector fields, of the grad-div minus curl-curl Laplacian).  The
discrete operators must reproduce that to the discretisation error of Nq = 4 elements and
converge as the grid is refined.  The GPU kernels are held to the oracle elsewhere, so this
pins the operator definitions the two share: the GLL derivative, the weak and strong
forms, the metric terms of the equiangular cubed sphere and the DSS (CPU only).
"""
import numpy as np
import pytest

import oracle as O
from geometry import OracleGeometry
from gbdycore import config as C

# harmonic polynomials P(x, y, z) of degree l and their gradients
HARMONICS = {
    "xy (l=2)": (2, lambda x, y, z: x * y, lambda x, y, z: np.stack([y, x, 0 * z], -1)),
    "2z^2-x^2-y^2 (l=2)": (2, lambda x, y, z: 2 * z * z - x * x - y * y,
                           lambda x, y, z: np.stack([-2 * x, -2 * y, 4 * z], -1)),
    "xyz (l=3)": (3, lambda x, y, z: x * y * z, lambda x, y, z: np.stack([y * z, x * z, x * y], -1)),
    "xy(x^2-y^2) (l=4)": (4, lambda x, y, z: x ** 3 * y - x * y ** 3,
                          lambda x, y, z: np.stack([3 * x * x * y - y ** 3, x ** 3 - 3 * x * y * y, 0 * z], -1)),
}


def _setup(h):
    cfg = C.DycoreConfig(h_elem=h, z_elem=2, z_max=30000.0, ft=np.float64)
    g = OracleGeometry(h, 2, cfg.z_max, False, 500.0, radius=cfg.constants["radius"], omega=cfg.constants["omega"])
    o = O.Oracle(g, cfg.oracle_params(), np.float64)
    return g, o


def _errors(h, name):
    l, P, dP = HARMONICS[name]
    g, o = _setup(h)
    x, y, z = g.xyz[..., 0], g.xyz[..., 1], g.xyz[..., 2]
    f = P(x, y, z)                                                     # [Nh, 16]
    grad = dP(x, y, z)                                                 # [Nh, 16, 3]
    rot = np.cross(g.xyz, grad)
    out = {}
    for kind, vec in (("gradient", grad), ("rotational", rot)):
        # covariant components on the level's basis r e_i of the surface field (1/(R r)) vec:
        # u_i = e_i . vec / R at every level
        u1 = np.einsum("end,end->en", g.ecov[:, :, 0], vec) / g.R
        u2 = np.einsum("end,end->en", g.ecov[:, :, 1], vec) / g.R
        X = np.zeros((g.Nh, 4, 16, g.Nv))
        X[:, 0] = f[..., None]
        X[:, 1] = u1[..., None]
        X[:, 2] = u2[..., None]
        L = o.laplacians(X)
        for v in range(g.Nv):
            lam = -l * (l + 1) / (g.R * g.rc[v]) ** 2
            if kind == "gradient":
                e = np.abs(L[:, 0, :, v] - lam * f).max() / np.abs(lam * f).max()
                out["scalar"] = max(out.get("scalar", 0.0), e)
            ev = max(np.abs(L[:, 1, :, v] - lam * u1).max(), np.abs(L[:, 2, :, v] - lam * u2).max())
            ev /= np.abs(lam) * max(np.abs(u1).max(), np.abs(u2).max())
            out[kind] = max(out.get(kind, 0.0), ev)
    return out


@pytest.mark.parametrize("name", list(HARMONICS))
def test_laplacians_of_spherical_harmonics(name):
    # max-norm relative errors; a second derivative of cubic elements converges at second
    # order at the nodes (measured: 4-9e-3 scalar, 1.4-3.7e-2 vector at h_elem 6, each
    # 2.3-4.4x smaller at h_elem 12 and again 2.8-4.3x at 24).  A wrong metric term,
    # derivative matrix or DSS weight would leave an O(1) error that does not converge.
    e6 = _errors(6, name)
    e12 = _errors(12, name)
    for k, lim6, lim12 in (("scalar", 1.5e-2, 5e-3), ("gradient", 5e-2, 1.2e-2), ("rotational", 5e-2, 1.2e-2)):
        assert e6[k] < lim6 and e12[k] < lim12, (name, k, e6[k], e12[k])
        assert e12[k] < e6[k] / 2, (name, k, e6[k], e12[k])


def test_constant_fields_have_zero_laplacians():
    g, o = _setup(6)
    X = np.zeros((g.Nh, 4, 16, g.Nv))
    X[:, 0] = 3.7
    L = o.laplacians(X)
    assert np.abs(L).max() < 1e-12 * 3.7 / g.R ** 2

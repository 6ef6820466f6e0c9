"""Oracle geometry: equiangular cubed sphere, GLL Nq=4, deep-atmosphere metrics.

TEST INFRASTRUCTURE ONLY. This module is part of the CPU oracle; only the test
suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
use it. The product library computes its own geometry in C++
(``csrc/geometry.cpp``); the tests compare the two.

What it restates (the reference delegates all of this to ClimaCore 0.15.1,
which is not vendored, so it is restated here from the mathematics):

* ``SphereGrid`` (src/simulation/grids.jl:42-89): EquiangularCubedSphere of
  ``h_elem`` x ``h_elem`` elements per panel, ``nh_poly = 3`` (Nq = 4 GLL
  nodes), deep-atmosphere global geometry (horizontal metric scaled by
  ``(R + z) / R``), radius default 6.371229e6 m (grids.jl:49).
* ``get_stretching`` (grids.jl:356): uniform levels or hyperbolic-tangent
  stretching with a target bottom layer thickness ``dz_bottom``.
* Vertical local geometry: centre Jacobian = layer thickness; interior face
  Jacobian = distance between adjacent centres; boundary faces use the
  adjacent layer thickness.
* DSS groups (src/prognostic_equations/constrain_state.jl:59-64 calls
  ``Spaces.weighted_dss!``): every set of collocated element nodes, found here
  by matching node positions on the unit sphere (the product finds them from
  the integer lattice of the cube instead).

The covariant basis ``e_i = dX/dxi^i`` is the exact derivative of the
equiangular map, evaluated analytically at each node.
"""
import math

import numpy as np

NQ = 4
NN = NQ * NQ

# Panel frames (n, t1, t2): outward normal and the two tangent directions along
# which the local coordinates (xi1, xi2) increase; t1 x t2 = n for every panel.
PANELS = np.array(
    [
        [[1, 0, 0], [0, 1, 0], [0, 0, 1]],
        [[0, 1, 0], [-1, 0, 0], [0, 0, 1]],
        [[-1, 0, 0], [0, -1, 0], [0, 0, 1]],
        [[0, -1, 0], [1, 0, 0], [0, 0, 1]],
        [[0, 0, 1], [0, 1, 0], [-1, 0, 0]],
        [[0, 0, -1], [0, 1, 0], [1, 0, 0]],
    ],
    dtype=np.float64,
)


def gll():
    """Nq=4 Gauss-Lobatto-Legendre nodes, weights and D[i][k] = l_k'(xi_i)."""
    s = 1.0 / math.sqrt(5.0)
    x = np.array([-1.0, -s, s, 1.0])
    w = np.array([1.0 / 6.0, 5.0 / 6.0, 5.0 / 6.0, 1.0 / 6.0])
    n = len(x)
    # barycentric weights
    lam = np.array([1.0 / np.prod([x[j] - x[m] for m in range(n) if m != j]) for j in range(n)])
    D = np.zeros((n, n))
    for i in range(n):
        for k in range(n):
            if i != k:
                D[i, k] = (lam[k] / lam[i]) / (x[i] - x[k])
        D[i, i] = -sum(D[i, k] for k in range(n) if k != i)
    return x, w, D


def vertical_faces(z_elem, z_max, stretch=False, dz_bottom=500.0):
    """Face heights z_f[0..z_elem] (uniform, or tanh-stretched with z_f[1] = dz_bottom)."""
    N = int(z_elem)
    if not stretch:
        return np.linspace(0.0, z_max, N + 1)
    target = dz_bottom / z_max

    def first(gam):
        return 1.0 + math.tanh(gam * (1.0 / N - 1.0)) / math.tanh(gam)

    lo, hi = 1e-8, 50.0  # first(gam) decreases monotonically in gam
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if first(mid) > target:
            lo = mid
        else:
            hi = mid
    gam = 0.5 * (lo + hi)
    zeta = np.arange(N + 1) / N
    zf = z_max * (1.0 + np.tanh(gam * (zeta - 1.0)) / math.tanh(gam))
    zf[0] = 0.0
    zf[-1] = z_max
    return zf


class OracleGeometry:
    """All geometric arrays the oracle needs, in FP64."""

    def __init__(self, h_elem, z_elem, z_max=30000.0, stretch=False, dz_bottom=500.0,
                 radius=6.371229e6, omega=7.2921159e-5):
        self.h = int(h_elem)
        self.Nh = 6 * self.h * self.h
        self.Nv = int(z_elem)
        self.R = float(radius)
        self.omega = float(omega)
        xg, wg, D = gll()
        self.xg, self.wg, self.D = xg, wg, D
        self.W = np.array([wg[n % NQ] * wg[n // NQ] for n in range(NN)])
        self._horizontal()
        self._dss_groups()
        zf = vertical_faces(z_elem, z_max, stretch, dz_bottom)
        self.zf = zf
        self.zc = 0.5 * (zf[1:] + zf[:-1])
        self.dzc = zf[1:] - zf[:-1]
        dzf = np.empty(self.Nv + 1)
        dzf[1:-1] = self.zc[1:] - self.zc[:-1]
        dzf[0] = self.dzc[0]
        dzf[-1] = self.dzc[-1]
        self.dzf = dzf
        self.rc = (self.R + self.zc) / self.R
        self.rf = (self.R + zf) / self.R
        self.z_max = float(z_max)

    def _horizontal(self):
        h, R = self.h, self.R
        dal = (math.pi / 2.0) / h
        Nh = self.Nh
        xyz = np.zeros((Nh, NN, 3))
        e = np.zeros((Nh, NN, 2, 3))
        for p in range(6):
            n, t1, t2 = PANELS[p]
            for ey in range(h):
                for ex in range(h):
                    el = (p * h + ey) * h + ex
                    for jn in range(NQ):
                        for inn in range(NQ):
                            a = -math.pi / 4 + (ex + (self.xg[inn] + 1) / 2) * dal
                            b = -math.pi / 4 + (ey + (self.xg[jn] + 1) / 2) * dal
                            ta, tb = math.tan(a), math.tan(b)
                            P = n + ta * t1 + tb * t2
                            r2 = P @ P
                            rn = math.sqrt(r2)
                            X = P / rn
                            node = inn + NQ * jn
                            xyz[el, node] = X
                            # d(P/|P|)/dP applied to dP/dalpha = sec^2 * t1
                            for d, (tv, tt) in enumerate(((t1, ta), (t2, tb))):
                                dP = (1.0 + tt * tt) * tv
                                dX = dP / rn - P * (P @ dP) / (rn ** 3)
                                e[el, node, d] = R * (dal / 2.0) * dX
        self.xyz = xyz
        self.ecov = e  # covariant basis vectors at radius R (Cartesian)
        g11 = np.einsum("enk,enk->en", e[:, :, 0], e[:, :, 0])
        g12 = np.einsum("enk,enk->en", e[:, :, 0], e[:, :, 1])
        g22 = np.einsum("enk,enk->en", e[:, :, 1], e[:, :, 1])
        det = g11 * g22 - g12 * g12
        self.Jh = np.sqrt(det)
        self.gdn = np.stack([g11, g12, g22], axis=-1)
        self.gup = np.stack([g22 / det, -g12 / det, g11 / det], axis=-1)
        gu = self.gup
        self.econ = np.stack(
            [gu[..., 0:1] * e[:, :, 0] + gu[..., 1:2] * e[:, :, 1],
             gu[..., 1:2] * e[:, :, 0] + gu[..., 2:3] * e[:, :, 1]], axis=2)
        zc = xyz[..., 2]
        self.sinlat = zc
        self.coslat = np.sqrt(np.maximum(xyz[..., 0] ** 2 + xyz[..., 1] ** 2, 0.0))
        self.lat = np.arctan2(zc, self.coslat)
        self.lon = np.arctan2(xyz[..., 1], xyz[..., 0])
        # local north unit vector (east/north basis); at a pole its choice is arbitrary
        # but the Coriolis horizontal part 2*Omega*cos(lat)*north vanishes there
        north = np.stack([-zc * np.cos(self.lon), -zc * np.sin(self.lon), self.coslat], axis=-1)
        fcov = 2.0 * self.omega * self.coslat[..., None] * np.stack(
            [np.einsum("enk,enk->en", e[:, :, d], north) for d in range(2)], axis=-1)
        self.fh0 = np.stack([gu[..., 0] * fcov[..., 0] + gu[..., 1] * fcov[..., 1],
                             gu[..., 1] * fcov[..., 0] + gu[..., 2] * fcov[..., 1]], axis=-1)

    def _dss_groups(self):
        key = np.round(self.xyz.reshape(-1, 3) * 1e9).astype(np.int64)
        _, inv, counts = np.unique(key, axis=0, return_inverse=True, return_counts=True)
        inv = inv.reshape(-1)
        order = np.argsort(inv, kind="stable")
        groups = {}
        for idx in order:
            g = inv[idx]
            if counts[g] > 1:
                groups.setdefault(g, []).append(int(idx))
        glist = sorted(groups.values(), key=lambda c: c[0])
        off = [0]
        cop = []
        wts = []
        Jh = self.Jh.reshape(-1)
        for c in glist:
            c = sorted(c)
            cop.extend(c)
            s = sum(Jh[i] for i in c)
            wts.extend(Jh[i] / s for i in c)
            off.append(len(cop))
        self.dss_off = np.array(off, dtype=np.int32)
        self.dss_copy = np.array(cop, dtype=np.int32)
        self.dss_w = np.array(wts, dtype=np.float64)
        self.unique_nodes = int(len(counts))

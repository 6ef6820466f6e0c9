"""Oracle restatement of the surface-elevation profiles and terrain-following mesh warps.

TEST INFRASTRUCTURE ONLY. This module is part of the CPU oracle; only the test suite may
use it. It is the first piece of the topography extension (the GPU metric terms and
kernels are not built yet): the analytic surface elevations the reference's idealised and
spherical cases use, and the warps that turn flat level heights into terrain-following ones.

What it restates:

* ``topography_function`` of the analytic profiles (src/topography/topography.jl):
  ``CosineTopography`` in 2D and 3D (:83-95), ``AgnesiTopography`` (:118-125),
  ``ScharTopography`` (:151-159), ``DCMIP200Topography`` (:186-205, the 2 km circular mountain
  on the equator at 270 degrees longitude) and ``Hughes2023Topography`` (:224-253, two 2 km
  ridges at 45 N).  Angles are in degrees as in the reference.
* ``LinearWarp`` and ``SLEVEWarp`` (topography.jl:272-307).  The warps themselves are
  ClimaCore's hypsography adaptions (ClimaCore 0.15.1, not vendored), restated from their
  published formulations: linear decay of the terrain with height (Gal-Chen and Somerville,
  1975), z = xi + z_s (1 - xi / z_top); and the one-scale SLEVE coordinate of Schaer et al.
  (2002) as the reference documents it, z = xi + z_s sinh((eta_h - eta) / (s eta_h)) / sinh(1 / s)
  for eta = xi / z_top <= eta_h, else z = xi.  Building the grid requires s z_top to exceed
  the highest surface (topography.jl:295-297).
"""
import math
from dataclasses import dataclass

import numpy as np


def cospi(x):
    return np.cos(np.pi * np.asarray(x, dtype=np.float64))


# ---------------------------------------------------------------- analytic profiles
@dataclass(frozen=True)
class CosineTopography:
    """h_max cos(2 pi x / lambda) (2D) or h_max cos(2 pi x / lambda) cos(2 pi y / lambda) (3D)."""
    dim: int = 2
    h_max: float = 25.0
    lam: float = 25e3

    def __call__(self, x, y=0.0):
        ly = math.inf if self.dim == 2 else self.lam
        return self.h_max * cospi(2 * np.asarray(x) / self.lam) * cospi(2 * np.asarray(y) / ly)


@dataclass(frozen=True)
class AgnesiTopography:
    """Witch of Agnesi: h_max / (1 + ((x - x_c) / a)^2)."""
    h_max: float = 25.0
    x_center: float = 50e3
    a: float = 5e3

    def __call__(self, x):
        return self.h_max / (1 + ((np.asarray(x, dtype=np.float64) - self.x_center) / self.a) ** 2)


@dataclass(frozen=True)
class ScharTopography:
    """h_max exp(-((x - x_c) / a)^2) cos^2(pi (x - x_c) / lambda)."""
    h_max: float = 25.0
    x_center: float = 50e3
    lam: float = 4e3
    a: float = 5e3

    def __call__(self, x):
        d = np.asarray(x, dtype=np.float64) - self.x_center
        return self.h_max * np.exp(-d ** 2 / self.a ** 2) * cospi(d / self.lam) ** 2


def dcmip200(lat, lon):
    """DCMIP-2-0-0 mountain (degrees): a cosine bell of 2 km over a great-circle radius of
    3 pi / 4 around (0 N, 270 E), modulated by cosine ridges of half-width pi / 16."""
    lat = np.asarray(lat, dtype=np.float64)
    lon = np.asarray(lon, dtype=np.float64)
    lat_m, lon_m = 0.0, 270.0
    d2r = np.pi / 180.0
    r = np.arccos(np.sin(lat_m * d2r) * np.sin(lat * d2r)
                  + np.cos(lat_m * d2r) * np.cos(lat * d2r) * np.cos((lon - lon_m) * d2r))
    R_m, zeta_m, h0 = 3 * np.pi / 4, np.pi / 16, 2000.0
    return np.where(r < R_m, h0 / 2 * (1 + cospi(r / R_m)) * cospi(r / zeta_m) ** 2, 0.0)


def hughes2023(lat, lon):
    """Hughes and Jablonowski (2023) ridges (degrees): super-Gaussian in latitude, Gaussian
    in longitude, 2 km peaks at (45 N, 72 E) and (45 N, 140 E), a tenth of the peak at 20
    degrees of latitude and 3.5 degrees of longitude from it."""
    lat = np.asarray(lat, dtype=np.float64)
    lon = np.asarray(lon, dtype=np.float64)
    h0, lat1, lat2, lon1, lon2, lon_w, lat_w = 2e3, 45.0, 45.0, 72.0, 140.0, 7.0, 40.0
    d = lat_w / 2 * (-math.log(0.1)) ** (-1 / 6)
    c = lon_w / 2 * (-math.log(0.1)) ** (-1 / 2)
    return h0 * (np.exp(-(((lat - lat1) / d) ** 6 + ((lon - lon1) / c) ** 2))
                 + np.exp(-(((lat - lat2) / d) ** 6 + ((lon - lon2) / c) ** 2)))


# ---------------------------------------------------------------- mesh warps
@dataclass(frozen=True)
class LinearWarp:
    """Terrain influence decaying linearly to zero at the model top."""

    def __call__(self, xi, z_surface, z_top):
        xi = np.asarray(xi, dtype=np.float64)
        return xi + np.asarray(z_surface, dtype=np.float64) * (1 - xi / z_top)


@dataclass(frozen=True)
class SLEVEWarp:
    """Smooth level vertical coordinate: the terrain decays like
    sinh((eta_h - eta) / (s eta_h)) / sinh(1 / s), flat above eta_h = eta."""
    eta: float = 0.7
    s: float = 10.0

    def __call__(self, xi, z_surface, z_top):
        xi = np.asarray(xi, dtype=np.float64)
        zs = np.asarray(z_surface, dtype=np.float64)
        if np.any(self.s * z_top <= zs):
            raise ValueError("SLEVEWarp: s * z_top must exceed the surface elevation")
        eta = xi / z_top
        decay = np.sinh((self.eta - eta) / (self.s * self.eta)) / math.sinh(1 / self.s)
        return np.where(eta <= self.eta, xi + zs * decay, xi)


def warped_faces(zf_flat, z_surface, warp):
    """Face heights of terrain-following columns: zf[..., k] for flat face heights zf_flat
    (0 .. z_top) over surfaces z_surface (any shape), with the given warp."""
    zf_flat = np.asarray(zf_flat, dtype=np.float64)
    z_top = float(zf_flat[-1])
    zs = np.asarray(z_surface, dtype=np.float64)[..., None]
    return warp(zf_flat, zs, z_top)


# ---------------------------------------------------------------- terrain-following geometry
def warped_geometry(g, z_surface, warp):
    """Local geometry of the terrain-following grid over the oracle's cubed sphere ``g``
    (an OracleGeometry), restated from the mathematics (ClimaCore computes it for the
    reference and is not vendored): the position is X = (R + z) x_hat with
    z = warp(zeta, z_s) on the flat faces zeta, so the covariant basis is

        E_i = (R + z) / R e_i + (dz/dxi^i) x_hat   (i = 1, 2; e_i the surface basis),
        E_3 = dz x_hat                              (dz: the cell's warped thickness; at a face
                                                     the distance between the centres around it),

    with dz/dxi^i the spectral (GLL) derivative of the warped heights of each level in its
    element and the centre heights the midpoints of the warped faces.  Returns a dict of numpy
    arrays: ``zf`` [Nh, 16, Nf] and ``zc`` [Nh, 16, Nv] heights, ``Jc``/``Jf`` the Jacobians
    E_3 . (E_1 x E_2), and ``gup_c``/``gup_f`` [..., 3, 3] the contravariant metric (the inverse
    of E_i . E_j), with ``Ec``/``Ef`` [..., 3, 3] the covariant basis (row i = E_i)."""
    R = g.R
    zs = np.asarray(z_surface, dtype=np.float64)
    zf = warped_faces(g.zf, zs, warp)                                # [Nh, 16, Nf]
    zc = 0.5 * (zf[..., 1:] + zf[..., :-1])
    dzc = zf[..., 1:] - zf[..., :-1]
    dzf = np.empty_like(zf)
    dzf[..., 1:-1] = zc[..., 1:] - zc[..., :-1]
    dzf[..., 0], dzf[..., -1] = dzc[..., 0], dzc[..., -1]
    D = g.D
    NQ = D.shape[0]

    def dxi(z):
        # [Nh, 16, L] -> d/dxi^1 and d/dxi^2 at every node (node n = i + NQ j)
        zz = z.reshape(z.shape[0], NQ, NQ, -1)                      # [e, j, i, L]
        d1 = np.einsum("ik,ejkl->ejil", D, zz).reshape(z.shape)
        d2 = np.einsum("jk,ekil->ejil", D, zz).reshape(z.shape)
        return d1, d2

    def basis(z, dz):
        r = (R + z) / R
        d1, d2 = dxi(z)
        xh = g.xyz[:, :, None, :]
        E = np.empty(z.shape + (3, 3))
        E[..., 0, :] = r[..., None] * g.ecov[:, :, None, 0, :] + d1[..., None] * xh
        E[..., 1, :] = r[..., None] * g.ecov[:, :, None, 1, :] + d2[..., None] * xh
        E[..., 2, :] = dz[..., None] * xh
        gdn = np.einsum("...ik,...jk->...ij", E, E)
        J = np.einsum("...k,...k->...", E[..., 2, :], np.cross(E[..., 0, :], E[..., 1, :]))
        # the metric's diagonal spans ~1e4 (dz^2) to ~1e12 (the horizontal scale squared):
        # invert the equilibrated matrix D g D (D = diag(g_ii)^-1/2) and scale back
        d = 1.0 / np.sqrt(np.einsum("...ii->...i", gdn))
        gup = d[..., :, None] * np.linalg.inv(d[..., :, None] * gdn * d[..., None, :]) * d[..., None, :]
        return E, J, gup

    Ec, Jc, gup_c = basis(zc, dzc)
    Ef, Jf, gup_f = basis(zf, dzf)
    return dict(zf=zf, zc=zc, Jc=Jc, Jf=Jf, gup_c=gup_c, gup_f=gup_f, Ec=Ec, Ef=Ef)


def winterp_faces(w, x):
    """rho J-weighted centre-to-face interpolation (the reference's ᶠwinterp, a
    WeightedInterpolateC2F with Extrapolate boundaries, src/utils/abbreviations.jl:184-187):
    interior face k+1/2 gets (w_k x_k + w_{k+1} x_{k+1}) / (w_k + w_{k+1}); the bottom and top
    faces take the adjacent centre's value.  w, x: [..., Nv] -> [..., Nv + 1]."""
    w = np.asarray(w, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    out = np.empty(x.shape[:-1] + (x.shape[-1] + 1,))
    out[..., 1:-1] = (w[..., :-1] * x[..., :-1] + w[..., 1:] * x[..., 1:]) / (w[..., :-1] + w[..., 1:])
    out[..., 0], out[..., -1] = x[..., 0], x[..., -1]
    return out


def impenetrable_u3(G, rho, u1, u2):
    """u_3 on the bottom and top faces that makes u^3 vanish there over terrain
    (set_velocity_at_surface!, set_velocity_at_top!; src/cache/precomputed_quantities.jl:473-547):
    u_h^3 = CT3(u_h) = g^31 u_1 + g^32 u_2 at the centres, brought to the faces by the rho J
    weighted interpolation ``winterp_faces``, and u_3 = -u_h^3 / g^33 with the face's metric.
    Only the two boundary faces are produced: that is where the filter acts, and there the
    interpolation extrapolates the adjacent centre, so the rho J weights do not enter (an
    interior face would need them).
    ``G`` is a warped_geometry; rho, u1, u2 are [Nh, 16, Nv] (u_h covariant).
    Returns [Nh, 16, 2]: the bottom and top faces."""
    gc, gf = G["gup_c"], G["gup_f"]
    uh3 = gc[..., 2, 0] * u1 + gc[..., 2, 1] * u2                 # [Nh, 16, Nv]
    uh3f = winterp_faces(np.asarray(rho) * G["Jc"], uh3)          # [Nh, 16, Nv + 1]
    return np.stack([-uh3f[..., 0] / gf[..., 0, 2, 2], -uh3f[..., -1] / gf[..., -1, 2, 2]], axis=-1)


def oracle_terrain(g, z_surface, warp, omega=None):
    """The per-point arrays the C++ oracle takes over terrain (OracleGeom's t_* fields), from
    ``warped_geometry``: heights, Jacobians, the contravariant metric of centres and faces and
    the covariant metric of the centres as (11, 12, 22, 13, 23, 33), the Coriolis components
    f^i = grad(xi^i) . 2 Omega z_hat (f^3 at the centres, f^1 and f^2 at the faces:
    compute_coriolis, src/cache/cache.jl:318-343, deep branch), and the centres' covariant and
    contravariant bases (rows E_i and E^i = g^ij E_j) for the DSS of covariant 3-vectors."""
    G = warped_geometry(g, z_surface, warp)
    om = g.omega if omega is None else omega
    Om = np.array([0.0, 0.0, 2.0 * om])
    pick = [(0, 0), (0, 1), (1, 1), (0, 2), (1, 2), (2, 2)]

    def six(M):
        return np.stack([M[..., i, j] for i, j in pick], axis=-1)

    Ec, Ef = G["Ec"], G["Ef"]
    gdn_c = np.einsum("...ik,...jk->...ij", Ec, Ec)
    Ecn = np.einsum("...ij,...jk->...ik", G["gup_c"], Ec)
    Efn = np.einsum("...ij,...jk->...ik", G["gup_f"], Ef)
    return dict(
        zc=G["zc"], zf=G["zf"], Jc=G["Jc"], Jf=G["Jf"],
        guc=six(G["gup_c"]), guf=six(G["gup_f"]), gdc=six(gdn_c),
        f3c=Ecn[..., 2, :] @ Om, f12f=np.stack([Efn[..., 0, :] @ Om, Efn[..., 1, :] @ Om], axis=-1),
        Ecc=Ec.reshape(Ec.shape[:-2] + (9,)), Ecn=Ecn.reshape(Ecn.shape[:-2] + (9,)))


def smooth_surface(xyz, h0=2000.0, lat0=20.0, lon0=30.0, width=40.0):
    """A smooth test surface (m) over unit-sphere node positions ``xyz`` [..., 3]: a Gaussian
    hill of height h0 and angular half-width ``width`` degrees centred at (lat0, lon0)."""
    la, lo = math.radians(lat0), math.radians(lon0)
    X0 = np.array([math.cos(la) * math.cos(lo), math.cos(la) * math.sin(lo), math.sin(la)])
    d = np.arccos(np.clip(np.asarray(xyz) @ X0, -1.0, 1.0))
    return h0 * np.exp(-(d / math.radians(width)) ** 2)


def dcmip200_nodes(xyz):
    """The DCMIP-2-0-0 mountain at unit-sphere node positions ``xyz`` [..., 3]."""
    xyz = np.asarray(xyz, dtype=np.float64)
    lat = np.degrees(np.arctan2(xyz[..., 2], np.hypot(xyz[..., 0], xyz[..., 1])))
    lon = np.degrees(np.arctan2(xyz[..., 1], xyz[..., 0])) % 360.0
    return dcmip200(lat, lon)

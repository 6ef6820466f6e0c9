"""The caller's element layout (gb_config.elem_map / elem_orient) on the host.

ClimaCore numbers the elements of a SpectralElementSpace2D along a space-filling
curve (``Topology2D(context, mesh, spacefillingcurve(mesh))``,
src/simulation/grids.jl:74-75) and gives each element its own local (xi^1, xi^2)
frame.  The library builds its geometry tables and DSS plan directly in such a
layout, so a state in the caller's layout is passed without any remapping;
this module holds the same node and covariant-component map for host arrays
(tests, conversions of files written in another layout).

Caller element e is library element ``elem_map[e]`` with its frame turned by
``elem_orient[e]`` quarter turns: the caller's node (i, j) is the library's
node ``(i, j)``, ``(3 - j, i)``, ``(3 - i, 3 - j)`` or ``(j, 3 - i)`` for
orientation 0, 1, 2, 3, and the caller's covariant components are those on
its own basis: (u_1, u_2), (u_2, -u_1), (-u_1, -u_2), (-u_2, u_1).
"""
import numpy as np

NQ = 4


def library_node(o, i, j):
    """The library's (i, j) of the caller's node (i, j) in a frame turned by o quarter turns."""
    return [(i, j), (3 - j, i), (3 - i, 3 - j), (j, 3 - i)][o & 3]


# NODE_OF[o][n]: the library node of the caller's node n = i + 4 j
NODE_OF = np.array([[library_node(o, n % NQ, n // NQ)[0] + NQ * library_node(o, n % NQ, n // NQ)[1]
                     for n in range(NQ * NQ)] for o in range(4)], dtype=np.int64)
# the caller's (u_1, u_2) from the library's: u'_k = sum_m R[o][k][m] u_m
ROT = np.array([[[1, 0], [0, 1]], [[0, 1], [-1, 0]], [[-1, 0], [0, -1]], [[0, -1], [1, 0]]], dtype=np.float64)


def to_caller(Yc, Yf, elem_map, elem_orient):
    """A state in the library's layout (c [Nh, 4, 16, Nv], f [Nh, 16, Nv + 1]) in the caller's."""
    emap = np.asarray(elem_map, np.int64)
    eori = np.asarray(elem_orient, np.int64) & 3
    nodes = NODE_OF[eori]                                     # [Nh, 16]
    c = np.asarray(Yc)[emap[:, None], :, nodes, :]            # [Nh, 16, 4, Nv]
    c = np.ascontiguousarray(c.transpose(0, 2, 1, 3))
    u = c[:, 1:3].copy()
    R = ROT[eori].astype(c.dtype)                             # [Nh, 2, 2]
    c[:, 1] = R[:, 0, 0, None, None] * u[:, 0] + R[:, 0, 1, None, None] * u[:, 1]
    c[:, 2] = R[:, 1, 0, None, None] * u[:, 0] + R[:, 1, 1, None, None] * u[:, 1]
    f = np.ascontiguousarray(np.asarray(Yf)[emap[:, None], nodes, :])
    return c, f


def from_caller(Xc, Xf, elem_map, elem_orient):
    """The inverse of to_caller: a state in the caller's layout in the library's."""
    emap = np.asarray(elem_map, np.int64)
    eori = np.asarray(elem_orient, np.int64) & 3
    nodes = NODE_OF[eori]
    Xc = np.asarray(Xc)
    R = ROT[eori].astype(Xc.dtype)
    u1 = R[:, 0, 0, None, None] * Xc[:, 1] + R[:, 1, 0, None, None] * Xc[:, 2]   # R is orthogonal: R^T
    u2 = R[:, 0, 1, None, None] * Xc[:, 1] + R[:, 1, 1, None, None] * Xc[:, 2]
    Z = np.stack([Xc[:, 0], u1, u2, Xc[:, 3]], axis=1)        # [Nh, 4, 16, Nv], caller nodes
    c = np.empty_like(Z)
    f = np.empty_like(np.asarray(Xf))
    c[emap[:, None], :, nodes, :] = Z.transpose(0, 2, 1, 3)
    f[emap[:, None], nodes, :] = np.asarray(Xf)
    return c, f


def random_layout(h_elem, seed=0, rotate=True):
    """A random element numbering (and, with rotate, random frames) of the cubed sphere."""
    rng = np.random.default_rng(seed)
    Nh = 6 * h_elem * h_elem
    emap = rng.permutation(Nh).astype(np.int32)
    eori = (rng.integers(0, 4, size=Nh) if rotate else np.zeros(Nh)).astype(np.int32)
    return emap, eori

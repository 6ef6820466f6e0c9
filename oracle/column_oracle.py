"""Oracle of the batched standalone-column Newton solve.

TEST INFRASTRUCTURE ONLY (imported by ``tests/`` and ``bench.py``'s CPU
baseline leg).  Each height group of the batch becomes one CPU ``Oracle``
instance whose "elements" are 16-column packs of a flat column geometry
(J_h = 1, g^ij = identity, no DSS groups, radius 1e30 so that r = 1 exactly),
and the Newton iteration is the one ``dycore_oracle.cpp``'s step performs
per implicit stage, repeated ``iters`` times: filter U, T = implicit_tendency(U),
R = U^ + dtgamma T - U, update_jacobian(U), dU = ldiv(R), U -= dU
(ClimaTimeSteppers' NewtonsMethod, src/simulation/integrator.jl:63-120;
the column operators follow implicit_tendency.jl:185-298 and
manual_sparse_jacobian.jl:713-870).  The final u_3 is filtered.
"""
from types import SimpleNamespace

import numpy as np

import oracle as O


def _geometry(nv, npack, zf):
    H = npack * 16
    xg = np.array([-1.0, -1.0 / np.sqrt(5.0), 1.0 / np.sqrt(5.0), 1.0])
    D = np.zeros((4, 4))  # the SE operators are not used by the column functions
    return SimpleNamespace(
        Nh=npack, Nv=nv, W=np.ones(16), D=D, Jh=np.ones(H),
        gup=np.tile([1.0, 0.0, 1.0], H), gdn=np.tile([1.0, 0.0, 1.0], H),
        sinlat=np.zeros(H), fh0=np.zeros(2 * H), ecov=np.tile([1.0, 0, 0, 0, 1.0, 0], H),
        econ=np.tile([1.0, 0, 0, 0, 1.0, 0], H), zf=np.asarray(zf, dtype=np.float64),
        dss_off=np.zeros(1, dtype=np.int32), dss_copy=np.zeros(1, dtype=np.int32), dss_w=np.zeros(1), xg=xg)


def newton(cfg, z_elem, Uc, Uf, Hc, Hf, dtgamma, iters, column_faces, dtype=np.float64):
    """Newton on every column: returns (Uc, Uf, rnorm[iters, 3]) in the batch layout.

    ``column_faces(cfg, z)`` gives a column's face heights."""
    z_elem = np.asarray(z_elem, dtype=np.int64)
    off = np.concatenate([[0], np.cumsum(z_elem)[:-1]])
    Uc = np.array(Uc, dtype=dtype)
    Uf = np.array(Uf, dtype=dtype)
    Hc = np.asarray(Hc, dtype=dtype)
    Hf = np.asarray(Hf, dtype=dtype)
    rn = np.zeros((iters, 3))
    params = cfg.oracle_params()
    params.update(radius=1e30, upwinding=0)
    for z in np.unique(z_elem):
        cols = np.nonzero(z_elem == z)[0]
        npack = (len(cols) + 15) // 16
        o = O.Oracle(_geometry(int(z), npack, column_faces(cfg, int(z))), params, dtype)
        slots = np.concatenate([cols, np.repeat(cols[:1], npack * 16 - len(cols))])  # pad with copies

        def pack(c, f):
            Pc = np.empty((npack * 16, 4, z), dtype)
            Pf = np.empty((npack * 16, z + 1), dtype)
            for s, k in enumerate(slots):
                Pc[s] = c[:, off[k]: off[k] + z]
                Pf[s] = f[off[k] + k: off[k] + k + z + 1]
            return (np.ascontiguousarray(Pc.reshape(npack, 16, 4, z).transpose(0, 2, 1, 3)),
                    np.ascontiguousarray(Pf.reshape(npack, 16, z + 1)))

        Pc, Pf = pack(Uc, Uf)
        Qc, Qf = pack(Hc, Hf)
        valid = np.zeros(npack * 16, bool)
        valid[: len(cols)] = True
        for it in range(iters):
            o.set_precomputed(Pc, Pf)
            Tc, Tf = o.implicit_tendency(Pc, Pf)
            Rc = Qc + dtgamma * Tc - Pc
            Rf = Qf + dtgamma * Tf - Pf
            mc = valid.reshape(npack, 16)
            rn[it, 0] += float(np.sum(Rc[:, 0][mc] ** 2))
            rn[it, 1] += float(np.sum(Rc[:, 3][mc] ** 2))
            rn[it, 2] += float(np.sum(Rf[mc] ** 2))
            o.update_jacobian(Pc, Pf, dtgamma)
            Xc, Xf = o.ldiv(Rc, Rf)
            Pc = np.ascontiguousarray(Pc - Xc)
            Pf = np.ascontiguousarray(Pf - Xf)
        o.set_precomputed(Pc, Pf)
        Pc = Pc.transpose(0, 2, 1, 3).reshape(npack * 16, 4, z)
        Pf = Pf.reshape(npack * 16, z + 1)
        for s, k in enumerate(cols):
            Uc[:, off[k]: off[k] + z] = Pc[s]
            Uf[off[k] + k: off[k] + k + z + 1] = Pf[s]
    return Uc, Uf, rn

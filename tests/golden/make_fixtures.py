"""Writes the oracle regression fixtures of tests/golden/ (run from the repository root:
``python tests/golden/make_fixtures.py``).

The reference holds no golden vectors for the dry-dycore arithmetic (its hot-path tests are
placeholders), and the reference itself (Julia) cannot run here, so these fixtures are the
oracle's own outputs on a small stretched grid: they pin the oracle against unintended change,
not against the reference.  Contents of ``oracle_h2z4.npz`` (FP64, h_elem 2, z_elem 4,
tanh-stretched to 30 km, the seeded perturbed state of tests/helpers.py):
``Yc``, ``Yf`` the input; ``Trc``, ``Trf`` remaining_tendency; ``Tic``, ``Tif``
implicit_tendency; ``Sc``, ``Sf`` one ARS343 step (dt 300 s); ``sums`` the global mass and
energy integrals of the input.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
ROOT = os.path.dirname(TESTS)
sys.path[:0] = [os.path.join(ROOT, "climaatmos.jl_gb300"), os.path.join(ROOT, "oracle"), TESTS]

import numpy as np  # noqa: E402

from helpers import make_oracle, perturbed_state, small_config  # noqa: E402

FIXTURE = os.path.join(HERE, "oracle_h2z4.npz")


def compute():
    cfg = small_config(h_elem=2, z_elem=4)
    o = make_oracle(cfg, np.float64)
    Yc, Yf = perturbed_state(cfg)
    Trc, Trf = o.remaining_tendency(Yc.copy(), Yf.copy())
    Tic, Tif = o.implicit_tendency(Yc.copy(), Yf.copy())
    Sc, Sf = Yc.copy(), Yf.copy()
    o.step(Sc, Sf, cfg.dt, 1)
    return dict(Yc=Yc, Yf=Yf, Trc=Trc, Trf=Trf, Tic=Tic, Tif=Tif, Sc=Sc, Sf=Sf, sums=o.global_sums(Yc))


if __name__ == "__main__":
    np.savez_compressed(FIXTURE, **compute())
    print("wrote", FIXTURE)

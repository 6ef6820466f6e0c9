"""The oracle against its committed regression fixtures (tests/golden/oracle_h2z4.npz, made by
tests/golden/make_fixtures.py): the explicit and implicit tendencies, one ARS343 step and the
global sums of a small stretched grid in FP64, to 1e-12 of each field's largest magnitude
(libm differences between machines stay far below that)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_fixtures as MF  # noqa: E402


@pytest.fixture(scope="module")
def pair():
    return dict(np.load(MF.FIXTURE)), MF.compute()


@pytest.mark.parametrize("key", ["Yc", "Yf", "Trc", "Trf", "Tic", "Tif", "Sc", "Sf", "sums"])
def test_oracle_matches_fixture(pair, key):
    ref, now = pair
    a, b = np.asarray(now[key]), ref[key]
    assert a.shape == b.shape and a.dtype == b.dtype
    scale = max(np.abs(b).max(), 1e-300)
    assert np.abs(a - b).max() <= 1e-12 * scale, key

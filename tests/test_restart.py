"""Checkpoint / restart of the prognostic state (the reference's save_state_to_disk_func,
src/callbacks/callbacks.jl:297-321, and get_state_restart, src/simulation/restart.jl:22-42):
file naming from the simulation time, the state and the time round-trip exactly, a different
model configuration warns, a different grid is refused; on the GPU a run restarted from a
checkpoint continues bitwise like the uninterrupted run."""
import os
import warnings

import numpy as np
import pytest

from gbdycore import restart as R
from helpers import perturbed_state, small_config


def test_file_name_from_time():
    assert R.restart_file_name(0.0) == "day0.0.npz"
    assert R.restart_file_name(86400.0 * 2 + 3661.5) == "day2.3661.npz"


def test_time_from_filename_known_answers():
    # the reference's known answers (test/utilities.jl:103-108)
    assert R.time_from_filename("day0.0.hdf5") == 0.0
    assert R.time_from_filename("day1.0.hdf5") == 86400.0
    assert R.time_from_filename("day1.3600.hdf5") == 86400.0 + 3600.0
    assert R.time_from_filename("day10.43200.hdf5") == 10 * 86400.0 + 43200.0
    for t in (0.0, 59.0, 86399.0, 86400.0, 90061.0, 10 ** 6):
        assert R.time_from_filename(R.restart_file_name(t)) == t


def test_sort_files_by_time(tmp_path):
    # as test/utilities.jl:92-101: names of random times, lexically sorted, back in time order
    rng = np.random.default_rng(0)
    t = rng.integers(1, 10 ** 6, 100)
    names = sorted(R.restart_file_name(float(x)) for x in t)
    assert R.sort_files_by_time(names) == [R.restart_file_name(float(x)) for x in np.sort(t)]
    assert R.latest_restart_file(str(tmp_path / "none")) is None
    for x in (86400.0 * 2, 86400.0 * 10, 3600.0):
        (tmp_path / R.restart_file_name(x)).write_bytes(b"")
    assert os.path.basename(R.latest_restart_file(str(tmp_path))) == "day10.0.npz"


def test_round_trip_and_checks(tmp_path):
    cfg = small_config(np.float32)
    Yc, Yf = perturbed_state(cfg, dtype=np.float32)
    path = R.save_state_to_disk(Yc, Yf, 7200.0, cfg, str(tmp_path))
    assert os.path.basename(path) == "day0.7200.npz"
    with warnings.catch_warnings():
        warnings.simplefilter("error")
        c, f, t = R.get_state_restart(path, cfg)
    assert t == 7200.0 and np.array_equal(c, Yc) and np.array_equal(f, Yf) and c.dtype == np.float32
    # another model (sponge on): loads with a warning
    with pytest.warns(UserWarning, match="different AtmosModel"):
        R.get_state_restart(path, cfg.with_(alpha_uh=1e-3, sponge_zd=15000.0))
    # the time step is not part of the model
    assert R.atmos_model_hash(cfg) == R.atmos_model_hash(cfg.with_(dt=10.0))
    # another grid or precision: refused
    with pytest.raises(ValueError):
        R.get_state_restart(path, cfg.with_(z_elem=cfg.z_elem + 1))
    with pytest.raises(ValueError):
        R.get_state_restart(path, cfg.with_(ft=np.float64))


@pytest.mark.gpu
def test_restarted_run_continues_bitwise(tmp_path):
    from gbdycore import simulation as sim
    cfg = small_config(np.float32)
    Yc, Yf = perturbed_state(cfg, dtype=np.float32)
    a = sim.AtmosSimulation(cfg, state=(Yc, Yf))
    a.step(2)
    path = a.save_state(str(tmp_path))
    a.step(3)
    b = sim.AtmosSimulation(cfg, detect_restart_file=True, output_dir=str(tmp_path))
    assert b.t == 2 * cfg.dt
    b.step(3)
    ac, af = a.Y.numpy()
    bc, bf = b.Y.numpy()
    assert np.array_equal(ac, bc) and np.array_equal(af, bf)

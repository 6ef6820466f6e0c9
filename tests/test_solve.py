"""solve_atmos's host logic (src/simulation/solve.jl:93-149): one untimed step, the timed
steps, the results record, and the crash path (the state written to the output directory,
ret_code "simulation_crashed"), on a fake simulation (CPU only; the GPU path that raises is
covered by test_gpu_parity.py::test_nonfinite_state_is_reported)."""
import pytest

from gbdycore import _native as N
from gbdycore import simulation as sim


class FakeSim:
    def __init__(self, fail_check=False, fail_step=False, output_dir=None, t=0.0, t_end=None, every=None,
                 nan_every=None, nan_at=None):
        self.steps, self.saved, self.scans, self.dt, self.Y = [], [], [], 120.0, object()
        self.t, self.t_end, self.dt_save_state_to_disk = t, t_end, every
        self.check_nan_every, self.nan_at = nan_every, nan_at
        self.fail_check, self.fail_step, self.output_dir = fail_check, fail_step, output_dir

    def step(self, n, use_graph=True):
        if self.fail_step:
            raise N.GBError(N.GB_ERR_TIMEOUT, "a device wait gave up")
        self.steps.append(n)
        self.t += n * self.dt

    def synchronize(self):
        pass

    def check_nans(self):
        self.scans.append(self.t)
        if self.nan_at is not None and self.t >= self.nan_at:
            raise N.GBError(N.GB_ERR_NONFINITE, "Found NaN in Y.c")

    def check(self):
        if self.fail_check:
            raise N.GBError(N.GB_ERR_NONFINITE, "non-finite Newton residual")

    def save_state(self, d):
        self.saved.append((d, self.t))


def test_success_record():
    s = FakeSim()
    r = sim.solve_atmos(s, 10)
    assert s.steps == [1, 10]
    assert r.ret_code == "success" and r.sol is s.Y and r.walltime >= 0
    assert r.seconds_per_step == pytest.approx(r.walltime / 10)
    if r.walltime > 0:
        assert r.sypd == pytest.approx(sim.simulated_years_per_day(120.0, r.seconds_per_step))


@pytest.mark.parametrize("kw", [dict(fail_check=True), dict(fail_step=True)])
def test_crash_saves_state_and_reports(kw, tmp_path):
    s = FakeSim(output_dir=str(tmp_path), **kw)
    with pytest.warns(UserWarning, match="simulation crashed"):
        r = sim.solve_atmos(s, 5)
    assert r.ret_code == "simulation_crashed" and r.sol is None and r.walltime is None
    assert [d for d, _ in s.saved] == [str(tmp_path)]


def test_crash_without_output_dir_saves_nothing():
    s = FakeSim(fail_check=True)
    with pytest.warns(UserWarning):
        r = sim.solve_atmos(s, 2)
    assert r.ret_code == "simulation_crashed" and s.saved == []


def test_runs_to_t_end():
    s = FakeSim(t=240.0, t_end=240.0 + 120.0 * 12)
    assert sim.solve_atmos(s).ret_code == "success"
    assert s.steps == [1, 11]  # the untimed step and the timed ones reach t_end
    with pytest.raises(ValueError):
        sim.solve_atmos(FakeSim())
    with pytest.raises(ValueError):
        sim.solve_atmos(FakeSim(t=100.0, t_end=100.0))


def test_checkpoints_on_schedule(tmp_path):
    # every 600 s = 5 steps of 120 s from t = 0: the warm-up step, then runs ending on t = 600, 1200
    s = FakeSim(output_dir=str(tmp_path), every=600.0)
    assert sim.solve_atmos(s, 12).ret_code == "success"
    assert s.steps == [1, 4, 5, 3]
    assert [t for _, t in s.saved] == [600.0, 1200.0]
    assert sim.solve_atmos(FakeSim(output_dir=str(tmp_path), every=float("inf")), 3).ret_code == "success"
    with pytest.raises(ValueError, match="output_dir"):
        sim.solve_atmos(FakeSim(every=600.0), 3)


def test_nan_scans_on_schedule_end_a_crashed_run(tmp_path):
    s = FakeSim(output_dir=str(tmp_path), nan_every=4, every=600.0)
    assert sim.solve_atmos(s, 11).ret_code == "success"
    assert s.steps == [1, 3, 1, 3, 2, 2]          # runs end on steps 1, 4, 5, 8, 10, 12
    # the initial state is scanned too (the callback's initialize), then every 4 steps
    assert s.scans == [0.0, 480.0, 960.0, 1440.0] and [t for _, t in s.saved] == [600.0, 1200.0]
    s = FakeSim(output_dir=str(tmp_path), nan_every=4, nan_at=900.0)
    with pytest.warns(UserWarning, match="Found NaN"):
        r = sim.solve_atmos(s, 11)
    assert r.ret_code == "simulation_crashed" and s.scans == [0.0, 480.0, 960.0]
    assert [t for _, t in s.saved] == [960.0]   # the crashed state


@pytest.mark.parametrize("n", [0, -1])
def test_nan_scan_off_for_zero_or_negative_period(n):
    # nan_checking_callback (get_callbacks.jl:316-330) builds no callback for check_nan_every <= 0
    s = FakeSim(nan_every=n)
    r = sim.solve_atmos(s, 7)
    assert r.ret_code == "success" and s.steps == [1, 7] and s.scans == []


def test_nan_scans_count_the_steps_of_a_restarted_run(tmp_path):
    # a run restarted at step 3 (t = 360 s) scans every 4 steps of its own (call_every_n_steps,
    # callback_helpers.jl:177-199, counts from the run's start); restart files stay on multiples
    # of dt_save_state_to_disk from t = 0
    s = FakeSim(output_dir=str(tmp_path), t=360.0, nan_every=4, every=600.0)
    assert sim.solve_atmos(s, 9).ret_code == "success"
    assert s.scans == [360.0, 360.0 + 480.0, 360.0 + 960.0]
    assert [t for _, t in s.saved] == [600.0, 1200.0]
    assert sum(s.steps) == 10

"""Host-side mirror of the reference's API for the dry dynamical-core path.

Names follow the reference (with Julia's ``!`` dropped):

* ``AtmosSimulation`` / ``solve_atmos``  (src/simulation/AtmosSimulations.jl:307,
  src/simulation/solve.jl:119; SYPD as in solve.jl:40-45),
* the ClimaODEFunction hooks wired in src/simulation/integrator.jl:189-225:
  ``remaining_tendency``, ``implicit_tendency``, ``update_jacobian``, ``ldiv``,
  ``correct_implicit_advection_tendency``, ``dss``,
  ``set_precomputed_quantities``,
* ``ars343_step_via_hooks``: the ClimaTimeSteppers IMEX ARK stage loop
  (ARS343, one Newton iteration, Jacobian refreshed every iteration)
  expressed through those hooks.

Every hook is one C-ABI call into libgbdycore.so on the GPU; state buffers
are torch CUDA tensors in the layout of include/gbdycore.h.  PyTorch only
provides device memory, streams and the elementwise stage algebra of the
hook-level loop.
"""
import ctypes
import math
import time

import numpy as np

from . import _native as N
from . import config as C
from . import restart as R
from . import setups as S


class Geometry:
    """Host copy of the library's grid (gb_geometry_export; no GPU needed)."""

    def __init__(self, cfg):
        L = N.load()
        c = N.make_config(cfg)
        nc, nf = ctypes.c_size_t(), ctypes.c_size_t()
        ng, ncp = ctypes.c_int(), ctypes.c_int()
        _check(None, L.gb_sizes(ctypes.byref(c), ctypes.byref(nc), ctypes.byref(nf), ctypes.byref(ng), ctypes.byref(ncp)))
        self.Nh, self.Nv = 6 * cfg.h_elem * cfg.h_elem, cfg.z_elem
        self.R = float(cfg.constants["radius"])
        H = self.Nh * 16
        self.xyz = np.zeros((self.Nh, 16, 3))
        self.ecov = np.zeros((self.Nh, 16, 2, 3))
        self.Jh = np.zeros((self.Nh, 16))
        self.gup = np.zeros((self.Nh, 16, 3))
        self.fh0 = np.zeros((self.Nh, 16, 2))
        self.zf = np.zeros(self.Nv + 1)
        self.dss_off = np.zeros(ng.value + 1, np.int32)
        self.dss_copy = np.zeros(ncp.value, np.int32)
        self.econ = np.zeros((self.Nh, 16, 2, 3))
        self.dss_w = np.zeros(ncp.value)
        g = N.GBGeometryHost()
        dp = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        ip = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        g.xyz, g.ecov, g.Jh, g.gup, g.fh0, g.zf = dp(self.xyz), dp(self.ecov), dp(self.Jh), dp(self.gup), dp(self.fh0), dp(self.zf)
        g.dss_off, g.dss_copy = ip(self.dss_off), ip(self.dss_copy)
        g.econ, g.dss_w = dp(self.econ), dp(self.dss_w)
        _check(None, L.gb_geometry_export(ctypes.byref(c), ctypes.byref(g)))
        self.zc = 0.5 * (self.zf[1:] + self.zf[:-1])
        self.n_center, self.n_face = nc.value, nf.value
        self.nfc = 5 if getattr(cfg, "moist", False) else 4   # centre components (5: with rho q_tot)
        assert H * self.nfc * self.Nv == self.n_center
        self.terrain = None
        if getattr(cfg, "z_surface", None) is not None:
            self.terrain = {"zc": terrain_centre_heights(cfg, self.zf)}


def warp_factor(cfg, zeta):
    """b(zeta) of the terrain-following levels z = zeta + z_s b(zeta) (gb_config.warp): linear
    decay to z_max, or the one-scale SLEVE decay (src/topography/topography.jl:272-307)."""
    zeta = np.asarray(zeta, dtype=np.float64)
    if getattr(cfg, "warp", "linear") == "linear":
        return 1.0 - zeta / cfg.z_max
    eta = zeta / cfg.z_max
    b = np.sinh((cfg.sleve_eta - eta) / (cfg.sleve_s * cfg.sleve_eta)) / np.sinh(1.0 / cfg.sleve_s)
    return np.where(eta <= cfg.sleve_eta, b, 0.0)


def terrain_centre_heights(cfg, zf):
    """Heights [Nh, 16, Nv] of the centres over cfg.z_surface [Nh, 16]: midway between the
    warped faces zeta_k + z_s b(zeta_k)."""
    zs = np.asarray(cfg.z_surface, dtype=np.float64).reshape(-1, 16)[..., None]
    zf = np.asarray(zf, dtype=np.float64)
    zw = zf + zs * warp_factor(cfg, zf)
    return 0.5 * (zw[..., 1:] + zw[..., :-1])


def _check(ctx, rc):
    if rc != N.GB_OK:
        msg = ""
        if ctx:
            buf = ctypes.create_string_buffer(512)
            N.load().gb_last_error(ctx, buf, 512)
            msg = buf.value.decode(errors="replace")
        raise N.GBError(rc, msg or "call failed")


class FieldVector:
    """Device state: ``c`` [Nh,4,16,Nv] (rho, u_1, u_2, rho e_tot; moist 0M: [Nh,5,16,Nv] with
    rho q_tot last), ``f`` [Nh,16,Nv+1] (u_3)."""

    def __init__(self, c, f):
        self.c, self.f = c, f

    @classmethod
    def from_numpy(cls, Yc, Yf, device="cuda"):
        import torch
        return cls(torch.from_numpy(np.ascontiguousarray(Yc)).to(device), torch.from_numpy(np.ascontiguousarray(Yf)).to(device))

    def similar(self):
        import torch
        return FieldVector(torch.zeros_like(self.c), torch.zeros_like(self.f))

    def copy(self):
        return FieldVector(self.c.clone(), self.f.clone())

    def numpy(self):
        return self.c.cpu().numpy(), self.f.cpu().numpy()

    def gb(self):
        assert self.c.is_contiguous() and self.f.is_contiguous()
        return N.GBFieldVec(self.c.data_ptr(), self.f.data_ptr())

    # elementwise algebra used by the hook-level stage loop
    def axpy_(self, a, X):
        self.c.add_(X.c, alpha=a)
        self.f.add_(X.f, alpha=a)
        return self

    def assign_(self, X):
        self.c.copy_(X.c)
        self.f.copy_(X.f)
        return self


class AtmosCache:
    """The library context (gb_ctx): geometry, Coriolis, DSS plan, scratch and
    the Jacobian blocks, i.e. the parts of the reference's cache ``p``
    (src/cache/cache.jl:165-305) that the hot path reads."""

    def __init__(self, cfg, stream=None):
        import torch
        self.cfg = cfg
        self.L = N.load()
        self._c = N.make_config(cfg)
        h = ctypes.c_void_p()
        _check(None, self.L.gb_ctx_create(ctypes.byref(self._c), ctypes.byref(h)))
        self.h = h
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        _check(self.h, self.L.gb_set_stream(self.h, ctypes.c_void_p(self.stream.cuda_stream)))
        self.dt = cfg.dt

    def close(self):
        if self.h:
            self.L.gb_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def call(self, name, *args):
        _check(self.h, getattr(self.L, name)(self.h, *args))

    def global_sums(self, Y):
        out = (ctypes.c_double * 2)()
        self.call("gb_global_sums", Y.gb(), out)
        return np.array(out[:])

    def conservation_sums(self, Y):
        """∫ρ, ∫ρe_tot and ∫ρq_tot (0 when dry) of the state, compensated FP64."""
        out = (ctypes.c_double * 3)()
        self.call("gb_conservation_sums", Y.gb(), out)
        return np.array(out[:])

    def newton_residual(self):
        out = (ctypes.c_double * 3)()
        self.call("gb_newton_residual", out)
        return np.array(out[:])


class Jacobian:
    """Handle of the Jacobian blocks, which live in the context (manual_sparse_jacobian.jl:603)."""

    def __init__(self, p):
        self.p = p


# ---------------------------------------------------------------- hooks
def set_precomputed_quantities(Y, p, t):
    p.call("gb_set_precomputed_quantities", Y.gb(), float(t))


def remaining_tendency(Yt, Yt_lim, Y, p, t):
    p.call("gb_remaining_tendency", Yt.gb(), Y.gb(), float(t))
    return Yt


def implicit_tendency(Yt, Y, p, t):
    p.call("gb_implicit_tendency", Yt.gb(), Y.gb(), float(t))


def update_jacobian(jacobian, Y, p, dtgamma, t):
    p.call("gb_update_jacobian", Y.gb(), float(dtgamma), float(t))


def ldiv(dY, jacobian, R):
    jacobian.p.call("gb_ldiv", dY.gb(), R.gb())


def correct_implicit_advection_tendency(Yt, Y, p, t):
    p.call("gb_correct_implicit_advection_tendency", Yt.gb(), Y.gb(), float(t))


def dss(Y, p, t):
    p.call("gb_dss", Y.gb())


def ars343_tableau():
    """Ascher, Ruuth & Spiteri (1997) ARS(3,4,3): (a_exp, a_imp, b_exp, b_imp)."""
    g = 0.4358665215084590
    a42 = a43 = 0.5529291480359398
    b1 = -1.5 * g * g + 4 * g - 0.25
    b2 = 1.5 * g * g - 5 * g + 1.25
    a31 = (1 - 4.5 * g + 1.5 * g * g) * a42 + (2.75 - 10.5 * g + 3.75 * g * g) * a43 - 3.5 + 13 * g - 4.5 * g * g
    a32 = (-1 + 4.5 * g - 1.5 * g * g) * a42 + (-2.75 + 10.5 * g - 3.75 * g * g) * a43 + 4 - 12.5 * g + 4.5 * g * g
    ae = np.array([[0, 0, 0, 0], [g, 0, 0, 0], [a31, a32, 0, 0], [1 - a42 - a43, a42, a43, 0]])
    ai = np.array([[0, 0, 0, 0], [0, g, 0, 0], [0, (1 - g) / 2, g, 0], [0, b1, b2, g]])
    b = np.array([0, b1, b2, g])
    return ae, ai, b, b.copy()


def ars343_step_via_hooks(Y, p, t, dt, dss_first_stage=True):
    """One ClimaTimeSteppers IMEX ARK step (ARS343, NewtonsMethod(max_iters=1))
    driven through the hooks only, as CTS does (AtmosSimulations.jl:317-323)."""
    ae, ai, be, bi = ars343_tableau()
    jac = Jacobian(p)
    Te = [Y.similar() for _ in range(4)]
    Ti = [Y.similar() for _ in range(4)]
    U, Uhat, R, dU, corr = Y.similar(), Y.similar(), Y.similar(), Y.similar(), Y.similar()
    for i in range(4):
        U.assign_(Y)
        for j in range(i):
            if ae[i, j]:
                U.axpy_(dt * ae[i, j], Te[j])
            if ai[i, j]:
                U.axpy_(dt * ai[i, j], Ti[j])
        if i > 0 or dss_first_stage:
            dss(U, p, t)
        if ai[i, i]:
            dtg = dt * ai[i, i]
            Uhat.assign_(U)
            set_precomputed_quantities(U, p, t)           # cache_imp!
            implicit_tendency(R, U, p, t)                  # R = U^ + dtg T_imp(U) - U
            R.c.mul_(dtg).add_(Uhat.c).sub_(U.c)
            R.f.mul_(dtg).add_(Uhat.f).sub_(U.f)
            update_jacobian(jac, U, p, dtg, t)
            ldiv(dU, jac, R)
            U.axpy_(-1.0, dU)
            set_precomputed_quantities(U, p, t)           # cache! after the solve
            if p.cfg.upwinding == "vanleer":
                correct_implicit_advection_tendency(corr, U, p, t)
                U.axpy_(dtg, corr)
            Ti[i].assign_(U).axpy_(-1.0, Uhat)
            Ti[i].c.mul_(1.0 / dtg)
            Ti[i].f.mul_(1.0 / dtg)
        else:
            set_precomputed_quantities(U, p, t)
        remaining_tendency(Te[i], None, U, p, t)
    for j in range(4):
        if be[j]:
            Y.axpy_(dt * be[j], Te[j])
        if bi[j]:
            Y.axpy_(dt * bi[j], Ti[j])
    dss(Y, p, t + dt)
    set_precomputed_quantities(Y, p, t + dt)
    return Y


def simulated_years_per_day(dt, seconds_per_step):
    """SYPD = (dt / year) / (wall seconds per step / day)  (src/simulation/solve.jl:40-45)."""
    return (dt / C.SECONDS_PER_YEAR) / (seconds_per_step / 86400.0)


class AtmosSimulation:
    """State + cache + time of one dry dynamical-core run on the GPU."""

    def __init__(self, config, workload="plain", state=None, device="cuda", restart_file=None,
                 detect_restart_file=False, output_dir=None, t_end=None, dt_save_state_to_disk=None,
                 check_nan_every=None):
        self.config = config
        self.t_end = t_end
        self.dt_save_state_to_disk = dt_save_state_to_disk  # seconds between checkpoints, None / inf: none
        self.check_nan_every = check_nan_every              # steps between NaN scans of the state, None: none
        self.geometry = Geometry(config)
        self.t = 0.0
        if restart_file is None and detect_restart_file and output_dir is not None:
            # the most recent restart file in output_dir, if any (restart.jl:147-160)
            restart_file = R.latest_restart_file(output_dir)
        if restart_file is not None:
            # handle_restart (src/simulation/restart.jl:58-84): the file's time takes precedence
            Yc, Yf, self.t = R.get_state_restart(restart_file, config)
        elif state is None:
            Yc, Yf = S.workload_state(self.geometry, config, workload)
        else:
            Yc, Yf = state
        self.Y = FieldVector.from_numpy(np.asarray(Yc, dtype=config.ft), np.asarray(Yf, dtype=config.ft), device)
        self.p = AtmosCache(config)
        self.dt = config.dt
        self.output_dir = output_dir

    def step(self, nsteps=1, use_graph=True):
        self.p.call("gb_step", self.Y.gb(), float(self.t), float(self.dt), int(nsteps), 1 if use_graph else 0)
        self.t += nsteps * self.dt

    def save_state(self, output_dir):
        """Checkpoint (save_state_to_disk_func, src/callbacks/callbacks.jl:297-321); returns the path."""
        Yc, Yf = self.Y.numpy()
        return R.save_state_to_disk(Yc, Yf, self.t, self.config, output_dir)

    def synchronize(self):
        import torch
        torch.cuda.synchronize()

    def check_nans(self):
        """Raise GBError if the state holds a NaN (check_nans, src/callbacks/callbacks.jl:420-438)."""
        import torch
        bad = [n for n, x in (("c", self.Y.c), ("f", self.Y.f)) if bool(torch.isnan(x).any())]
        if bad:
            raise N.GBError(N.GB_ERR_NONFINITE, "Found NaN in " + ", ".join("Y." + b for b in bad))

    def check(self):
        """Raise GBError if a kernel of the steps so far flagged a failure (a non-finite Newton
        residual, a device wait that timed out); gb_newton_residual reads the status word."""
        self.p.newton_residual()


class AtmosSolveResults:
    """What solve_atmos returns (solve.jl:93-97): ``sol`` the final state (None after a
    crash), ``ret_code`` "success" or "simulation_crashed", ``walltime`` [s] of the timed
    steps (None after a crash); ``seconds_per_step`` and ``sypd`` as solve.jl:40-45 logs them."""

    def __init__(self, sol, ret_code, walltime, seconds_per_step=None, sypd=None):
        self.sol = sol
        self.ret_code = ret_code
        self.walltime = walltime
        self.seconds_per_step = seconds_per_step
        self.sypd = sypd

    def __repr__(self):
        return "AtmosSolveResults(ret_code=%r, walltime=%r, sypd=%r)" % (self.ret_code, self.walltime, self.sypd)


def check_conservation(first, last, moist, energy_surface_change=0.0, energy_radiation_input=0.0):
    """The relative budgets of check_conservation (src/simulation/solve.jl:216-265) from the
    conservation sums (∫ρ, ∫ρe_tot, ∫ρq_tot) of the first and the last state of a run
    (``AtmosCache.conservation_sums``).  A surface without a slab ocean: the energy budget is
    closed by the surface's and the top's net energy fluxes (zero without radiation and surface
    fluxes) and no water leaves through the surface."""
    energy = abs(last[1] - first[1] + energy_surface_change - energy_radiation_input) / first[1]
    mass = (last[0] - first[0]) / first[0]
    water = abs(last[2] - first[2]) / last[2] if moist else 0.0
    return {"energy_conservation": energy, "mass_conservation": mass, "water_conservation": water}


def solve_atmos(sim, nsteps=None, use_graph=True):
    """One untimed step, then ``nsteps`` timed steps (solve.jl:119-149); without ``nsteps``
    the run goes to ``sim.t_end`` as the reference's does (the untimed step included).  A
    library failure ends the run as the reference's catch does: the state is written to
    ``sim.output_dir`` (when set) and the results carry ret_code "simulation_crashed"."""
    if nsteps is None:
        if getattr(sim, "t_end", None) is None:
            raise ValueError("solve_atmos: give nsteps or an AtmosSimulation with t_end")
        nsteps = int(round((sim.t_end - sim.t) / sim.dt)) - 1
        if nsteps < 0:
            raise ValueError("solve_atmos: t_end is less than one step ahead")
    every = getattr(sim, "dt_save_state_to_disk", None)
    every = None if every is None or math.isinf(every) else max(1, int(round(every / sim.dt)))
    if every and not getattr(sim, "output_dir", None):
        raise ValueError("solve_atmos: dt_save_state_to_disk needs an output_dir")
    # check_nan_every <= 0 turns the scan off (nan_checking_callback, get_callbacks.jl:316-330)
    n_nan = getattr(sim, "check_nan_every", None)
    nan_every = int(n_nan) if n_nan and n_nan > 0 else None
    taken = [0]   # steps of this run: call_every_n_steps counts from the run's start

    def steps(n):
        # in runs of steps that end on the callbacks' steps: the NaN scan every `nan_every` steps
        # of this run (call_every_n_steps, src/callbacks/callback_helpers.jl:177-199), then the
        # restart file on multiples of `every` steps from t = 0
        # (save_state_to_disk_func, src/callbacks/callbacks.jl:297-321)
        while n > 0:
            i = int(round(sim.t / sim.dt))
            k = min([n] + ([every - i % every] if every else []) +
                    ([nan_every - taken[0] % nan_every] if nan_every else []))
            sim.step(k, use_graph)
            n -= k
            taken[0] += k
            i = int(round(sim.t / sim.dt))
            if nan_every and taken[0] % nan_every == 0:
                sim.check_nans()
            if every and i % every == 0:
                sim.synchronize()
                sim.save_state(sim.output_dir)

    try:
        if nan_every:
            sim.check_nans()    # the callback's initialize scans the initial state (skip_first = false)
        steps(1)
        sim.synchronize()
        t0 = time.perf_counter()
        steps(nsteps)
        sim.synchronize()
        wall = time.perf_counter() - t0
        sim.check()
    except N.GBError as e:
        import warnings
        if getattr(sim, "output_dir", None):
            sim.save_state(sim.output_dir)
        warnings.warn("simulation crashed: %s" % e)
        return AtmosSolveResults(None, "simulation_crashed", None)
    sps = wall / max(nsteps, 1)
    return AtmosSolveResults(sim.Y, "success", wall, sps, simulated_years_per_day(sim.dt, sps))


# ---------------------------------------------------------------- reverse mode
# Every *_vjp accumulates into its cotangent arguments; each returns the
# (d/dnu, d/d sponge rate) contributions as a length-2 array.
def _dpar():
    return (ctypes.c_double * 2)(0.0, 0.0)


def dss_transpose(X, p):
    p.call("gb_dss_transpose", X.gb())


def remaining_tendency_vjp(Ybar, Tbar, Y, p, t=0.0):
    d = _dpar()
    p.call("gb_remaining_tendency_vjp", Ybar.gb(), Tbar.gb(), Y.gb(), float(t), d)
    return np.array(d[:])


def reduced_like(Y):
    """A zero implicit-tendency FieldVector: c [Nh, 2, 16, Nv] (rho, rho e_tot), f like Y.f."""
    import torch
    Nh, _, nn, Nv = Y.c.shape
    return FieldVector(torch.zeros((Nh, 2, nn, Nv), dtype=Y.c.dtype, device=Y.c.device), torch.zeros_like(Y.f))


def implicit_stage(U, Timp, Uhat, p, dtgamma):
    p.call("gb_implicit_stage", U.gb(), Timp.gb(), Uhat.gb(), float(dtgamma))


def implicit_stage_vjp(Uhat_bar, Ubar, Timp_bar, Uhat, p, dtgamma):
    d = _dpar()
    p.call("gb_implicit_stage_vjp", Uhat_bar.gb(), Ubar.gb(), Timp_bar.gb(), Uhat.gb(), float(dtgamma), d)
    return np.array(d[:])


def step_vjp(Ybar, Y, p, t, dt):
    d = _dpar()
    p.call("gb_step_vjp", Ybar.gb(), Y.gb(), float(t), float(dt), d)
    return np.array(d[:])


def gradient(p, Y0, nsteps, loss_and_grad, dt=None, checkpoint_every=5, record_segments=None):
    """Reverse-mode gradient of a loss of the state after ``nsteps`` steps from Y0.

    The rrule pattern (ChainRulesCore.rrule of the solve): the forward half
    advances a copy of Y0 keeping a checkpoint every ``checkpoint_every``
    steps; ``loss_and_grad(Y_N) -> (J, dJ/dY_N FieldVector)``; the pullback
    returns (J, dJ/dY0, dJ/dnu, dJ/d sponge rate, library bytes at the peak).
    ``record_segments`` (default: the context's setting, initially 1) is how many trailing
    segments the forward half keeps the stage data of, so that the pullback recomputes only
    the segments before them (gb_adjoint_set_record_segments)."""
    dt = p.dt if dt is None else dt
    if record_segments is not None:
        p.call("gb_adjoint_set_record_segments", int(record_segments))
    Y = Y0.copy()
    p.call("gb_adjoint_forward", Y.gb(), 0.0, float(dt), int(nsteps), int(checkpoint_every))
    J, Ybar = loss_and_grad(Y)
    d = _dpar()
    peak = ctypes.c_size_t(0)
    p.call("gb_adjoint_reverse", Ybar.gb(), d, ctypes.byref(peak))
    return J, Ybar, float(d[0]), float(d[1]), int(peak.value)

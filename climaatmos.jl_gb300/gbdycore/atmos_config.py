"""A ClimaAtmos job configuration read into a DycoreConfig.

A ClimaAtmos job is a flat YAML file of options (config/model_configs/*.yml) merged over the
defaults of config/default_configs/default_config.yml (src/config/yaml_helper.jl), plus
optional ClimaParams overrides in a TOML file (toml/*.toml: ``[name]`` tables with a
``value``).  ``from_atmos_config`` applies the reference's defaults for the options the dry
dynamical core reads, maps them onto this library's configuration and refuses, by name, every
option set to something the library does not implement (moisture, EDMF, topography, other
time steppers, ...), so that a job is either run as the reference would run it or not at all.
"""
import math
import re

import numpy as np

from . import config as C

# The reference's defaults of the options read here (config/default_configs/default_config.yml).
DEFAULTS = {
    "config": "sphere", "h_elem": 6, "z_elem": 10, "z_max": 30000.0, "z_stretch": True, "dz_bottom": 500.0,
    "dt": "600secs", "t_end": "10days", "FLOAT_TYPE": "Float32", "hyperdiff": "Hyperdiffusion",
    "vorticity_hyperdiffusion_coefficient": 0.1857, "hyperdiffusion_prandtl_number": 0.2,
    "divergence_damping_factor": 5.0, "rayleigh_sponge": False, "energy_q_tot_upwinding": "vanleer_limiter",
    "rad": None, "deep_atmosphere": True, "ode_algo": "ARS343", "max_newton_iters_ode": 1,
    "use_newton_rtol": False, "output_dir": None, "restart_file": None, "detect_restart_file": False,
    "initial_condition": "DecayingProfile", "dt_save_state_to_disk": "Inf", "check_nan_every": 1024,
}

# Options whose effective value (the job's, else the reference's default, listed first) must
# be the one this library implements (listed second).  The reference's default run applies the
# surface flux tendency (src/prognostic_equations/surface_flux.jl:101-103); this library's dry
# step does not, so a job must disable it as the Held-Suarez jobs do.
REQUIRED = {
    "microphysics_model": ("dry", "dry"), "topography": ("NoWarp", "NoWarp"), "turbconv": (None, None),
    "prognostic_tke": (False, False), "implicit_diffusion": (False, False),
    "orographic_gravity_wave": (None, None), "non_orographic_gravity_wave": (False, False),
    "vert_diff": (None, None), "viscous_sponge": (False, False),
    "disable_surface_flux_tendency": (False, True),
}

# Options that only concern output, logging or the host run and are accepted as given.
HOST_ONLY = {"job_id", "output_dir_style", "dt_save_to_sol", "log_progress",
             "diagnostics", "netcdf_interpolation_num_points", "output_default_diagnostics",
             "check_conservation", "log_to_file", "reproducible_restart",
             "use_itime", "start_date", "toml"}

# CAM-SE preset (src/types.jl:517-522): the hyperviscosity of Lauritzen et al. (2018).
CAM_SE = {"vorticity_hyperdiffusion_coefficient": 0.150 * 1.238, "divergence_damping_factor": 5.0,
          "hyperdiffusion_prandtl_number": 0.2}


def time_to_seconds(s):
    """Seconds of a duration option such as ``10secs``, ``2mins``, ``1.5h``, ``3days``, ``50weeks``
    or ``Inf`` (src/utils/utilities.jl:555-574); numbers are taken as seconds."""
    if isinstance(s, (int, float)) and not isinstance(s, bool):
        return float(s)
    if s == "Inf":
        return math.inf
    m = re.fullmatch(r"(\d+(?:\.\d+)?)(s|secs|m|mins|h|hours|d|days|weeks)", str(s))
    if not m:
        raise ValueError("Bad format for flag %s. Examples: `10secs`, `20mins`, `30hours`, `40days`, `50weeks`" % s)
    factor = {"s": 1, "secs": 1, "m": 60, "mins": 60, "h": 3600, "hours": 3600, "d": 86400, "days": 86400,
              "weeks": 604800}[m.group(2)]
    return float(m.group(1)) * factor


def parse_checkpoint_frequency(period):
    """Seconds between checkpoints, ``inf`` for none (src/callbacks/get_callbacks.jl:231-247): a
    number is seconds, a string anything time_to_seconds reads; ``<N>months`` needs the
    calendar, which this library does not keep (ValueError)."""
    if isinstance(period, str) and "months" in period:
        raise ValueError("checkpoint frequency %r: calendar months are not supported" % period)
    sec = time_to_seconds(period)
    return sec if math.isinf(sec) else float(round(sec))


def _scalar(text):
    t = text.strip()
    if t in ("~", "null", ""):
        return None
    if t in ("true", "false"):
        return t == "true"
    if len(t) >= 2 and t[0] == t[-1] and t[0] in "\"'":
        return t[1:-1]
    try:
        return int(t)
    except ValueError:
        pass
    try:
        return float(t)
    except ValueError:
        return t


def _strip_comment(line):
    quote = None
    for i, ch in enumerate(line):
        if quote:
            quote = None if ch == quote else quote
        elif ch in "\"'":
            quote = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            return line[:i]
    return line


def parse_flat_yaml(text):
    """The ``key: value`` pairs of a flat YAML job file (comments, quotes, ``~``, booleans and
    numbers); a nested or multi-line value raises ValueError."""
    out = {}
    for n, line in enumerate(text.splitlines(), 1):
        body = _strip_comment(line).rstrip()
        if not body.strip():
            continue
        if body[0] in " \t" or ":" not in body:
            raise ValueError("line %d: only flat `key: value` lines are read: %r" % (n, line))
        key, value = body.split(":", 1)
        if value.strip() in ("|", ">"):
            raise ValueError("line %d: multi-line values are not read" % n)
        out[key.strip()] = _scalar(value)
    return out


def node_horizontal_length_scale(h_elem, radius, nq=4):
    """Mean distance between the nodes of the cubed sphere, sqrt(4 pi / 6) R / ((Nq - 1) h_elem)
    (the scale the reference's hyperdiffusion uses; src/types.jl:510-513 states it for ne30)."""
    return math.sqrt(4 * math.pi / 6) * radius / ((nq - 1) * h_elem)


def from_atmos_config(options, params=None):
    """(DycoreConfig, t_end in s, host options) of a job: ``options`` is the job's YAML (a dict
    or the text of the file), ``params`` the ClimaParams overrides (a dict of values, or the
    text of a TOML file).  The host options are the output directory, the restart settings and
    the job's ``initial_condition``, which this library does not build: the caller supplies the
    initial state (or a restart file)."""
    if isinstance(options, str):
        options = parse_flat_yaml(options)
    if isinstance(params, str):
        import tomllib
        params = {k: (v["value"] if isinstance(v, dict) else v) for k, v in tomllib.loads(params).items()}
    params = dict(params or {})
    o = dict(DEFAULTS)
    o.update(options)
    bad = []
    for k in options:
        if k not in DEFAULTS and k not in HOST_ONLY and k not in REQUIRED:
            bad.append("%s (not an option of the dry dynamical core)" % k)
    for k, (default, want) in REQUIRED.items():
        v = options.get(k, default)
        if v != want:
            bad.append("%s: %r (this library implements %r)" % (k, v, want))
    checks = [("config", "sphere"), ("deep_atmosphere", True), ("ode_algo", "ARS343"), ("max_newton_iters_ode", 1),
              ("use_newton_rtol", False)]
    bad += ["%s: %r" % (k, o[k]) for k, want in checks if o[k] != want]
    if o["rad"] not in (None, "held_suarez"):
        bad.append("rad: %r" % o["rad"])
    if o["energy_q_tot_upwinding"] not in ("vanleer_limiter", "none"):
        bad.append("energy_q_tot_upwinding: %r" % o["energy_q_tot_upwinding"])
    if o["FLOAT_TYPE"] not in ("Float32", "Float64"):
        bad.append("FLOAT_TYPE: %r" % o["FLOAT_TYPE"])
    if o["hyperdiff"] not in ("Hyperdiffusion", "CAM_SE", None):
        bad.append("hyperdiff: %r" % o["hyperdiff"])
    if bad:
        raise ValueError("options this library does not implement: " + "; ".join(bad))

    constants = dict(C.CONSTANTS)
    radius = float(params.pop("planet_radius", constants["radius"]))
    constants["radius"] = radius
    h_elem = int(o["h_elem"])
    if o["hyperdiff"] is None:
        nu, prandtl, damp = 0.0, 1.0, 0.0
    else:
        if o["hyperdiff"] == "CAM_SE":
            for k, v in CAM_SE.items():
                if not math.isclose(float(o[k]), v, abs_tol=1e-8):
                    raise ValueError("CAM_SE hyperdiffusion overwrites %s, use `hyperdiff: Hyperdiffusion`" % k)
        coeff = float(o["vorticity_hyperdiffusion_coefficient"])
        nu = coeff * node_horizontal_length_scale(h_elem, radius) ** 3
        prandtl, damp = float(o["hyperdiffusion_prandtl_number"]), float(o["divergence_damping_factor"])
    zd = a_uh = a_w = 0.0
    if o["rayleigh_sponge"]:
        missing = [k for k in ("zd_rayleigh", "alpha_rayleigh_uh", "alpha_rayleigh_w") if k not in params]
        if missing:
            raise ValueError("rayleigh_sponge: ClimaParams is not available here; give %s" % ", ".join(missing))
        zd, a_uh, a_w = (float(params.pop(k)) for k in ("zd_rayleigh", "alpha_rayleigh_uh", "alpha_rayleigh_w"))
    cfg = C.DycoreConfig(
        h_elem=h_elem, z_elem=int(o["z_elem"]), z_max=float(o["z_max"]), z_stretch=bool(o["z_stretch"]),
        dz_bottom=float(o["dz_bottom"]), ft=np.float32 if o["FLOAT_TYPE"] == "Float32" else np.float64,
        dt=time_to_seconds(o["dt"]), nu=nu, prandtl=prandtl, divergence_damping=damp, sponge_zd=zd,
        alpha_uh=a_uh, alpha_w=a_w, upwinding="vanleer" if o["energy_q_tot_upwinding"] == "vanleer_limiter" else "none",
        constants=constants, held_suarez=o["rad"] == "held_suarez")
    host = {k: o.get(k) for k in ("output_dir", "restart_file", "detect_restart_file", "initial_condition")}
    host["dt_save_state_to_disk"] = parse_checkpoint_frequency(o["dt_save_state_to_disk"])
    host["check_nan_every"] = int(o["check_nan_every"])
    return cfg, time_to_seconds(o["t_end"]), host

"""Checkpoint / restart of the prognostic state.

Mirrors the reference's restart files (save_state_to_disk_func,
src/callbacks/callbacks.jl:297-321; get_state_restart, src/simulation/restart.jl:22-42):
the file is named ``day{day}.{sec}`` from the elapsed simulation time and holds the state
``Y`` with two attributes, ``time`` (s) and ``atmos_model_hash`` (a hash of the model
configuration); a restart warns when the hash differs from the running model's.  The
container is numpy's ``.npz`` (``Y_c`` centres ``[Nh][4][16][Nv]``, ``Y_f`` faces
``[Nh][16][Nv+1]``, the library's layout) instead of ClimaCore's HDF5 (no HDF5 library is
available here), so the files are not interchangeable with the reference's.
"""
import hashlib
import json
import os
import warnings

import numpy as np

FORMAT = "gbdycore-restart-1"


def _model_record(cfg):
    """The configuration fields that define the model (grid, numerics, physics)."""
    return {
        "h_elem": cfg.h_elem, "z_elem": cfg.z_elem, "z_max": cfg.z_max, "z_stretch": bool(cfg.z_stretch),
        "dz_bottom": cfg.dz_bottom, "ft": np.dtype(cfg.ft).name, "nu": cfg.nu, "prandtl": cfg.prandtl,
        "divergence_damping": cfg.divergence_damping, "sponge_zd": cfg.sponge_zd, "alpha_uh": cfg.alpha_uh,
        "alpha_w": cfg.alpha_w, "upwinding": cfg.upwinding, "constants": dict(sorted(cfg.constants.items())),
        "held_suarez": bool(cfg.held_suarez), "hs": dict(sorted(cfg.hs.items())),
    }


def atmos_model_hash(cfg):
    """A stable 63-bit hash of the model configuration (the time step is not part of it)."""
    text = json.dumps(_model_record(cfg), sort_keys=True, default=float)
    return int.from_bytes(hashlib.sha256(text.encode()).digest()[:8], "little") >> 1


def restart_file_name(t):
    """``day{day}.{sec}`` of simulation time t (s), as the reference names its files."""
    day = int(np.floor(t / 86400.0))
    sec = int(np.floor(t % 86400.0))
    return "day%d.%d.npz" % (day, sec)


def time_from_filename(path):
    """Simulation time (s) from a ``day{day}.{sec}.*`` file name
    (src/utils/utilities.jl:158-163)."""
    parts = os.path.basename(path).split(".")
    return float(parts[0].replace("day", "")) * 86400.0 + float(parts[1])


def sort_files_by_time(paths):
    """The paths ordered by the time in their names (src/utils/utilities.jl:171-172)."""
    return sorted(paths, key=time_from_filename)


def latest_restart_file(output_dir):
    """The restart file of the latest time in output_dir, or None (the last of the
    time-sorted ``day*`` files, as auto_detect_restart_file, src/simulation/restart.jl:109-134)."""
    if not os.path.isdir(output_dir):
        return None
    files = [os.path.join(output_dir, f) for f in os.listdir(output_dir)
             if f.startswith("day") and f.endswith(".npz")]
    return sort_files_by_time(files)[-1] if files else None


def save_state_to_disk(Yc, Yf, t, cfg, output_dir):
    """Write the state (numpy arrays) at time t; returns the file path."""
    os.makedirs(output_dir, exist_ok=True)
    path = os.path.join(output_dir, restart_file_name(t))
    with open(path, "wb") as fh:
        np.savez(fh, Y_c=np.ascontiguousarray(Yc), Y_f=np.ascontiguousarray(Yf), time=np.float64(t),
                 atmos_model_hash=np.uint64(atmos_model_hash(cfg)), format=np.array(FORMAT),
                 model=np.array(json.dumps(_model_record(cfg), sort_keys=True, default=float)))
    return path


def get_state_restart(path, cfg):
    """(Y_c, Y_f, time) from a restart file.  The state must fit cfg's grid and precision
    (ValueError otherwise); a different model hash warns, as the reference does."""
    with np.load(path, allow_pickle=False) as z:
        if str(z["format"]) != FORMAT:
            raise ValueError("%s: not a restart file of this library" % path)
        Yc, Yf, t = z["Y_c"], z["Y_f"], float(z["time"])
        h = int(z["atmos_model_hash"])
    Nh = 6 * cfg.h_elem * cfg.h_elem
    if Yc.shape != (Nh, 4, 16, cfg.z_elem) or Yf.shape != (Nh, 16, cfg.z_elem + 1):
        raise ValueError("%s: state shape %s / %s does not match the configured grid" % (path, Yc.shape, Yf.shape))
    if Yc.dtype != np.dtype(cfg.ft):
        raise ValueError("%s: state precision %s, configured %s" % (path, Yc.dtype, np.dtype(cfg.ft)))
    if h != atmos_model_hash(cfg):
        warnings.warn("Restart file %s was constructed with a different AtmosModel" % path)
    return Yc, Yf, t

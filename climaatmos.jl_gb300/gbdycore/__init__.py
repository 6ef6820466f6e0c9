"""gbdycore: GB300-native dry dynamical-core IMEX step of ClimaAtmos.jl.

The compute path is libgbdycore.so (hand-written CUDA for sm_103a, C ABI in
include/gbdycore.h); this package is the host-side mirror of the reference's
simulation API and hook surface.
"""
from . import config, setups  # noqa: F401

__all__ = ["config", "setups", "simulation", "build"]

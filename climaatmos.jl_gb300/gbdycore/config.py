"""Model configuration: pinned constants and the workload configurations.

Mirrors the keyword surface of ``AtmosSimulation{FT}(; ...)``
(src/simulation/AtmosSimulations.jl:307) and ``SphereGrid``
(src/simulation/grids.jl:42-89) for the dry dynamical core, and pins the
physical constants that the reference takes from ClimaParams 1.1.4
(src/parameters/Parameters.jl:541-568), which is not available here.
"""
from dataclasses import dataclass, field, replace

import numpy as np

# Physical constants.  R_d and cp_d are fixed by the workload definition;
# the rest are the ClimaParams defaults for the named quantities; the radius
# is the SphereGrid default (src/simulation/grids.jl:49).
CONSTANTS = dict(
    grav=9.81,
    omega=7.2921159e-5,
    R_d=287.0,
    cp_d=1004.0,
    cv_d=1004.0 - 287.0,
    T_0=273.16,          # reference temperature of internal energy
    p_ref=1.0e5,         # reference pressure of the Exner function
    T_min_ref=220.0,     # reference-state minimum temperature (refstate_thermodynamics.jl:79)
    T_surf_ref=290.0,    # reference-state surface temperature
    T_min_sgs=150.0,     # temperature floor of the precomputed T (precomputed_quantities.jl:787-796)
    radius=6.371229e6,
)

# Held-Suarez forcing parameters (dry values; Held and Suarez 1994, the values
# ClimaParams names day, sigma_b, Delta T_y (dry), T_equator (dry), Delta theta_z,
# T_min_hs, p_ref_theta and MSLP; held_suarez.jl:40-70).
HELD_SUAREZ = dict(
    day=86400.0,
    sigma_b=0.7,
    dT_y=60.0,
    T_equator=315.0,
    dtheta_z=10.0,
    T_min=200.0,
    p_ref_theta=1.0e5,
    MSLP=101325.0,
)

# Moist thermodynamic constants of the 0M microphysics (EquilibriumMicrophysics0M): the
# ClimaParams defaults under their Thermodynamics.jl names; R_v = R / M_w with the gas constant
# 8.3144598 J/(mol K) and the molar mass of water 0.01801528 kg/mol.
MOIST = dict(
    R_v=8.3144598 / 0.01801528,
    cp_v=1859.0,
    cp_l=4181.0,
    cp_i=2100.0,
    LH_v0=2.5008e6,
    LH_s0=2.8344e6,
    T_triple=273.16,
    press_triple=611.657,
    T_freeze=273.15,
    T_icenuc=233.0,
    pow_icenuc=1.0,
)

SECONDS_PER_YEAR = 3.1536e7  # 365-day year, as in simulated_years_per_day (src/simulation/solve.jl:40-45)


def hyperdiffusion_nu(h_elem, nu30=1.0e15):
    """Absolute fourth-order hyperdiffusivity nu = nu30 (h_elem / 30)^-3 m^4/s.

    The workload definition names nu30 = 1e16, but with its time steps that
    value lies outside the explicit stability region of ARS343 (at h_elem=6,
    dt=400 s the limit is between 3e17 and 6e17 against the named 1.25e18).
    The default is therefore the classic spectral-element value nu30 = 1e15,
    which is stable at every workload's time step; pass ``nu=`` to a config
    to use another value.
    """
    return nu30 * (h_elem / 30.0) ** -3


@dataclass
class DycoreConfig:
    """Grid, numerics and physics of one dry dynamical-core run.

    ``ft`` is ``np.float32`` or ``np.float64``.  ``upwinding`` selects the
    ``energy_q_tot_upwinding`` option: ``"vanleer"`` (the reference default,
    src/types.jl:1916) or ``"none"``.
    """

    h_elem: int = 6
    z_elem: int = 10
    z_max: float = 30000.0
    z_stretch: bool = False
    dz_bottom: float = 500.0
    ft: type = np.float32
    dt: float = 400.0
    nu: float = None                 # nu_4 for momentum; defaults to hyperdiffusion_nu(h_elem)
    prandtl: float = 1.0             # nu_scalar = nu / prandtl
    divergence_damping: float = 5.0  # divergence_damping_factor (src/types.jl:1925-1929)
    sponge_zd: float = 0.0
    alpha_uh: float = 0.0
    alpha_w: float = 0.0
    upwinding: str = "vanleer"
    constants: dict = field(default_factory=lambda: dict(CONSTANTS))
    held_suarez: bool = False        # rad: held_suarez (src/config/model_getters.jl:636)
    hs: dict = field(default_factory=lambda: dict(HELD_SUAREZ))
    # numerics.test_dycore_consistency (src/utils/debug_utils.jl:58-70): NaN-fill scratch first
    test_dycore_consistency: bool = False
    # the caller's element layout: (elem_map [Nh], elem_orient [Nh]) arrays, None: library order
    layout: tuple = None
    # terrain-following levels (src/topography/topography.jl): the surface elevation of every
    # node [Nh, 16] in m (None: flat), the warp ("linear" or "sleve") and SLEVE's eta_h and s
    z_surface: object = None
    warp: str = "linear"
    sleve_eta: float = 0.7
    sleve_s: float = 10.0
    # moist 0M (microphysics_model: 0M, EquilibriumMicrophysics0M): rho q_tot is the fifth centre
    # component; the column hooks only.  sa_iters: Newton iterations of the saturation adjustment
    moist: bool = False
    moist_constants: dict = field(default_factory=lambda: dict(MOIST))
    sa_iters: int = 16

    def __post_init__(self):
        if self.nu is None:
            self.nu = hyperdiffusion_nu(self.h_elem)

    @property
    def nu_s(self):
        return self.nu / self.prandtl

    def with_(self, **kw):
        return replace(self, **kw)

    def oracle_params(self, dss_stage1=True):
        """The parameter record of the CPU oracle (test infrastructure)."""
        p = dict(self.constants)
        p.update(nu_v=self.nu, nu_s=self.nu_s, div_damp=self.divergence_damping, sponge_zd=self.sponge_zd,
                 alpha_uh=self.alpha_uh, alpha_w=self.alpha_w, z_max=self.z_max, dt_model=self.dt,
                 upwinding=1 if self.upwinding == "vanleer" else 0, dss_stage1=1 if dss_stage1 else 0,
                 held_suarez=1 if self.held_suarez else 0)
        p.update({"hs_" + k: v for k, v in self.hs.items()})
        p.update(self.moist_constants)
        p.update(moist=1 if self.moist else 0, sa_iters=self.sa_iters)
        return p


# Workload configurations of the dry IMEX step.
def plain_h6():
    """Plain dry IMEX step: h_elem=6, Nq=4, z_elem=10 uniform to 30 km, dt=400 s, 10 steps."""
    return DycoreConfig(h_elem=6, z_elem=10, z_max=30000.0, z_stretch=False, dt=400.0)


def production_h30():
    """Production resolution: h_elem=30, z_elem=63 tanh-stretched from 30 m to 30 km, dt=120 s."""
    return DycoreConfig(h_elem=30, z_elem=63, z_max=30000.0, z_stretch=True, dz_bottom=30.0, dt=120.0)


def differentiation_h16(rate=1.0e-4):
    """Differentiation: h_elem=16, z_elem=45, dt=200 s, Rayleigh sponge above 20 km."""
    return DycoreConfig(h_elem=16, z_elem=45, z_max=30000.0, z_stretch=True, dz_bottom=500.0, dt=200.0,
                        sponge_zd=20000.0, alpha_uh=rate, alpha_w=rate)


def precision_h60():
    """Precision / checkpointed adjoint at scale: h_elem=60, z_elem=63 stretched, dt=60 s."""
    return DycoreConfig(h_elem=60, z_elem=63, z_max=30000.0, z_stretch=True, dz_bottom=30.0, dt=60.0)

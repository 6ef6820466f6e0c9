"""A ClimaAtmos job configuration read into this library's configuration (CPU only):
time_to_seconds against the reference's known answers (test/utilities.jl:17-45), the
reference's defaults and hyperdiffusion scaling, a Held-Suarez job, and the refusal of
options the dry dynamical core does not implement."""
import math

import numpy as np
import pytest

from gbdycore import atmos_config as A


def test_time_to_seconds_known_answers():
    t = A.time_to_seconds
    assert t("10s") == 10 and t("10secs") == 10
    assert t("2m") == 120 and t("2mins") == 120
    assert t("1h") == 3600 and t("1hours") == 3600
    assert t("3d") == 3 * 86400 and t("3days") == 3 * 86400
    assert t("50weeks") == 50 * 7 * 86400
    assert t("1.5h") == 1.5 * 3600
    assert t("Inf") == math.inf
    for bad in ("10", "10lightyears"):
        with pytest.raises(ValueError):
            t(bad)


def test_flat_yaml():
    d = A.parse_flat_yaml('# job\nh_elem: 30  # per edge\ndt: "120secs"\nz_stretch: true\nrad: ~\n'
                          'note: "a # b"\nlist: [a, b]\n')
    assert d == {"h_elem": 30, "dt": "120secs", "z_stretch": True, "rad": None, "note": "a # b", "list": "[a, b]"}
    with pytest.raises(ValueError):
        A.parse_flat_yaml("a:\n  nested: 1\n")
    with pytest.raises(ValueError):
        A.parse_flat_yaml("help: |\n  text\n")


def test_defaults_and_hyperdiffusion_scaling():
    cfg, t_end, host = A.from_atmos_config({"disable_surface_flux_tendency": True})
    assert (cfg.h_elem, cfg.z_elem, cfg.z_max, cfg.z_stretch, cfg.dz_bottom) == (6, 10, 30000.0, True, 500.0)
    assert cfg.dt == 600.0 and t_end == 10 * 86400.0 and cfg.ft is np.float32
    assert cfg.upwinding == "vanleer" and cfg.divergence_damping == 5.0 and cfg.prandtl == 0.2
    assert not cfg.held_suarez and cfg.alpha_uh == cfg.alpha_w == 0.0
    # nu_4 = coeff h^3, h the mean nodal distance: for ne30 sqrt(4 pi / 6) R / 90 (src/types.jl:510-513)
    c30, _, _ = A.from_atmos_config({"disable_surface_flux_tendency": True, "h_elem": 30})
    h = math.sqrt(4 * math.pi / 6) * 6.371229e6 / 90
    assert c30.nu == pytest.approx(0.1857 * h ** 3, rel=1e-12) and c30.nu == pytest.approx(2.0e14, rel=2e-3)
    assert host == {"output_dir": None, "restart_file": None, "detect_restart_file": False,
                    "initial_condition": "DecayingProfile", "dt_save_state_to_disk": math.inf,
                    "check_nan_every": 1024}


def test_held_suarez_job():
    job = """
z_max: 55000.0
viscous_sponge: false
implicit_diffusion: false
dt_save_state_to_disk: "2days"
t_end: "2days"
disable_surface_flux_tendency: true
rad: "held_suarez"
toml: [toml/sphere_held_suarez.toml]
FLOAT_TYPE: "Float64"
energy_q_tot_upwinding: none
"""
    cfg, t_end, _ = A.from_atmos_config(job)
    assert cfg.held_suarez and cfg.z_max == 55000.0 and t_end == 2 * 86400.0
    assert cfg.ft is np.float64 and cfg.upwinding == "none"


def test_sponge_parameters_from_toml():
    params = "[zd_rayleigh]\nvalue = 15000.0\n[alpha_rayleigh_uh]\nvalue = 1e-4\n[alpha_rayleigh_w]\nvalue = 1.0\n"
    cfg, _, _ = A.from_atmos_config({"disable_surface_flux_tendency": True, "rayleigh_sponge": True}, params)
    assert (cfg.sponge_zd, cfg.alpha_uh, cfg.alpha_w) == (15000.0, 1e-4, 1.0)
    with pytest.raises(ValueError, match="zd_rayleigh"):
        A.from_atmos_config({"disable_surface_flux_tendency": True, "rayleigh_sponge": True})


def test_cam_se_and_no_hyperdiffusion():
    base = {"disable_surface_flux_tendency": True}
    cfg, _, _ = A.from_atmos_config(dict(base, hyperdiff="CAM_SE"))
    assert cfg.prandtl == 0.2 and cfg.divergence_damping == 5.0
    with pytest.raises(ValueError, match="CAM_SE"):
        A.from_atmos_config(dict(base, hyperdiff="CAM_SE", vorticity_hyperdiffusion_coefficient=0.5))
    cfg, _, _ = A.from_atmos_config(dict(base, hyperdiff=None))
    assert cfg.nu == 0.0


@pytest.mark.parametrize("opt", [
    {},                                             # the reference's default run applies surface fluxes
    {"microphysics_model": "0M"}, {"topography": "DCMIP200"}, {"turbconv": "prognostic_edmfx"},
    {"ode_algo": "SSP333"}, {"max_newton_iters_ode": 2}, {"rad": "gray"}, {"config": "column"},
    {"deep_atmosphere": False}, {"energy_q_tot_upwinding": "third_order"}, {"some_unknown_option": 1},
])
def test_unimplemented_options_are_refused_by_name(opt):
    job = dict({"disable_surface_flux_tendency": True}, **opt) if opt else {}
    with pytest.raises(ValueError) as e:
        A.from_atmos_config(job)
    key = next(iter(opt)) if opt else "disable_surface_flux_tendency"
    assert key in str(e.value)


def test_checkpoint_frequency():
    # src/callbacks/get_callbacks.jl:231-247
    p = A.parse_checkpoint_frequency
    assert p("2days") == 172800.0 and p(3600) == 3600.0 and p(90.4) == 90.0 and math.isinf(p("Inf"))
    with pytest.raises(ValueError, match="months"):
        p("2months")
    _, _, host = A.from_atmos_config({"disable_surface_flux_tendency": True, "dt_save_state_to_disk": "1hours"})
    assert host["dt_save_state_to_disk"] == 3600.0

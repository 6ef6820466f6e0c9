#!/usr/bin/env python
"""Throughput of the dry dynamical-core IMEX step (SYPD) on the production workload.

Workload: h_elem=30 cubed sphere (5400 elements, Nq=4), z_elem=63 levels
tanh-stretched from 30 m to 30 km, FP32, dt=120 s, balanced lapse-rate state
with the seeded wind perturbation and Gaussian rho e_tot bump.  One "step" is
one full ARS343 IMEX step (4 explicit stages, 3 implicit stages with one
Newton iteration each), replayed from a captured CUDA graph.

The working set per step (state, four explicit and three implicit stage
tendencies, Laplacians: ~0.9 GB) exceeds the 129 MB L2, so no L2 flush is
inserted between steps.

--impl reference times the CPU port of the reference's step (the C++ oracle,
OpenMP over all host cores): the reference itself is Julia and cannot run here.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "climaatmos.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "SYPD"
UNIT = "simulated years per day"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-config1", action="store_true")
    ap.add_argument("--precision-steps", type=int, default=20)
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--fp64-steps", type=int, default=5)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--batch-columns", type=int, default=20000)
    ap.add_argument("--batch-reps", type=int, default=10)
    ap.add_argument("--no-batching", action="store_true")
    ap.add_argument("--adjoint-steps", type=int, default=10)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--fd-directions", type=int, default=32)
    ap.add_argument("--no-differentiation", action="store_true")
    ap.add_argument("--no-h60", action="store_true")
    ap.add_argument("--held-suarez-steps", type=int, default=20)
    ap.add_argument("--held-suarez-long", type=int, default=1000)
    ap.add_argument("--no-held-suarez", action="store_true")
    ap.add_argument("--topography-steps", type=int, default=20)
    ap.add_argument("--no-topography", action="store_true")
    ap.add_argument("--no-moist", action="store_true")
    # bracket one forward step ("step") or one reverse pass ("reverse") by
    # cudaProfilerStart/Stop, for `ncu --profile-from-start off`; no effect otherwise
    # ("topography": one step of the terrain-following workload)
    ap.add_argument("--profile-region", default="none", choices=["none", "step", "reverse", "topography"])
    return ap.parse_args(argv)


def workload():
    from gbdycore import config as C
    return C.production_h30()


def workload_desc(cfg):
    P = 6 * cfg.h_elem ** 2 * 16 * cfg.z_elem
    return {"workload": "dry IMEX step, production resolution: h_elem=%d (%d elements), Nq=4, z_elem=%d "
                        "tanh-stretched dz_bottom=%g m to %g m, FP32, dt=%g s, ARS343 + 1 Newton iteration"
                        % (cfg.h_elem, 6 * cfg.h_elem ** 2, cfg.z_elem, cfg.dz_bottom, cfg.z_max, cfg.dt),
            "h_elem": cfg.h_elem, "z_elem": cfg.z_elem, "centre_points": P, "dt_s": cfg.dt,
            "nu4": cfg.nu, "upwinding": cfg.upwinding,
            "l2": "no flush: per-step working set ~0.9 GB > 129 MB L2"}


def sypd(dt, seconds_per_step):
    return (dt / 3.1536e7) / (seconds_per_step / 86400.0)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm),
                "window": "untimed steps of the workload (~0.6 s) and the timed steps after them"}


# ------------------------------------------------------------------ CPU baseline (oracle port)
def cpu_step_seconds(cfg, steps, warmup):
    """Seconds per step of the C++ port of the reference step on all host cores."""
    from geometry import OracleGeometry
    import oracle as O
    from gbdycore import setups as S
    g = OracleGeometry(cfg.h_elem, cfg.z_elem, cfg.z_max, cfg.z_stretch, cfg.dz_bottom)
    Yc, Yf = S.workload_state(g, cfg, "production")
    o = O.Oracle(g, cfg.oracle_params(), np.float32)
    Yc, Yf = Yc.astype(np.float32), Yf.astype(np.float32)
    for _ in range(warmup):
        o.step(Yc, Yf, cfg.dt, 1)
    t0 = time.perf_counter()
    for _ in range(steps):
        o.step(Yc, Yf, cfg.dt, 1)
    dt = (time.perf_counter() - t0) / max(steps, 1)
    return dt, O.max_threads()


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    cfg = workload()
    sec, cores = cpu_step_seconds(cfg, args.steps, args.warmup)
    v = sypd(cfg.dt, sec)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded balanced state, the workload's perturbations)",
            "config": workload_desc(cfg), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d full production steps after %d warm-up (C++ port of the reference step, "
                                       "OpenMP); the Julia reference cannot run on this machine" % (args.steps, args.warmup)},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm
KERNELS = [  # (id, name, launches per step)
    (0, "k_passA (Laplacians, prep_hyperdiffusion)", 4),
    (1, "k_passB (explicit tendency)", 3),
    (2, "k_col_stage (implicit column solve)", 3),
    (3, "k_dss (direct stiffness summation)", 8),
    (9, "k_passB_final (last stage's explicit tendency with the final combination folded in)", 1),
]
LAUNCHES_PER_STEP = sum(k[2] for k in KERNELS)  # 19: the launches of one graph-replayed step
REVERSE_KERNELS = [  # (id, name, launches per reverse step)
    (6, "k_passB_vjp (explicit tendency transpose)", 4),
    (5, "k_passA_vjp (Laplacian transpose)", 4),
    (7, "k_col_stage_vjp (implicit column stage transpose)", 3),
    (8, "k_dss_t (DSS transpose)", 8),
]


def algorithmic_bytes(cfg, kid, fb=4):
    """Compulsory HBM bytes of one launch (state-sized fields + geometry actually read)."""
    Nh, Nv = 6 * cfg.h_elem ** 2, cfg.z_elem
    P = Nh * 16 * Nv
    F = Nh * 16 * (Nv + 1)
    S = 4 * P + F
    T = 2 * P + F                  # implicit tendency (rho, rho e_tot, u_3)
    geo = Nh * 11 * 16             # per-node metric terms
    words = {
        0: S + 4 * P + geo,        # read state + geometry, write 4 Laplacian fields
        1: 2 * S + 4 * P + geo,    # read state + Laplacians + geometry, write tendency
        2: 5 * S + 3 * T,          # stage 4: read u_n + 3 T_exp + 2 T_imp, write U + T_imp
        3: int(1.5 * S),           # read + write the 12 of 16 element-boundary nodes
        4: 5 * S + 3 * T,          # read u_n + 3 T_exp + 3 T_imp, write u_{n+1}
        9: 5 * S + 4 * P + geo,    # read U_4 + Laplacians + 3 T_exp + geometry, write u_{n+1}
    }[kid]
    return words * fb


def contract_bytes_per_step(cfg, fb=4):
    Nh, Nv = 6 * cfg.h_elem ** 2, cfg.z_elem
    P = Nh * 16 * Nv
    S = 4 * P + Nh * 16 * (Nv + 1)
    return (51 * S + 56 * P) * fb


# ncu-measured DRAM traffic per launch on the production FP32 workload (bytes)
NCU_TRAFFIC = {"k_passB": 200229376 + 72189440, "k_col_stage": 572398336 + 152322048}


def measured_peak():
    try:
        m = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def run_gb300(args):
    import ctypes
    import torch
    import torch.distributed as dist
    from gbdycore import replicas as rep
    from gbdycore import simulation as sim

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    cfg = workload()
    s = sim.AtmosSimulation(cfg, workload="production")   # inputs resident in HBM
    stream = torch.cuda.current_stream()
    for _ in range(args.warmup):
        s.step(1)
    torch.cuda.synchronize()
    rep.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    # the sampler reads the clocks every 200 ms, longer than the timed steps take: it runs over
    # ~0.6 s of untimed steps of the same workload that lead straight into the timed ones,
    # which then start again from the state the warm-up left
    y0c, y0f, t0 = s.Y.c.clone(), s.Y.f.clone(), s.t
    t_load = time.perf_counter()
    while time.perf_counter() - t_load < 0.6:
        s.step(10)
        torch.cuda.synchronize()
    s.Y.c.copy_(y0c)
    s.Y.f.copy_(y0f)
    s.t = t0
    del y0c, y0f
    rep.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s.step(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    ms = rep.max_over_ranks(ms, device="cuda")
    rep.barrier()
    finite = bool(torch.isfinite(s.Y.c).all() and torch.isfinite(s.Y.f).all())
    if args.profile_region == "step":
        torch.cuda.profiler.start()
        s.step(1)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    v1 = sypd(cfg.dt, ms / 1e3)
    value = rep.job_value(v1)  # independent replicas, one per GPU

    # per-kernel timing (CUDA events on the context stream, inside the library)
    peak, peak_kind = measured_peak()
    ktime = {}
    for kid, name, per_step in KERNELS:
        out = ctypes.c_double()
        s.p.call("gb_time_kernel", kid, s.Y.gb(), 20, ctypes.byref(out))
        ktime[kid] = out.value
    kinfo = {kid: (name, per_step) for kid, name, per_step in KERNELS}
    share = {kid: ktime[kid] * kinfo[kid][1] for kid in ktime}
    dom = max(share, key=share.get)
    ach = algorithmic_bytes(cfg, dom) / (ktime[dom] * 1e-3) / 1e9
    # DRAM bytes (read + write) of one launch from an ncu capture of this workload
    traffic = NCU_TRAFFIC.get(kinfo[dom][0].split()[0]) if cfg == workload() else None
    roof = {"kernel": kinfo[dom][0], "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "peak_kind": peak_kind, "traffic": traffic,
            "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum, one launch "
                              "(profiles/k_passB_h30z63_fp32.md, profiles/k_col_stage_g_h30z63_fp32.md)",
            "algorithmic_bytes_per_launch": algorithmic_bytes(cfg, dom), "ms_per_launch": ktime[dom],
            "kernels": {kinfo[k][0]: {"ms": ktime[k], "launches_per_step": kinfo[k][1],
                                        "GBps": algorithmic_bytes(cfg, k) / (ktime[k] * 1e-3) / 1e9}
                        for k in ktime}}
    cb = contract_bytes_per_step(cfg)
    step_roof = {"contract_bytes_per_step": cb, "achieved_GBps": cb / (ms * 1e-3) / 1e9,
                 "frac": cb / (ms * 1e-3) / 1e9 / peak}

    # end to end through the C ABI with host buffers: H2D state, one step, D2H state
    hc = torch.empty(s.Y.c.shape, dtype=s.Y.c.dtype, pin_memory=True)
    hf = torch.empty(s.Y.f.shape, dtype=s.Y.f.dtype, pin_memory=True)
    hc.copy_(s.Y.c)
    hf.copy_(s.Y.f)
    torch.cuda.synchronize()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(stream)
    for _ in range(args.e2e_steps):
        s.Y.c.copy_(hc, non_blocking=True)
        s.Y.f.copy_(hf, non_blocking=True)
        s.step(1)
        hc.copy_(s.Y.c, non_blocking=True)
        hf.copy_(s.Y.f, non_blocking=True)
    e3.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e2.elapsed_time(e3) / args.e2e_steps
    nbytes = hc.numel() * hc.element_size() + hf.numel() * hf.element_size()
    e2e = {"value": sypd(cfg.dt, ms_e2e / 1e3) * world, "unit": UNIT, "h2d_bytes_per_step": nbytes,
           "d2h_bytes_per_step": nbytes, "ms_per_step": ms_e2e}

    # plain form: the same step through the individual hooks (one C-ABI call per hook,
    # unfused stage algebra in torch), as ClimaTimeSteppers drives the reference
    plain_ms = None
    if not args.no_plain:
        Yp = s.Y.copy()
        sim.ars343_step_via_hooks(Yp, s.p, 0.0, cfg.dt)
        torch.cuda.synchronize()
        e4, e5 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e4.record(stream)
        for k in range(args.plain_steps):
            sim.ars343_step_via_hooks(Yp, s.p, k * cfg.dt, cfg.dt)
        e5.record(stream)
        torch.cuda.synchronize()
        plain_ms = e4.elapsed_time(e5) / args.plain_steps
        del Yp

    # precision: the FP32 step against the FP64 step of the same library (which
    # matches the FP64 oracle to 1e-10), per prognostic field after n steps
    prec = None
    if not args.no_precision:
        from gbdycore import setups as S
        n = args.precision_steps
        c64 = cfg.with_(ft=np.float64)
        g = s.geometry
        Yc, Yf = S.workload_state(g, c64, "production")
        s64 = sim.AtmosSimulation(c64, state=(Yc, Yf))
        s32 = sim.AtmosSimulation(cfg, state=(Yc.astype(np.float32), Yf.astype(np.float32)))
        s64.step(n)
        s32.step(n)
        a, b = s32.Y.numpy(), s64.Y.numpy()
        prec = {"steps": n}
        prec.update(field_errors(a, b))
        del s64, s32

    # the FP64 library on the same workload: the configuration whose velocities meet the
    # metric's 1e-5 against FP64 (it is the FP64 computation); FP32 state storage alone keeps
    # u_h at ~4e-5 after 20 steps (the oracle's storage-floor build)
    fp64 = None
    if not args.no_fp64:
        from gbdycore import setups as S
        c64 = cfg.with_(ft=np.float64)
        Yc, Yf = S.workload_state(s.geometry, c64, "production")
        s64 = sim.AtmosSimulation(c64, state=(Yc, Yf))
        s64.step(2)
        torch.cuda.synchronize()
        e6, e7 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e6.record(stream)
        s64.step(args.fp64_steps)
        e7.record(stream)
        torch.cuda.synchronize()
        ms64 = e6.elapsed_time(e7) / args.fp64_steps
        fp64 = {"ms_per_step": ms64, "value": sypd(cfg.dt, ms64 / 1e3), "unit": UNIT, "dtype": "f64",
                "steps": args.fp64_steps, "fp32_over_fp64_speed": ms64 / ms,
                "what": "the same production step in FP64 (state and arithmetic): the configuration that meets "
                        "<= 1e-5 against FP64 on every field"}
        del s64

    batching = None
    if not args.no_batching:
        batching = measure_batching(args)
    held_suarez = None
    if not args.no_held_suarez:
        held_suarez = measure_held_suarez(args, ms)
    moist = None
    if not args.no_moist:
        try:
            moist = measure_moist(args)
        except Exception as e:  # reported in the line, not fatal
            moist = {"error": "%s: %s" % (type(e).__name__, e)}
    topography = None
    if not args.no_topography:
        try:
            topography = measure_topography(args, ms)
        except Exception as e:  # reported in the line, not fatal to the headline
            topography = {"error": "%s: %s" % (type(e).__name__, e)}
    config1 = None
    if not args.no_config1:
        try:
            config1 = measure_config1(args, rank == 0 and world == 1 and not args.no_cpu_baseline)
        except Exception as e:  # reported in the line, not fatal to the headline
            config1 = {"error": "%s: %s" % (type(e).__name__, e)}

    adjoint = None
    if not args.no_adjoint:
        adjoint = measure_adjoint(args, s, ms)
    differentiation = None
    if not args.no_differentiation:
        differentiation = measure_differentiation(args)
    h60 = None
    if not args.no_h60:
        del s
        torch.cuda.empty_cache()
        h60 = measure_precision_h60(args)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sec, cores = cpu_step_seconds(cfg, 2, 1)
        cpu = {"value": sypd(cfg.dt, sec), "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "2 full production steps after 1 warm-up, C++ port of the reference step (FP32, OpenMP); "
                         "%.2f s per step" % sec}
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded balanced state with the workload's perturbations)",
                "config": dict(workload_desc(cfg), parallelism="replicas" if world > 1 else "single GPU",
                               finite=finite),
                "roofline": roof, "step_roofline": step_roof, "cpu_baseline": cpu, "e2e": e2e,
                "plain_step": None if plain_ms is None else {
                    "ms_per_step": plain_ms, "value": sypd(cfg.dt, plain_ms / 1e3), "unit": UNIT,
                    "chosen_over_plain": plain_ms / ms,
                    "what": "same step through the individual hooks (remaining/implicit tendency, Jacobian, ldiv, "
                            "post-Newton correction, DSS) with unfused torch stage algebra"},
                "fp32_vs_fp64": prec, "fp64_step": fp64, "batching": batching, "adjoint": adjoint,
                "differentiation": differentiation, "precision_h60": h60, "held_suarez": held_suarez,
                "topography": topography, "moist_0m": moist, "config1": config1,
                "clocks": clk, "gpu_launches": LAUNCHES_PER_STEP * args.steps}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


def measure_batching(args):
    """Standalone columns of uneven height: 20,000 columns, z_elem ~ U{30..127}
    (seed 2), z_max 30 km uniform, FP32 storage, 2 Newton iterations per column
    (Jacobian build + block-tridiagonal solve each), dtgamma = gamma * 120 s.
    One persistent graph-captured launch (variant chosen by the autotuner) vs
    the plain form, one launch per height group."""
    import torch
    from gbdycore import columns as CB, config as C
    cfg = C.DycoreConfig(h_elem=1, z_elem=10, z_max=30000.0, z_stretch=False, ft=np.float32, dt=120.0)
    z = CB.batch_heights(args.batch_columns, 30, 127, seed=2)
    Yc, Yf = CB.batch_state(cfg, z, seed=2)
    B = CB.ColumnBatch(cfg, z)
    Uh = B.state(Yc, Yf)
    U = Uh.copy()
    dtg = 0.4358665215084590 * 120.0
    choice, tune_ms = B.autotune(U, Uh, dtg, 2, reps=3)
    stream = torch.cuda.current_stream()

    def timed(mode):
        U.assign_(Uh)
        B.solve(U, Uh, dtg, 2, mode, residual=False)   # warm-up (captures the graph)
        torch.cuda.synchronize()
        tot = 0.0
        for _ in range(args.batch_reps):
            U.assign_(Uh)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            B.solve(U, Uh, dtg, 2, mode, residual=False)
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / args.batch_reps

    ms = {m: timed(m) for m in ("graph", "persistent", "per_height")}
    U.assign_(Uh)
    rn = B.solve(U, Uh, dtg, 2, "graph", residual=True)
    C_tot = int(z.sum())
    # compulsory traffic: read U^ and the initial iterate (4 centre + 1 face fields each), write the iterate
    nbytes = 4 * (3 * (4 * C_tot + C_tot + len(z)))
    return {"columns": int(len(z)), "z_elem": "U{30..127}, seed 2", "distinct_heights": int(len(np.unique(z))),
            "newton_iters": 2, "centres": C_tot,
            "ms": ms, "columns_per_s": len(z) / (ms["graph"] * 1e-3),
            "persistent_graph_over_per_height": ms["per_height"] / ms["graph"],
            "launches": {"graph": 3, "per_height": int(len(np.unique(z))) + 1},
            "autotune": {"choice": int(choice), "variant_ms": [float(x) for x in tune_ms],
                         "variants": ["128 thr/4 CTAs, 4 levels/lane", "128/4, 2 levels/lane (<=64 faces)",
                                      "128/6, 2 levels/lane", "256/2, 2 levels/lane", "64/8, 2 levels/lane"]},
            "GBps": nbytes / (ms["graph"] * 1e-3) / 1e9,
            "residual_sq_fp64": rn.tolist()}


def field_errors(a, b):
    """FP32 (a) against FP64 (b) per prognostic field: max-norm and RMS relative errors."""
    names = ["rho", "u_1", "u_2", "rho_e_tot"]
    out, rms = {}, {}
    for c in range(4):
        d = a[0][:, c].astype(np.float64) - b[0][:, c]
        out[names[c]] = float(np.abs(d).max() / np.abs(b[0][:, c]).max())
        rms[names[c]] = float(np.sqrt(np.mean(d * d) / np.mean(b[0][:, c] ** 2)))
    d = a[1].astype(np.float64) - b[1]
    out["u_3"] = float(np.abs(d).max() / max(np.abs(b[1]).max(), 1e-300))
    rms["u_3"] = float(np.sqrt(np.mean(d * d) / max(np.mean(b[1] ** 2), 1e-300)))
    out["rms"] = rms
    out["norm"] = "max |FP32 - FP64| / max |FP64| per field; rms: |FP32 - FP64|_2 / |FP64|_2"
    return out


def _timed(fn):
    import torch
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    st = torch.cuda.current_stream()
    e0.record(st)
    out = fn()
    e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), out


def _rhoe_loss(target):
    """J = 1/2 |rho e_tot - target|^2 over the stored centre nodes and its gradient."""
    def lg(YN):
        d = YN.c[:, 3] - target
        G = YN.similar()
        G.c[:, 3] = d
        return 0.5 * float((d.double() * d.double()).sum().item()), G
    return lg


def measure_adjoint(args, s, fwd_ms):
    """Reverse-mode cost on the production workload (h_elem=30, z_elem=63, FP32):
    gradient of 1/2 |rho e_tot(t_n) - target|^2 over n steps with a checkpoint
    every 5 steps; the pullback recomputes each segment (one forward step per
    step) and runs the reverse kernels."""
    import torch
    from gbdycore import simulation as sim
    n = args.adjoint_steps
    Y0 = s.Y.copy()
    target = Y0.c[:, 3] * 1.001
    lg = _rhoe_loss(target)
    sim.gradient(s.p, Y0, n, lg, checkpoint_every=5)          # warm-up: allocates the reverse buffers, records, checkpoints
    Y = Y0.copy()
    f_ms, _ = _timed(lambda: s.p.call("gb_adjoint_forward", Y.gb(), 0.0, float(s.dt), n, 5))
    J, Ybar = lg(Y)
    import ctypes
    d = (ctypes.c_double * 2)()
    peak = ctypes.c_size_t(0)
    if args.profile_region == "reverse":
        torch.cuda.profiler.start()
    r_ms, _ = _timed(lambda: s.p.call("gb_adjoint_reverse", Ybar.gb(), d, ctypes.byref(peak)))
    if args.profile_region == "reverse":
        torch.cuda.profiler.stop()
    finite = bool(torch.isfinite(Ybar.c).all() and torch.isfinite(Ybar.f).all())
    # the pullback alone: one segment of 5 steps, recorded by the checkpointed forward
    # pass, so the reverse pass recomputes nothing
    Y1 = Y0.copy()
    s.p.call("gb_adjoint_forward", Y1.gb(), 0.0, float(s.dt), 5, 5)
    _, Ybar1 = lg(Y1)
    d1 = (ctypes.c_double * 2)()
    p_ms, _ = _timed(lambda: s.p.call("gb_adjoint_reverse", Ybar1.gb(), d1, None))
    # the same reverse pass with the stage data of both segments kept by the forward half
    # (gb_adjoint_set_record_segments(ctx, 2)): no recompute, the same gradient
    s.p.call("gb_adjoint_set_record_segments", 2)
    Y2 = Y0.copy()
    s.p.call("gb_adjoint_forward", Y2.gb(), 0.0, float(s.dt), n, 5)
    _, Ybar2 = lg(Y2)
    d2 = (ctypes.c_double * 2)()
    r2_ms, _ = _timed(lambda: s.p.call("gb_adjoint_reverse", Ybar2.gb(), d2, None))
    same = bool(torch.equal(Ybar2.c, Ybar.c) and torch.equal(Ybar2.f, Ybar.f))
    s.p.call("gb_adjoint_set_record_segments", 1)
    # per-kernel times of the reverse kernels (CUDA events inside the library)
    kern = {}
    for kid, name, per_step in REVERSE_KERNELS:
        out = ctypes.c_double()
        s.p.call("gb_time_kernel", kid, s.Y.gb(), 20, ctypes.byref(out))
        kern[name] = {"ms": out.value, "launches_per_step": per_step}
    return {"steps": n, "checkpoint_every": 5, "forward_ms_per_step": fwd_ms, "kernels": kern,
            "pullback_ms_per_step": p_ms / 5, "pullback_over_forward": (p_ms / 5) / fwd_ms,
            "checkpointed_forward_ms_per_step": f_ms / n, "reverse_ms_per_step": r_ms / n,
            "adjoint_over_forward": (r_ms / n) / fwd_ms,
            "what": "reverse = per-segment recompute (1 forward step per step, stage data kept; the last "
                    "segment is recorded by the checkpointed forward pass) + reverse kernels; ratio against "
                    "the graph-replayed forward step",
            "dJ_dnu": d[0], "dJ_drate": d[1], "library_bytes": int(peak.value), "finite": finite,
            "segments_kept_2": {"reverse_ms_per_step": r2_ms / n, "adjoint_over_forward": (r2_ms / n) / fwd_ms,
                                "same_gradient_bitwise": same}}


def max_horizontal_wind(s):
    """max |u_h| (m/s) from the covariant components: |u|^2 = g^ij u_i u_j / r^2 (deep atmosphere)."""
    import torch
    g = s.geometry
    gup = torch.as_tensor(g.gup, dtype=torch.float64, device=s.Y.c.device)        # (Nh, 16, 3)
    r2 = torch.as_tensor(((g.R + g.zc) / g.R) ** 2, dtype=torch.float64, device=s.Y.c.device)
    u1 = s.Y.c[:, 1].double()                                                        # (Nh, 16, Nv)
    u2 = s.Y.c[:, 2].double()
    q = (gup[..., 0:1] * u1 * u1 + 2 * gup[..., 1:2] * u1 * u2 + gup[..., 2:3] * u2 * u2) / r2
    return float(q.clamp_min(0).sqrt().max().item())


def measure_config1(args, with_cpu):
    """The reference's CPU-runnable case (h_elem=6, z_elem=10 uniform to 30 km, dt=400 s, FP32):
    its steps graph-replayed on the GPU (the 0.7 MB state stays in L2: launch- and latency-bound)
    and, as this case's CPU baseline, the C++ port of the same steps on the host cores."""
    import torch
    from gbdycore import config as C, simulation as sim
    cfg = C.plain_h6()
    s = sim.AtmosSimulation(cfg, workload="plain")
    s.step(3)
    torch.cuda.synchronize()
    n, reps = 10, 20
    ms, _ = _timed(lambda: [s.step(n) for _ in range(reps)])
    ms /= n * reps
    out = {"workload": "h_elem=6, z_elem=10 uniform to 30 km, dt=400 s, FP32, %d-step runs" % n,
           "ms_per_step": ms, "value": sypd(cfg.dt, ms / 1e3), "unit": UNIT,
           "finite": bool(torch.isfinite(s.Y.c).all() and torch.isfinite(s.Y.f).all())}
    if with_cpu:
        from geometry import OracleGeometry
        import oracle as O
        from gbdycore import setups as S
        g = OracleGeometry(cfg.h_elem, cfg.z_elem, cfg.z_max, cfg.z_stretch, cfg.dz_bottom)
        Yc, Yf = S.workload_state(g, cfg, "plain")
        o = O.Oracle(g, cfg.oracle_params(), np.float32)
        Yc, Yf = Yc.astype(np.float32), Yf.astype(np.float32)
        o.step(Yc, Yf, cfg.dt, 1)
        t0 = time.perf_counter()
        o.step(Yc, Yf, cfg.dt, n)
        sec = (time.perf_counter() - t0) / n
        out["cpu_baseline"] = {"value": sypd(cfg.dt, sec), "unit": UNIT, "ms_per_step": sec * 1e3,
                               "cores": O.max_threads(), "kind": "port",
                               "sample": "%d steps after 1 warm-up, C++ port of the reference step (FP32, OpenMP)" % n}
    return out


def measure_held_suarez(args, fwd_ms):
    """The production step with the Held-Suarez forcing in the explicit tendency
    (rad: held_suarez): SYPD, the cost over the plain dry step, and the state
    after the timed steps (finite, mass conserved)."""
    import torch
    from gbdycore import config as C, simulation as sim
    cfg = C.production_h30().with_(held_suarez=True)
    s = sim.AtmosSimulation(cfg, workload="production")
    m0 = s.p.global_sums(s.Y)[0]
    s.step(3)
    torch.cuda.synchronize()
    n = args.held_suarez_steps
    ms, _ = _timed(lambda: s.step(n))
    ms /= n
    m1 = s.p.global_sums(s.Y)[0]
    finite = bool(torch.isfinite(s.Y.c).all() and torch.isfinite(s.Y.f).all())
    out = {"steps": n + 3, "ms_per_step": ms, "value": sypd(cfg.dt, ms / 1e3), "unit": UNIT,
           "over_dry_step": ms / fwd_ms, "mass_rel_change": abs(m1 - m0) / abs(m0), "finite": finite,
           "parameters": dict(cfg.hs)}
    # a longer forced run: the model stays finite and conserves mass while it spins up
    if args.held_suarez_long > 0:
        e1 = s.p.global_sums(s.Y)[1]
        k = args.held_suarez_long
        s.step(k)
        torch.cuda.synchronize()
        m2, e2 = s.p.global_sums(s.Y)
        out["long_run"] = {
            "steps": k, "simulated_days": k * cfg.dt / 86400.0,
            "finite": bool(torch.isfinite(s.Y.c).all() and torch.isfinite(s.Y.f).all()),
            "mass_rel_change": abs(m2 - m0) / abs(m0), "energy_rel_change": abs(e2 - e1) / abs(e1),
            "max_wind_m_s": max_horizontal_wind(s)}
    del s
    torch.cuda.empty_cache()
    return out


def measure_topography(args, fwd_ms):
    """The production step over terrain-following levels: the DCMIP-2-0-0 mountain (2 km)
    under the linear warp, FP32: SYPD, the cost over the flat step, the terrain kernels'
    times and achieved bandwidth of their algorithmic bytes (those of the flat kernels plus the
    four terrain rows of each element), mass conservation, and the FP32 state against the FP64
    library after the timed steps."""
    import ctypes
    import torch
    from gbdycore import config as C, simulation as sim
    from gbdycore import setups as S
    base = C.production_h30()
    g = sim.Geometry(base)
    lat = np.degrees(np.arctan2(g.xyz[..., 2], np.hypot(g.xyz[..., 0], g.xyz[..., 1])))
    lon = np.degrees(np.arctan2(g.xyz[..., 1], g.xyz[..., 0])) % 360.0
    zs = dcmip200_surface(lat, lon)
    cfg = base.with_(z_surface=zs, warp="linear")
    s = sim.AtmosSimulation(cfg, workload="production")
    m0 = s.p.global_sums(s.Y)[0]
    s.step(3)
    torch.cuda.synchronize()
    n = args.topography_steps
    ms, _ = _timed(lambda: s.step(n))
    ms /= n
    if args.profile_region == "topography":
        torch.cuda.profiler.start()
        s.step(1)
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
    m1 = s.p.global_sums(s.Y)[0]
    kern = {}
    fb = 4
    extra = 6 * cfg.h_elem ** 2 * 4 * 16 * fb  # the TG_N terrain rows of every element
    for name, kid in (("k_topo_passA", 0), ("k_topo_passB", 1), ("k_col_stage_g (terrain)", 2)):
        t = ctypes.c_double()
        s.p.call("gb_time_kernel", kid, s.Y.gb(), 20, ctypes.byref(t))
        b = algorithmic_bytes(cfg, kid) + (extra if kid < 2 else 0)
        kern[name] = {"ms": t.value, "algorithmic_bytes": b, "GBps": b / (t.value * 1e-3) / 1e9}
    finite = bool(torch.isfinite(s.Y.c).all() and torch.isfinite(s.Y.f).all())
    # FP32 against the FP64 library over the same terrain
    c64 = cfg.with_(ft=np.float64)
    Yc, Yf = S.workload_state(sim.Geometry(c64), c64, "production")
    s64 = sim.AtmosSimulation(c64, state=(Yc, Yf))
    s32 = sim.AtmosSimulation(cfg, state=(Yc.astype(np.float32), Yf.astype(np.float32)))
    k = args.precision_steps
    s64.step(k)
    s32.step(k)
    prec = {"steps": k}
    prec.update(field_errors(s32.Y.numpy(), s64.Y.numpy()))
    out = {"surface": "DCMIP-2-0-0 mountain (2 km peak on the equator at 270 E), linear warp",
           "steps": n + 3, "ms_per_step": ms, "value": sypd(cfg.dt, ms / 1e3), "unit": UNIT,
           "over_flat_step": ms / fwd_ms, "mass_rel_change": abs(m1 - m0) / abs(m0), "finite": finite,
           "kernels": kern, "fp32_vs_fp64": prec}
    del s, s64, s32
    torch.cuda.empty_cache()
    return out


def measure_moist(args):
    """Moist 0M column hooks on the production grid (h_elem 30, z_elem 63, FP32): one Newton
    iteration's hook calls (set_precomputed_quantities, implicit_tendency, update_jacobian, ldiv,
    correct_implicit_advection_tendency) with rho q_tot and the saturation adjustment, against the
    same calls of the dry context; per hook its CUDA-event time and the bandwidth of its
    algorithmic bytes (state in, tendency or solution out, Jacobian rows)."""
    import torch
    from gbdycore import config as C, simulation as sim
    from gbdycore import setups as S
    base = C.production_h30()
    out = {}
    for name, cfg in (("dry", base), ("moist", base.with_(moist=True))):
        g = sim.Geometry(cfg)
        if cfg.moist:
            Yc, Yf = S.moist_initial_state(g, cfg, seed=1, sigma=2.0)
        else:
            Yc, Yf = S.initial_state(g, cfg, seed=1, sigma=2.0)
        p = sim.AtmosCache(cfg)
        Y = sim.FieldVector.from_numpy(Yc, Yf)
        Y.f.normal_(0.0, 0.05)
        sim.set_precomputed_quantities(Y, p, 0.0)
        T, dY = Y.similar(), Y.similar()
        dtg = 0.4358665215084590 * cfg.dt
        nfc = Yc.shape[1]
        fb = 4
        Nh, Nv = g.Nh, cfg.z_elem
        S_b, F_b = Nh * 16 * Nv * fb, Nh * 16 * (Nv + 1) * fb
        nq = 19 if cfg.moist else 15
        calls = {
            "implicit_tendency": (lambda: sim.implicit_tendency(T, Y, p, 0.0), 2 * (nfc * S_b + F_b)),
            "update_jacobian": (lambda: sim.update_jacobian(sim.Jacobian(p), Y, p, dtg, 0.0), nfc * S_b + F_b + nq * F_b),
            "ldiv": (lambda: sim.ldiv(dY, sim.Jacobian(p), T), 2 * (nfc * S_b + F_b) + nq * F_b),
            "correct_implicit": (lambda: sim.correct_implicit_advection_tendency(dY, Y, p, 0.0), 2 * (nfc * S_b + F_b)),
        }
        res = {}
        reps = 20
        for k, (fn, b) in calls.items():
            fn()
            torch.cuda.synchronize()
            ms, _ = _timed(lambda: [fn() for _ in range(reps)])
            ms /= reps
            res[k] = {"ms": ms, "algorithmic_bytes": b, "GBps": b / (ms * 1e-3) / 1e9}
        res["newton_iteration_ms"] = sum(v["ms"] for v in res.values())
        res["finite"] = bool(torch.isfinite(T.c).all() and torch.isfinite(dY.c).all())
        out[name] = res
        del p, Y, T, dY
        torch.cuda.empty_cache()
    out["moist_over_dry"] = out["moist"]["newton_iteration_ms"] / out["dry"]["newton_iteration_ms"]
    # FP32 against FP64 (the library's own FP64 path) for the moist implicit tendency
    c64 = base.with_(moist=True, ft=np.float64)
    g64 = sim.Geometry(c64)
    Mc, Mf = S.moist_initial_state(g64, c64, seed=1, sigma=2.0, dtype=np.float64)
    Mf = np.random.default_rng(5).normal(0.0, 0.05, size=Mf.shape) * np.diff(
        np.concatenate([[g64.zf[0]], g64.zc, [g64.zf[-1]]]))[None, None, :]
    res = {}
    for ft in (np.float64, np.float32):
        cf = c64.with_(ft=ft)
        pf = sim.AtmosCache(cf)
        Yf_ = sim.FieldVector.from_numpy(Mc.astype(ft), Mf.astype(ft))
        Tf_ = Yf_.similar()
        sim.implicit_tendency(Tf_, Yf_, pf, 0.0)
        res[np.dtype(ft).name] = Tf_.numpy()
        del pf, Yf_, Tf_
    a, b = res["float32"], res["float64"]
    names = ["rho", "u_1", "u_2", "rho_e_tot", "rho_q_tot"]
    err = {n: float(np.abs(a[0][:, c] - b[0][:, c]).max() / max(np.abs(b[0][:, c]).max(), 1e-300))
           for c, n in enumerate(names) if np.abs(b[0][:, c]).max() > 0}
    err["u_3"] = float(np.abs(a[1] - b[1]).max() / np.abs(b[1]).max())
    out["implicit_tendency_fp32_vs_fp64"] = err
    out["what"] = ("h_elem 30, z_elem 63, FP32; q_tot = 0.018 exp(-z / 2.5 km): condensate below ~2 km and on "
                   "the mixed-phase levels; the saturation adjustment in every hook that forms the precomputed "
                   "quantities")
    return out


def dcmip200_surface(lat, lon):
    """The DCMIP-2-0-0 mountain (src/topography/topography.jl:186-205): a cosine bell of 2 km
    over a great-circle radius of 3 pi / 4 around (0 N, 270 E), modulated by cosine ridges of
    half-width pi / 16; latitude and longitude in degrees."""
    d2r = np.pi / 180.0
    r = np.arccos(np.clip(np.cos(lat * d2r) * np.cos((lon - 270.0) * d2r), -1.0, 1.0))
    R_m, zeta_m = 3 * np.pi / 4, np.pi / 16
    return np.where(r < R_m, 1000.0 * (1 + np.cos(np.pi * r / R_m)) * np.cos(np.pi * r / zeta_m) ** 2, 0.0)


def measure_differentiation(args):
    """Gradient of J = 1/2 |rho e_tot(t_end) - rho e_tot*|^2 over 8 steps (dt 200 s)
    on h_elem=16, z_elem=45 with a Rayleigh sponge of rate 1e-4 s^-1 above 20 km,
    with respect to the initial state, nu and the sponge rate; target = the run
    from a seed-3 perturbed state.  FP32 timing; FP64 gradient checked against
    central differences (relative step eps, FP64) in random directions."""
    import torch
    from gbdycore import config as C, setups as S, simulation as sim
    out = {}
    cfg32 = C.differentiation_h16()
    nsteps = 8
    for ft in (np.float32, np.float64):
        cfg = cfg32.with_(ft=ft)
        g = sim.Geometry(cfg)
        Yc, Yf = S.initial_state(g, cfg, seed=0, sigma=1.0, dtype=np.float64)
        Tc, Tf = S.initial_state(g, cfg, seed=3, sigma=1.0, dtype=np.float64)
        p = sim.AtmosCache(cfg)
        T = sim.FieldVector.from_numpy(Tc.astype(ft), Tf.astype(ft))
        p.call("gb_step", T.gb(), 0.0, float(cfg.dt), nsteps, 1)
        lg = _rhoe_loss(T.c[:, 3].clone())
        Y0 = sim.FieldVector.from_numpy(Yc.astype(ft), Yf.astype(ft))
        sim.gradient(p, Y0, nsteps, lg, checkpoint_every=4)  # warm-up: allocates the reverse buffers
        ms, (J, G, dnu, drate, peak) = _timed(lambda: sim.gradient(p, Y0, nsteps, lg, checkpoint_every=4))
        key = "fp32" if ft == np.float32 else "fp64"
        out[key] = {"gradient_ms": ms, "J": J, "dJ_dnu": dnu, "dJ_drate": drate, "library_bytes": peak}
        if ft == np.float32:
            # the two halves timed apart: the checkpointed forward (which records the last segment)
            # and the pullback (the adjoint proper: recompute of the earlier segment + reverse kernels)
            import ctypes
            d = (ctypes.c_double * 2)()
            pk = ctypes.c_size_t(0)
            Yh = Y0.copy()
            fwd_ms, _ = _timed(lambda: p.call("gb_adjoint_forward", Yh.gb(), 0.0, float(cfg.dt), nsteps, 4))
            _, Yb = lg(Yh)
            rev_ms, _ = _timed(lambda: p.call("gb_adjoint_reverse", Yb.gb(), d, ctypes.byref(pk)))
            out[key]["checkpointed_forward_ms"] = fwd_ms
            out[key]["reverse_ms"] = rev_ms
            # both segments' stage data kept by the forward half: the pullback recomputes nothing
            sim.gradient(p, Y0, nsteps, lg, checkpoint_every=4, record_segments=2)
            ms2, (_, G2, _, _, peak2) = _timed(lambda: sim.gradient(p, Y0, nsteps, lg, checkpoint_every=4))
            Yh = Y0.copy()
            p.call("gb_adjoint_forward", Yh.gb(), 0.0, float(cfg.dt), nsteps, 4)
            _, Yb = lg(Yh)
            rev2, _ = _timed(lambda: p.call("gb_adjoint_reverse", Yb.gb(), d, ctypes.byref(pk)))
            p.call("gb_adjoint_set_record_segments", 1)
            out[key]["two_segments_kept"] = {"gradient_ms": ms2, "reverse_ms": rev2, "library_bytes": peak2,
                                             "same_gradient": bool(torch.equal(G.c, G2.c) and torch.equal(G.f, G2.f))}
        if ft == np.float64:
            def fwd(Xc, Xf, q=p):
                Z = sim.FieldVector.from_numpy(Xc, Xf)
                q.call("gb_step", Z.gb(), 0.0, float(cfg.dt), nsteps, 0)
                return lg(Z)[0]
            rng = np.random.default_rng(3)
            errs = {1e-6: [], 1e-8: []}
            for k in range(args.fd_directions):
                dc = rng.standard_normal(Yc.shape)
                for c in range(4):
                    dc[:, c] *= np.sqrt(np.mean(Yc[:, c] ** 2))
                df = rng.standard_normal(Yf.shape) * max(np.sqrt(np.mean(Yf ** 2)), 1e-3 * np.sqrt(np.mean(Yc[:, 1] ** 2)))
                ad = float((G.c.cpu().numpy() * dc).sum() + (G.f.cpu().numpy() * df).sum())
                for eps in errs:
                    fd = (fwd(Yc + eps * dc, Yf + eps * df) - fwd(Yc - eps * dc, Yf - eps * df)) / (2 * eps)
                    errs[eps].append(abs(ad - fd) / abs(fd))
            par = {}
            for name, mk, val, scale in (("nu", lambda s_: cfg.with_(nu=cfg.nu * s_), dnu, cfg.nu),
                                         ("rate", lambda s_: cfg.with_(alpha_uh=1e-4 * s_, alpha_w=1e-4 * s_), drate, 1e-4)):
                vals = []
                for s_ in (1 + 1e-4, 1 - 1e-4):
                    q = sim.AtmosCache(mk(s_))
                    vals.append(fwd(Yc, Yf, q))
                fd = (vals[0] - vals[1]) / (2e-4 * scale)
                par[name] = {"adjoint": val, "fd": fd, "rel": abs(val - fd) / abs(fd)}
            out["fd_check_fp64"] = {
                "directions": args.fd_directions,
                "rel_err_eps_1e-6": {"median": float(np.median(errs[1e-6])), "max": float(np.max(errs[1e-6]))},
                "rel_err_eps_1e-8": {"median": float(np.median(errs[1e-8])), "max": float(np.max(errs[1e-8]))},
                "parameters_eps_1e-4": par,
                "note": "the van Leer limiter makes the 8-step map piecewise smooth: central differences "
                        "with eps = 1e-6 can straddle limiter branch switches; eps = 1e-8 shown beside it"}
        del p
    f32 = C.differentiation_h16()
    s32 = sim.AtmosSimulation(f32, state=S.initial_state(sim.Geometry(f32), f32, seed=0, sigma=1.0))
    s32.step(2)
    fms, _ = _timed(lambda: s32.step(nsteps))
    out["fp32"]["forward_ms"] = fms
    out["fp32"]["gradient_over_forward"] = out["fp32"]["gradient_ms"] / fms
    out["fp32"]["reverse_over_forward"] = out["fp32"]["reverse_ms"] / fms
    k2 = out["fp32"]["two_segments_kept"]
    k2["gradient_over_forward"] = k2["gradient_ms"] / fms
    k2["reverse_over_forward"] = k2["reverse_ms"] / fms
    out["workload"] = "h_elem=16, z_elem=45 stretched (dz_bottom 500 m), dt=200 s, 8 steps, sponge 1e-4 s^-1 above 20 km"
    return out


def measure_precision_h60(args):
    """h_elem=60 (21,600 elements), z_elem=63 stretched, dt=60 s: 20 FP32 steps
    against the FP64 run of the same library (per-field max error / max |FP64|),
    and the 20-step adjoint with a checkpoint every 5 steps (peak device memory)."""
    import ctypes
    import torch
    from gbdycore import config as C, setups as S, simulation as sim
    cfg = C.precision_h60()
    g = sim.Geometry(cfg)
    Yc, Yf = S.workload_state(g, cfg, "precision")
    out = {"workload": "h_elem=60, z_elem=63 tanh-stretched (dz_bottom 30 m), dt=60 s, 20 steps, seed 4"}
    s64 = sim.AtmosSimulation(cfg.with_(ft=np.float64), state=(Yc.astype(np.float64), Yf.astype(np.float64)))
    s64.step(20)
    a64 = s64.Y.numpy()
    sums64 = s64.p.global_sums(s64.Y)
    del s64
    torch.cuda.empty_cache()
    s32 = sim.AtmosSimulation(cfg, state=(Yc.astype(np.float32), Yf.astype(np.float32)))
    Y0 = s32.Y.copy()
    s32.step(20)                      # the same 20 steps as the FP64 run
    a32 = s32.Y.numpy()
    sums32 = s32.p.global_sums(s32.Y)
    ms, _ = _timed(lambda: s32.step(20))   # timing (graph already captured)
    err = field_errors(a32, a64)
    out.update({"fp32_ms_per_step": ms / 20, "fp32_vs_fp64_after_20_steps": err,
                "mass_energy_fp32_vs_fp64_rel": [float(abs(sums32[i] - sums64[i]) / abs(sums64[i])) for i in range(2)]})
    del a64
    target = Y0.c[:, 3] * 1.001
    lg = _rhoe_loss(target)
    torch.cuda.synchronize()
    free0, total = torch.cuda.mem_get_info()
    Y = Y0.copy()
    fwd_ms, _ = _timed(lambda: s32.p.call("gb_adjoint_forward", Y.gb(), 0.0, float(cfg.dt), 20, 5))
    J, Ybar = lg(Y)
    d = (ctypes.c_double * 2)()
    peak = ctypes.c_size_t(0)
    rev_ms, _ = _timed(lambda: s32.p.call("gb_adjoint_reverse", Ybar.gb(), d, ctypes.byref(peak)))
    free1, _ = torch.cuda.mem_get_info()
    out["adjoint_20_steps"] = {"checkpoint_every": 5, "record_segments": 1, "forward_ms": fwd_ms,
                               "forward_note": "first call: includes allocating the stage records and checkpoints",
                               "reverse_ms": rev_ms,
                               "reverse_over_forward_steps": rev_ms / (20 * ms / 20),
                               "library_bytes": int(peak.value),
                               "device_bytes_in_use_after_reverse": int(total - free1),
                               "finite": bool(torch.isfinite(Ybar.c).all() and torch.isfinite(Ybar.f).all())}
    # HBM for recomputation: the forward half keeps the stage data of the last K segments, so
    # the pullback recomputes 4 - K of the four (gb_adjoint_set_record_segments)
    for K, key in ((2, "adjoint_20_steps_two_segments_kept"), (3, "adjoint_20_steps_three_segments_kept")):
        s32.p.call("gb_adjoint_set_record_segments", K)
        Y = Y0.copy()
        s32.p.call("gb_adjoint_forward", Y.gb(), 0.0, float(cfg.dt), 20, 5)   # allocates the extra records
        J, Ybar2 = lg(Y)
        s32.p.call("gb_adjoint_reverse", Ybar2.gb(), d, ctypes.byref(peak))
        Y = Y0.copy()
        fwd2, _ = _timed(lambda: s32.p.call("gb_adjoint_forward", Y.gb(), 0.0, float(cfg.dt), 20, 5))
        J, Ybar2 = lg(Y)
        rev2, _ = _timed(lambda: s32.p.call("gb_adjoint_reverse", Ybar2.gb(), d, ctypes.byref(peak)))
        free2, _ = torch.cuda.mem_get_info()
        out[key] = {
            "checkpoint_every": 5, "record_segments": K, "forward_ms": fwd2, "reverse_ms": rev2,
            "reverse_over_forward_steps": rev2 / ms, "library_bytes": int(peak.value),
            "device_bytes_in_use_after_reverse": int(total - free2),
            "same_gradient_as_one_kept": bool(torch.equal(Ybar.c, Ybar2.c) and torch.equal(Ybar.f, Ybar2.f))}
    s32.p.call("gb_adjoint_set_record_segments", 1)
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())

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


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--plain-steps", type=int, default=3)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--precision-steps", type=int, default=20)
    ap.add_argument("--no-precision", action="store_true")
    ap.add_argument("--batch-columns", type=int, default=20000)
    ap.add_argument("--batch-reps", type=int, default=10)
    ap.add_argument("--no-batching", action="store_true")
    return ap.parse_args()


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
                "reasons": sorted(reasons), "samples": len(sm)}


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
    (1, "k_passB (explicit tendency)", 4),
    (2, "k_col_stage (implicit column solve)", 3),
    (3, "k_dss (direct stiffness summation)", 8),
    (4, "k_final (stage combination)", 1),
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
    }[kid]
    return words * fb


def contract_bytes_per_step(cfg, fb=4):
    Nh, Nv = 6 * cfg.h_elem ** 2, cfg.z_elem
    P = Nh * 16 * Nv
    S = 4 * P + Nh * 16 * (Nv + 1)
    return (51 * S + 56 * P) * fb


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
    if world > 1:
        dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    s.step(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    finite = bool(torch.isfinite(s.Y.c).all() and torch.isfinite(s.Y.f).all())
    v1 = sypd(cfg.dt, ms / 1e3)
    value = v1 * world        # independent replicas, one per GPU

    # per-kernel timing (CUDA events on the context stream, inside the library)
    peak, peak_kind = measured_peak()
    ktime = {}
    for kid, name, per_step in KERNELS:
        out = ctypes.c_double()
        s.p.call("gb_time_kernel", kid, s.Y.gb(), 20, ctypes.byref(out))
        ktime[kid] = out.value
    share = {kid: ktime[kid] * KERNELS[kid][2] for kid in ktime}
    dom = max(share, key=share.get)
    ach = algorithmic_bytes(cfg, dom) / (ktime[dom] * 1e-3) / 1e9
    roof = {"kernel": KERNELS[dom][1], "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
            "frac": ach / peak, "peak_kind": peak_kind, "traffic": None,
            "algorithmic_bytes_per_launch": algorithmic_bytes(cfg, dom), "ms_per_launch": ktime[dom],
            "kernels": {KERNELS[k][1]: {"ms": ktime[k], "launches_per_step": KERNELS[k][2],
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
        names = ["rho", "u_1", "u_2", "rho_e_tot"]
        prec = {"steps": n}
        for c in range(4):
            prec[names[c]] = float(np.abs(a[0][:, c] - b[0][:, c]).max() / np.abs(b[0][:, c]).max())
        prec["u_3"] = float(np.abs(a[1] - b[1]).max() / max(np.abs(b[1]).max(), 1e-300))
        prec["norm"] = "max |FP32 - FP64| / max |FP64| per field"
        del s64, s32

    batching = None
    if not args.no_batching:
        batching = measure_batching(args)

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
                "fp32_vs_fp64": prec, "batching": batching,
                "clocks": clk, "gpu_launches": 20 * args.steps}
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


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_gb300(args)


if __name__ == "__main__":
    sys.exit(main())

"""Precision study (test infrastructure, beside the oracle it runs): FP32 against FP64 on the CPU oracle (correctly rounded libm, the reference's formulation)
after n steps of the production workload (h_elem=30, z_elem=63, dt=120 s): the FP32 error
floor of the formulation itself, to set beside the GPU's (bench.py `fp32_vs_fp64`).  The
oracle's precision-study builds run in child processes (the library is loaded once per
process): ``--store32`` (ORACLE_VARIANT=store32) is FP64 arithmetic with every stored field
rounded to FP32, which separates the error of FP32 storage from that of FP32 arithmetic;
``--phid`` (ORACLE_VARIANT=phid) is FP32 with g z - Phi_r formed as a deviation from
per-level reference values.  Every run starts from the FP32-representable initial state.

    python oracle/precision_study.py [n_steps] [--store32] [--phid]   (~1 minute per run of 2 steps on 8 cores)
"""
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [os.path.join(ROOT, "climaatmos.jl_gb300"), HERE, os.path.join(ROOT, "tests")]

import numpy as np  # noqa: E402

from gbdycore import config as C, setups as S  # noqa: E402
from helpers import field_errors, make_oracle, oracle_geometry  # noqa: E402


def _start():
    cfg = C.production_h30()
    g = oracle_geometry(cfg.with_(ft=np.float64))
    Yc, Yf = S.workload_state(g, cfg.with_(ft=np.float64), "production")
    return cfg, Yc.astype(np.float32).astype(np.float64), Yf.astype(np.float32).astype(np.float64)


def run(dtype, n):
    cfg, Yc, Yf = _start()
    o = make_oracle(cfg, dtype, dss_stage1=False)
    a = (Yc.astype(dtype), Yf.astype(dtype))
    o.step(a[0], a[1], cfg.dt, n)
    return a[0].astype(np.float64), a[1].astype(np.float64)


def _child(variant, dtype, n):
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "run.npz")
        env = dict(os.environ, ORACLE_VARIANT=variant)
        subprocess.check_call([sys.executable, os.path.abspath(__file__), str(n), "--emit", out, dtype], env=env)
        z = np.load(out)
        return z["c"], z["f"]


def main(n=20, store32=False, phid=False):
    ref = run(np.float64, n)
    e = field_errors(*run(np.float32, n), *ref)
    print("oracle FP32 vs FP64 after %d steps (max-norm relative): %s" % (n, {k: float(v) for k, v in e.items()}))
    if store32:
        e = field_errors(*_child("store32", "float64", n), *ref)
        print("oracle FP64 arithmetic with FP32 storage vs FP64 after %d steps: %s"
              % (n, {k: float(v) for k, v in e.items()}))
    if phid:
        e = field_errors(*_child("phid", "float32", n), *ref)
        print("oracle FP32 with g z - Phi_r as a deviation vs FP64 after %d steps: %s"
              % (n, {k: float(v) for k, v in e.items()}))


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    n = int(args[0]) if args else 20
    if "--emit" in sys.argv:
        i = sys.argv.index("--emit")
        c, f = run(np.dtype(sys.argv[i + 2]).type, n)
        np.savez(sys.argv[i + 1], c=c, f=f)
    else:
        main(n, "--store32" in sys.argv, "--phid" in sys.argv)

"""FP32 against FP64 on the CPU oracle (correctly rounded libm, the reference's formulation)
after n steps of the production workload (h_elem=30, z_elem=63, dt=120 s): the FP32 error
floor of the formulation itself, to set beside the GPU's (bench.py `fp32_vs_fp64`).

    python tests/precision_oracle.py [n_steps]      (~2 minutes for 20 steps on 8 cores)
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [os.path.join(ROOT, "climaatmos.jl_gb300"), os.path.join(ROOT, "oracle"), HERE]

import numpy as np  # noqa: E402

from gbdycore import config as C, setups as S  # noqa: E402
from helpers import field_errors, make_oracle, oracle_geometry  # noqa: E402


def main(n=20):
    cfg = C.production_h30()
    g = oracle_geometry(cfg.with_(ft=np.float64))
    Yc, Yf = S.workload_state(g, cfg.with_(ft=np.float64), "production")
    o64 = make_oracle(cfg, np.float64, dss_stage1=False)
    o32 = make_oracle(cfg, np.float32, dss_stage1=False)
    a = (Yc.copy(), Yf.copy())
    b = (Yc.astype(np.float32), Yf.astype(np.float32))
    o64.step(a[0], a[1], cfg.dt, n)
    o32.step(b[0], b[1], cfg.dt, n)
    e = field_errors(b[0].astype(np.float64), b[1].astype(np.float64), a[0], a[1])
    print("oracle FP32 vs FP64 after %d steps (max-norm relative): %s" % (n, {k: float(v) for k, v in e.items()}))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 20)

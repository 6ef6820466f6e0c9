"""The multi-process form (replicas only) on CPU ranks over gloo, world size 2.

Each rank runs its own replica of the seeded small workload on the CPU oracle
(one ARS343 step); the replicas agree bitwise, the timing bookkeeping takes the
maximum over ranks, and the whole-job value is world x the per-replica rate.
The reference arm runs on rank 0 only.
"""
import os
import socket
import sys

import numpy as np
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    sys.path[:0] = [os.path.join(ROOT, "climaatmos.jl_gb300"), os.path.join(ROOT, "oracle"), HERE, ROOT]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist
    from gbdycore import replicas as rep
    from helpers import make_oracle, perturbed_state, small_config
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cfg = small_config(np.float64, h_elem=2, z_elem=6)
        Yc, Yf = perturbed_state(cfg)
        o = make_oracle(cfg, np.float64, dss_stage1=False)
        o.step(Yc, Yf, cfg.dt, 1)
        mine = torch.tensor([float(np.abs(Yc).sum() + np.abs(Yf).sum()), float(Yc.reshape(-1)[123])],
                            dtype=torch.float64)
        allv = [torch.zeros_like(mine) for _ in range(world)]
        dist.all_gather(allv, mine)
        ms = rep.max_over_ranks(1.0 + rank)
        rep.barrier()
        import bench
        rc = bench.run_reference(bench.parse(["--impl", "reference", "--steps", "1", "--warmup", "0"])) \
            if rank != 0 else 0
        out[rank] = (float(allv[0][0]), float(allv[1][0]), float(allv[0][1]), float(allv[1][1]), ms,
                     rep.job_value(2.5), rc)
    finally:
        dist.destroy_process_group()


def test_two_cpu_replicas_over_gloo():
    world = 2
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(world, _free_port(), out), nprocs=world, join=True, start_method="spawn")
    for r in range(world):
        s0, s1, p0, p1, ms, val, rc = out[r]
        assert s0 == s1 and p0 == p1          # the replicas agree bitwise
        assert ms == 2.0                      # the slower rank's time
        assert val == 5.0                     # world x the per-replica rate
        assert rc == 0                        # the reference arm: rank 1 exits without work

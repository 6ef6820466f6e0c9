"""Multi-GPU form of the step: independent replicas, one per rank.

The step shards by elements (DSS halos, global sums), but every run here has one
GPU per box, so the multi-process form is replicas only: each rank advances its
own copy of the workload, with no collective on the data path.  What crosses
ranks is bookkeeping: a barrier around the timed region and the maximum step
time over ranks; the whole-job value is world x the per-replica rate.
"""
import torch
import torch.distributed as dist


def world():
    return dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1


def max_over_ranks(ms, device=None):
    """The largest of the ranks' step times (ms); ms itself on one rank."""
    if world() == 1:
        return float(ms)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier():
    if world() > 1:
        dist.barrier()


def job_value(per_replica_rate, n=None):
    """Whole-job throughput of n (default: world) independent replicas."""
    return per_replica_rate * (world() if n is None else n)

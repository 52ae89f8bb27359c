"""Multi-GPU runs of the path: independent replicas, one process per GPU.

Tiled Cholesky of one matrix would shard as a 2-D block-cyclic tile
distribution with a panel broadcast per step; this build runs on one GPU per
process, so N GPUs run N independent factor-and-solve replicas (each rank
its own seeded system) with no data-path collective.  The only collectives
are the host-side aggregation of the benchmark: the barrier around the timed
region, the slowest rank's time (MAX) and the total work (SUM).
"""
from __future__ import annotations

import os

import torch
import torch.distributed as dist


def world():
    return int(os.environ.get("WORLD_SIZE", "1"))


def rank():
    return int(os.environ.get("RANK", "0"))


def _tensor(v):
    dev = "cuda" if dist.is_initialized() and dist.get_backend() == "nccl" else "cpu"
    return torch.tensor([float(v)], dtype=torch.float64, device=dev)


def max_over_ranks(v: float) -> float:
    if not (dist.is_initialized() and dist.get_world_size() > 1):
        return float(v)
    t = _tensor(v)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(v: float) -> float:
    if not (dist.is_initialized() and dist.get_world_size() > 1):
        return float(v)
    t = _tensor(v)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def barrier():
    if torch.cuda.is_available():
        torch.cuda.synchronize()
    if dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()
        if torch.cuda.is_available():
            torch.cuda.synchronize()

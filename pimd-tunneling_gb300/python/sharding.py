"""Multi-GPU layout of a TI batch: independent rings, no per-step exchange.

The (trajectory x lambda) rings are independent (pimd_par.f90 sends each MPI
rank its tasks once, pimd_par.f90:282-308, and gathers one integrand per task,
:389).  Here each rank takes a contiguous block of rings balanced by its bead
count, propagates it on its own GPU, and the only collective is one all-reduce
of the per-lambda (sum, sum of squares, count) triples at the end.
"""
import numpy as np


def shard_rings(beads_per_ring, world_size, rank):
    """Contiguous [start, stop) block of rings for `rank`, balanced by sum of P."""
    w = np.asarray(beads_per_ring, dtype=np.float64)
    cum = np.concatenate([[0.0], np.cumsum(w)])
    total = cum[-1]
    bounds = [int(np.searchsorted(cum, total * r / world_size, side="left")) for r in range(world_size + 1)]
    bounds[0], bounds[-1] = 0, len(w)
    for r in range(1, world_size + 1):
        bounds[r] = max(bounds[r], bounds[r - 1])
    return bounds[rank], bounds[rank + 1]


def lambda_partials(integrands, ring_lambda, nlambda):
    """Per-lambda (sum, sum of squares, count) of this rank's ring integrands."""
    out = np.zeros((nlambda, 3))
    for v, l in zip(integrands, ring_lambda):
        out[l, 0] += v
        out[l, 1] += v * v
        out[l, 2] += 1.0
    return out


def allreduce_partials(partials, group=None):
    """Sum the (sum, sumsq, count) triples over ranks (one small all-reduce)."""
    import torch
    import torch.distributed as dist
    t = torch.from_numpy(np.ascontiguousarray(partials, dtype=np.float64))
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        if dist.get_backend(group) == "nccl":
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy()


def mean_var(partials):
    """pimd_par.f90:401-409: mean and E[I^2] - E[I]^2 per lambda point."""
    s, s2, n = partials[:, 0], partials[:, 1], partials[:, 2]
    mean = np.where(n > 0, s / np.maximum(n, 1), 0.0)
    var = np.where(n > 0, s2 / np.maximum(n, 1) - mean * mean, 0.0)
    return mean, var

"""Multi-GPU layout of a TI batch: independent rings, no per-step exchange.

The (trajectory x lambda) rings are independent (pimd_par.f90 sends each MPI
rank its tasks once, pimd_par.f90:282-308, and gathers one integrand per task,
:389).  Here each rank takes a contiguous block of rings balanced by its bead
count, propagates it on its own GPU, and the only exchange is one gather of
the per-lambda (sum, sum of squares, count) triples at the end, through the
caller's own communicator.
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


def combine_partials(partials, allgather=None):
    """Sum the (sum, sum of squares, count) triples over ranks: the one exchange
    of the run, replacing pimd_par's MPI_Gather of the integrands (:389).
    allgather is the caller's communicator: a callable that takes this rank's
    array and returns the list of every rank's array in rank order (mpi4py's
    comm.allgather, or a wrapper of the caller's torch.distributed group); None
    for a single rank.  The sum runs in rank order, so every rank gets the same
    bits."""
    p = np.ascontiguousarray(partials, dtype=np.float64)
    if allgather is None:
        return p.copy()
    parts = [np.asarray(a, dtype=np.float64).reshape(p.shape) for a in allgather(p)]
    tot = np.zeros_like(p)
    for a in parts:
        tot += a
    return tot


def mean_var(partials):
    """pimd_par.f90:401-409: mean and E[I^2] - E[I]^2 per lambda point."""
    s, s2, n = partials[:, 0], partials[:, 1], partials[:, 2]
    mean = np.where(n > 0, s / np.maximum(n, 1), 0.0)
    var = np.where(n > 0, s2 / np.maximum(n, 1) - mean * mean, 0.0)
    return mean, var

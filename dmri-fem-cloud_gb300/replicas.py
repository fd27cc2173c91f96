"""Several GPUs: independent replicas, no data-path collective.

Every signal (mesh x direction x b x sequence) is an independent Crank-Nicolson
integration that shares only read-only matrices, so a multi-GPU run splits the
signal list into contiguous, mesh-major blocks, one per rank, and each rank
integrates its block on its own GPU.  The only communication is on the host
side after the solves: the max of the ranks' timings and one gather of the
signals on rank 0.  The reference's MPI strategy (one mesh partitioned across
ranks, DmriFemLib.py:626-637 bounding-box all-reduce, collective assembly and
Krylov solves) is not used: it needs a halo exchange per SpMV.

These helpers take a ``torch.distributed`` process group (nccl on GPUs, gloo on
the CPU) or run single-process when none is initialised.
"""

import numpy as np


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def world():
    d = _dist()
    return (d.get_rank(), d.get_world_size()) if d else (0, 1)


def shard(n_signals, rank, world_size, mesh_of=None):
    """Indices of the signals rank ``rank`` integrates: contiguous blocks of the
    list sorted by mesh (stable), sizes differing by at most one, so each rank
    uploads as few meshes as possible."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError("bad rank %d / world size %d" % (rank, world_size))
    order = np.arange(n_signals) if mesh_of is None else np.argsort(np.asarray(mesh_of), kind="stable")
    base, extra = divmod(n_signals, world_size)
    lo = rank * base + min(rank, extra)
    hi = lo + base + (1 if rank < extra else 0)
    return order[lo:hi]


def max_over_ranks(value, device="cpu"):
    """The largest value over all ranks (the step time a multi-GPU run reports)."""
    d = _dist()
    if d is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def gather_signals(indices, values, n_signals, device="cpu"):
    """Place every rank's ``values`` (one row per signal index) into one
    (n_signals, ...) array on rank 0 (other ranks get None).  Indices must
    cover 0..n_signals-1 exactly once across the ranks."""
    indices = np.asarray(indices, np.int64)
    values = np.asarray(values, np.float64).reshape(len(indices), -1)
    d = _dist()
    if d is None:
        parts = [(indices, values)]
    else:
        parts = [None] * d.get_world_size()
        d.all_gather_object(parts, (indices, values))
        if d.get_rank() != 0:
            return None
    width = max((v.shape[1] for _, v in parts if len(v)), default=1)
    out = np.full((n_signals, width), np.nan)
    seen = np.zeros(n_signals, bool)
    for idx, v in parts:
        if np.any(seen[idx]):
            raise ValueError("a signal index was integrated by two ranks")
        seen[idx] = True
        out[idx] = v
    if not seen.all():
        raise ValueError("signals %s were integrated by no rank" % np.flatnonzero(~seen)[:8].tolist())
    return out

"""Replica decomposition across ranks: disjoint particle ranges, integer tallies summed on the host.

The GB300 equivalent of the reference's MPI layer (input broadcast, per-rank run,
state gather and sum to rank 0; src/MolflowCLI.cpp:76-101,165-196): every rank traces
the particle ids [rank * stride, ...) with the same seed, and the GlobalSimuState-shaped
tallies are added across ranks.  The integer fields (hit, desorption and absorption counts,
angle-map cells) are summed as 64-bit integers, so their sum does not depend on the order of
the ranks.  The float64 fields (velocity sums, texture and profile sums, direction vectors) are
summed as doubles: their sum can differ in the last bits with the reduction order.
"""
import numpy as np

RANK_STRIDE = 1 << 48


def rank_particle_offset(rank, stride=RANK_STRIDE):
    return int(rank) * int(stride)


def reduce_state(state, group=None, dst=None):
    """Sum a SimuState over all ranks of the torch.distributed group (in place).
    With dst set, only that rank is guaranteed to hold the sum (reduce), else all (all_reduce)."""
    import torch
    import torch.distributed as dist
    # NCCL reduces device tensors only: stage each array through this rank's GPU
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" else torch.device("cpu")
    for name in ("global_", "facet_counts", "facet_sums", "texture", "profile", "direction", "anglemap"):
        arr = getattr(state, name)
        if arr.size == 0:
            continue
        if arr.dtype == np.uint64:
            t = torch.from_numpy(arr.view(np.int64).copy()).to(dev)
        else:
            t = torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64).copy()).to(dev)
        if dst is None:
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        else:
            dist.reduce(t, dst=dst, op=dist.ReduceOp.SUM, group=group)
        out = t.cpu().numpy()
        if arr.dtype == np.uint64:
            arr[...] = out.view(np.uint64)
        else:
            arr[...] = out
    return state

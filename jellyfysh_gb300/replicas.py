"""Replicas over several GPUs: one process per GPU, independent chains on each, no collective on the data path.

Chains are independent Markov chains, so a batch splits across ranks with no exchange step; the only collectives
are the host-side reductions of the results (events and the max-over-ranks time of a timed region, estimator
histograms and counters).  ``shard`` gives each rank a contiguous block of chains balanced by work (units x
events), and the reductions run on any ``torch.distributed`` backend (NCCL on GPUs, gloo on the CPU).
"""
from typing import Sequence, Tuple

import numpy as np


def shard(work: Sequence[float], world: int, rank: int) -> Tuple[int, int]:
    """[first, last) of the chains of `rank`: contiguous blocks with about equal summed work (e.g. N x events per
    chain); every chain belongs to exactly one rank."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a world of %d" % (rank, world))
    w = np.asarray(work, dtype=np.float64)
    if len(w) == 0:
        return 0, 0
    cumulative = np.concatenate([[0.0], np.cumsum(w)])
    total = cumulative[-1]
    # the block boundaries: the first chain whose preceding work reaches rank / world of the total
    bounds = [int(np.searchsorted(cumulative[:-1], total * r / world, side="left")) for r in range(world)]
    bounds = [0] + bounds[1:] + [len(w)]
    for r in range(1, world + 1):  # keep the blocks ordered (ties of zero work)
        bounds[r] = max(bounds[r], bounds[r - 1])
    return bounds[rank], bounds[rank + 1]


def timed_throughput(events: float, elapsed_ms: float, device=None) -> Tuple[float, float, float]:
    """Whole-job (events summed over ranks, elapsed time maximal over ranks, events per second) of a timed region
    that every rank ran; a single process returns its own figures."""
    import torch
    import torch.distributed as dist
    values = torch.tensor([float(events), float(elapsed_ms)], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        total = values[:1].clone()
        longest = values[1:].clone()
        dist.all_reduce(total, op=dist.ReduceOp.SUM)
        dist.all_reduce(longest, op=dist.ReduceOp.MAX)
        values = torch.cat([total, longest])
    events_all, ms = float(values[0]), float(values[1])
    return events_all, ms, events_all / (ms / 1000.0) if ms > 0 else float("inf")


def sum_over_ranks(array: np.ndarray, device=None) -> np.ndarray:
    """Elementwise sum of a host array (histograms, counters) over all ranks."""
    import torch
    import torch.distributed as dist
    tensor = torch.from_numpy(np.ascontiguousarray(array, dtype=np.float64)).to(device if device else "cpu")
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(tensor, op=dist.ReduceOp.SUM)
    return tensor.cpu().numpy()

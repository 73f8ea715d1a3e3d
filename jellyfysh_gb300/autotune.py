"""Launch-shape autotuner of the mixed-precision event rounds.

A round is two launches (FP32 screen with one warp per chain; the settle kernel's FP64 re-solves and commits); their
shape is the number of warps per screening block and the number of chain groups on streams of their own.  The best shape depends on the
batch (number of chains, their N and neighbourhood sizes, the far field): ``tune`` times every candidate shape on the
batch itself for a few event rounds and keeps the fastest.  The batch's device state is saved before and restored
after the timing, so tuning changes no chain: the results do not depend on the launch shape in any case (every shape
gives the same events bit for bit).

One warp screens one chain: a chain's event is one pass over its nearby cells (27 for one neighbour layer, 343 for
three) and 32 lanes cover it; several warps per chain would leave lanes idle and add a block-level merge.
"""
import time
from typing import Dict, Iterable, Tuple

WARPS = (1, 2, 4, 8)
GROUPS = (1, 2)


def tune(batch, events: int = 8, warps: Iterable[int] = WARPS, groups: Iterable[int] = GROUPS,
         repeats: int = 2) -> Tuple[Tuple[int, int], Dict[Tuple[int, int], float]]:
    """Time `events` event rounds of the mixed mode for every (warps per block, chain groups) and apply the fastest
    to `batch`.  Returns (best shape, seconds per round by shape)."""
    torch = batch._torch
    saved = [t.clone() for t in batch.state_tensors()]
    timings = {}
    try:
        for w in warps:
            for g in groups:
                batch.set_block_warps(w)
                batch.set_groups(g)
                batch.run(events, mode="mixed")  # captures the shape's graphs outside the timing
                best = float("inf")
                for _ in range(repeats):
                    torch.cuda.synchronize(batch.device)
                    start = time.perf_counter()
                    batch.run(events, mode="mixed", sync=False)
                    torch.cuda.synchronize(batch.device)
                    best = min(best, (time.perf_counter() - start) / events)
                timings[(w, g)] = best
    finally:
        for target, source in zip(batch.state_tensors(), saved):
            target.copy_(source)
        torch.cuda.synchronize(batch.device)
    shape = min(timings, key=timings.get)
    batch.set_block_warps(shape[0])
    batch.set_groups(shape[1])
    return shape, timings

"""Splitting independent trials over ranks (one process per GPU) and the one exchange the batched
adjoint needs: the sum of per-trial gradients in global trial order.

The reference runs one fly per worker over one shared read-only graph (src/brainsetup.js:10-28,
src/lifwasm.js:90-98); trials never exchange anything during a forward pass, so a batch splits
over GPUs by trial with no data-path collective.

  interleaved : rank r runs trials r, r + W, r + 2W, ... -- uneven trial lengths spread evenly;
                used where nothing is summed across trials (the forward ensemble).
  blocks      : rank r runs one contiguous run of trials -- used where per-trial results are
                summed (the adjoint's per-edge gradients), because then an ordered sum needs one
                hand-over per rank, not one per trial.

ordered_sum adds per-trial arrays in global trial order b = 0, 1, ..., B - 1, exactly as one
process adding them in a loop would (the same float64 additions in the same order), so the result
is bit-identical whatever the number of ranks: rank 0 sums its block, hands the running sum to
rank 1, which continues with its own block, and so on; the last rank's sum is broadcast. Each hand
over is a point-to-point send of one array (NCCL on GPUs, gloo on CPUs).
"""
from __future__ import annotations

import numpy as np


def trials_of_rank(n_trials: int, rank: int, world: int, mode: str = "interleaved") -> np.ndarray:
    """Global ids of the trials rank `rank` of `world` runs, ascending."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    if mode == "interleaved":
        return np.arange(rank, n_trials, world, dtype=np.int64)
    if mode == "blocks":
        lo = n_trials * rank // world
        hi = n_trials * (rank + 1) // world
        return np.arange(lo, hi, dtype=np.int64)
    raise ValueError(f"unknown mode {mode!r}")


def local_ordered_sum(arrays, start=None):
    """((start + a0) + a1) + ... in float64, the arrays in the order given."""
    import torch

    acc = None if start is None else start.clone()
    for a in arrays:
        a = a.to(torch.float64)
        acc = a.clone() if acc is None else acc.add_(a)
    return acc


def ordered_sum(local_arrays, n_trials: int, rank: int, world: int, shape, device="cpu", group=None):
    """The float64 sum over all trials in global order, given this rank's per-trial arrays (in
    its block's order, `trials_of_rank(..., mode="blocks")`). Every rank receives the result.
    With world == 1 this is local_ordered_sum."""
    import torch

    if world == 1:
        out = local_ordered_sum(local_arrays)
        return out if out is not None else torch.zeros(shape, dtype=torch.float64, device=device)
    import torch.distributed as dist

    mine = trials_of_rank(n_trials, rank, world, "blocks")
    if len(local_arrays) != mine.shape[0]:
        raise ValueError(f"rank {rank} holds {len(local_arrays)} arrays for {mine.shape[0]} trials")
    # the running sum arrives from the previous rank that holds any trial (empty blocks pass it on)
    start = None
    if rank > 0:
        flag = torch.zeros(1, dtype=torch.int64, device=device)
        dist.recv(flag, src=rank - 1, group=group)
        if int(flag.item()):
            start = torch.empty(shape, dtype=torch.float64, device=device)
            dist.recv(start, src=rank - 1, group=group)
    acc = local_ordered_sum(local_arrays, start)
    if rank < world - 1:
        dist.send(torch.tensor([1 if acc is not None else 0], dtype=torch.int64, device=device), dst=rank + 1,
                  group=group)
        if acc is not None:
            dist.send(acc.contiguous(), dst=rank + 1, group=group)
    out = acc if rank == world - 1 else None
    if out is None:
        out = torch.zeros(shape, dtype=torch.float64, device=device)
    # the last rank's total goes to everyone (a zero array if no rank held a trial)
    dist.broadcast(out, src=world - 1, group=group)
    return out

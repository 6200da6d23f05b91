"""Multi-GPU evaluation by replicas (one process per GPU).

Parameter sets of a batch are independent, so several GPUs evaluate disjoint
shards of one global batch with a full copy of the model each (tables are
replicated per GPU); there is no data-path collective. The only exchanges are
host-level: gathering the shards' log-likelihoods (and gradients) back into the
global batch order, and the max over ranks of a timing.

``shard`` splits a global batch of ``n`` rows into ``world`` contiguous, balanced
slices; ``gather_rows`` all-gathers each rank's rows (shards may differ in length
by one) and concatenates them in rank order, so the result is the global batch in
its original order on every rank. ``ReplicaBatch`` combines both around any
per-shard evaluator (an engine's batched log-likelihood or gradient, or a CPU
function in tests). Works with any torch.distributed backend (NCCL for GPU
tensors, gloo for CPU tensors).
"""

from __future__ import annotations

from typing import Callable, Tuple


def shard(n: int, rank: int, world: int) -> slice:
    """Contiguous slice of rows [0, n) owned by ``rank``; the first n % world ranks
    take one row more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return slice(start, start + base + (1 if rank < extra else 0))


def gather_rows(local, n: int, dist, group=None):
    """All-gather the rows each rank computed for its ``shard`` of an n-row batch;
    returns the n rows in global order (a tensor on the local tensor's device)."""
    import torch

    world = dist.get_world_size(group)
    sizes = [shard(n, r, world).stop - shard(n, r, world).start for r in range(world)]
    cap = max(sizes)
    pad = torch.zeros((cap,) + tuple(local.shape[1:]), dtype=local.dtype, device=local.device)
    pad[: local.shape[0]] = local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    return torch.cat([p[:s] for p, s in zip(parts, sizes)], dim=0)


def max_over_ranks(value: float, dist, device="cpu", group=None) -> float:
    """The maximum of a per-rank number (e.g. the time of the slowest rank)."""
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


class ReplicaBatch:
    """Evaluate a global batch across ranks: each rank runs ``evaluate`` on its
    shard (a (rows, P) tensor) and every rank receives the gathered outputs.

    ``evaluate`` returns one tensor or a tuple of tensors with one row per
    parameter set (e.g. (log L, neglect) or (log L, gradient, neglect))."""

    def __init__(self, evaluate: Callable, dist, group=None):
        self.evaluate = evaluate
        self.dist = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)

    def __call__(self, params) -> Tuple:
        n = params.shape[0]
        out = self.evaluate(params[shard(n, self.rank, self.world)])
        single = not isinstance(out, tuple)
        outs = (out,) if single else out
        full = tuple(gather_rows(o, n, self.dist, self.group) for o in outs)
        return full[0] if single else full

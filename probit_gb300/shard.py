"""Sharding a batch of independent GPs across ranks (one process per GPU).

The problems of a batch are independent, so a batch shards by whole problems
with no device collective: every rank evaluates the problems that the
longest-processing-time rule gives it (cost ~ N^3, the factorisation; the
list is the same on every rank, so no exchange is needed to agree on it), on
its own GPU with its own :class:`~probit_gb300.LaplaceBatch`, and the
per-problem results (a value and a gradient, a few floats each) are gathered
on the host over the process group (``gloo`` or ``nccl``; objects, not device
tensors).
"""

from __future__ import annotations

import heapq


def lpt_partition(costs, nparts):
    """Assign item k (cost costs[k]) to one of `nparts` parts, largest cost
    first, each to the currently least loaded part (ties: lowest part).
    Returns a list of `nparts` index lists, each in increasing index order.
    Deterministic, so every rank computes the same partition."""
    if nparts < 1:
        raise ValueError("nparts must be >= 1")
    order = sorted(range(len(costs)), key=lambda k: (-float(costs[k]), k))
    heap = [(0.0, p) for p in range(nparts)]
    parts = [[] for _ in range(nparts)]
    for k in order:
        load, p = heapq.heappop(heap)
        parts[p].append(k)
        heapq.heappush(heap, (load + float(costs[k]), p))
    return [sorted(p) for p in parts]


def shard_indices(costs, rank, world):
    """The items rank `rank` of `world` evaluates."""
    return lpt_partition(costs, world)[rank]


def gather_results(local_indices, local_results, n_total, group=None):
    """Every rank passes its items' indices and results; every rank gets the
    list of all `n_total` results in index order (host objects over the
    process group)."""
    import torch.distributed as dist

    world = dist.get_world_size(group)
    mine = list(zip(local_indices, local_results))
    allp = [None] * world
    dist.all_gather_object(allp, mine, group=group)
    out = [None] * n_total
    for part in allp:
        for k, r in part:
            if out[k] is not None:
                raise RuntimeError(f"item {k} evaluated on two ranks")
            out[k] = r
    missing = [k for k, r in enumerate(out) if r is None]
    if missing:
        raise RuntimeError(f"items {missing[:8]} evaluated on no rank")
    return out


class ShardedBatch:
    """A batch of GPs spread over the ranks of a process group.

    ``gps`` / ``params`` are the whole batch (the same on every rank);
    each rank builds a :class:`~probit_gb300.LaplaceBatch` of its share on its
    current CUDA device (``batch_cls`` stands in for it where no GPU is
    used).  ``value_and_grad()(params)`` returns, on every rank, the values
    and gradients of all problems in batch order; with ``world == 1`` no
    process group is needed."""

    def __init__(self, gps, params, group=None, rank=None, world=None, batch_cls=None):
        if batch_cls is None:
            from .batch import LaplaceBatch as batch_cls
        if rank is None or world is None:
            import torch.distributed as dist

            rank = dist.get_rank(group) if rank is None else rank
            world = dist.get_world_size(group) if world is None else world
        self.group = group
        self.rank = rank
        self.world = world
        self.n = len(gps)
        self.local = shard_indices([float(gp.N) ** 3 for gp in gps], self.rank, self.world)
        self.batch = batch_cls([gps[k] for k in self.local], [params[k] for k in self.local]) if self.local else None

    def value_and_grad(self):
        local_vg = self.batch.value_and_grad() if self.batch is not None else None

        def vg(params):
            if local_vg is not None:
                vals, grads = local_vg([params[k] for k in self.local])
                res = list(zip(vals, grads))
            else:
                res = []
            if self.world == 1:
                allr = res
            else:
                allr = gather_results(self.local, res, self.n, self.group)
            return [r[0] for r in allr], [r[1] for r in allr]

        return vg


def run_sharded_rounds(gps, params, rounds, warmup=1, group=None, rank=None, world=None, batch_cls=None,
                       sync=None):
    """Evaluate a batch sharded over the ranks ``rounds`` times and time it.

    Each round is one ``ShardedBatch.value_and_grad()`` call: every rank
    evaluates its LPT share (one batched launch sequence on its GPU) and the
    per-problem results are gathered on every rank.  A barrier precedes the
    timed rounds; ``sync`` (e.g. ``torch.cuda.synchronize``) is called on both
    sides of them; the time is the maximum over ranks.  Returns a dict with
    the rank's problem count, the problems per second of the whole job
    (len(gps) * rounds / max time), every rank's local time and the last
    round's results in batch order."""
    import time

    sb = ShardedBatch(gps, params, group=group, rank=rank, world=world, batch_cls=batch_cls)
    vg = sb.value_and_grad()
    for _ in range(warmup):
        out = vg(params)
    dist = None
    if sb.world > 1:
        import torch.distributed as dist

        dist.barrier(group)
    if sync:
        sync()
    t0 = time.perf_counter()
    for _ in range(rounds):
        out = vg(params)
    if sync:
        sync()
    local_s = time.perf_counter() - t0
    times = [local_s]
    if dist is not None:
        times = [None] * sb.world
        dist.all_gather_object(times, local_s, group=group)
    wall = max(times)
    return {"ranks": sb.world, "rank": sb.rank, "local_problems": len(sb.local), "rounds": rounds,
            "value": len(gps) * rounds / wall, "max_s": wall, "per_rank_s": times,
            "values": out[0], "grads": out[1]}

"""Sharding a batch by whole problems (probit_gb300.shard): the
longest-processing-time partition, and the host-side gather of per-problem
results over a world_size-2 gloo process group on the CPU."""

import os
import socket

import numpy as np
import pytest

from probit_gb300 import shard


def test_lpt_partition_covers_and_balances():
    rng = np.random.default_rng(0)
    N = np.exp(rng.uniform(np.log(32), np.log(4096), size=300)).astype(int)
    costs = N.astype(float) ** 3
    for parts in (1, 2, 3, 8):
        p = shard.lpt_partition(costs, parts)
        flat = sorted(k for q in p for k in q)
        assert flat == list(range(len(costs)))
        loads = [costs[q].sum() for q in p]
        # LPT bound: max load <= mean load + the largest single cost
        assert max(loads) <= sum(loads) / parts + costs.max() + 1e-6
        assert p == shard.lpt_partition(list(costs), parts)   # deterministic


def test_lpt_partition_edge_cases():
    assert shard.lpt_partition([], 2) == [[], []]
    assert shard.lpt_partition([5.0], 3) == [[0], [], []]
    with pytest.raises(ValueError):
        shard.lpt_partition([1.0], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n, out_path):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        costs = [float((k * 37) % 101 + 1) ** 3 for k in range(n)]
        mine = shard.shard_indices(costs, rank, world)
        res = [(k, k * 10.0) for k in mine]          # stands in for (value, gradient) of problem k
        allr = shard.gather_results(mine, res, n)
        np.save(f"{out_path}.{rank}.npy", np.array(allr, dtype=float))
    finally:
        dist.destroy_process_group()


def test_gather_over_gloo_world_2(tmp_path):
    import torch.multiprocessing as mp

    n = 23
    out = str(tmp_path / "r")
    mp.spawn(_worker, args=(2, _free_port(), n, out), nprocs=2, join=True)
    want = np.array([(k, k * 10.0) for k in range(n)], dtype=float)
    for rank in range(2):
        assert np.array_equal(np.load(f"{out}.{rank}.npy"), want)


class _FakeGP:
    def __init__(self, N):
        self.N = N


class _FakeBatch:
    """Stands in for LaplaceBatch on the CPU: value = N, gradient = (N, param)."""

    def __init__(self, gps, params):
        self.gps, self.params = gps, params

    def value_and_grad(self):
        def vg(params):
            return [float(g.N) for g in self.gps], [(float(g.N), p) for g, p in zip(self.gps, params)]

        return vg


def _sharded_worker(rank, world, port, out_path):
    import torch.distributed as dist

    import probit_gb300.batch as B

    B.LaplaceBatch = _FakeBatch
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        Ns = [40, 4000, 128, 900, 2048, 33, 513, 3000, 64]
        gps = [_FakeGP(n) for n in Ns]
        params = [float(k) for k in range(len(Ns))]
        sb = shard.ShardedBatch(gps, params)
        vals, grads = sb.value_and_grad()(params)
        np.save(f"{out_path}.{rank}.npy", np.array([vals, [g[0] for g in grads], [g[1] for g in grads]]))
        np.save(f"{out_path}.{rank}.local.npy", np.array(sb.local))
    finally:
        dist.destroy_process_group()


def test_sharded_batch_order_over_gloo_world_2(tmp_path):
    import torch.multiprocessing as mp

    out = str(tmp_path / "s")
    mp.spawn(_sharded_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    Ns = [40, 4000, 128, 900, 2048, 33, 513, 3000, 64]
    for rank in range(2):
        got = np.load(f"{out}.{rank}.npy")
        assert np.array_equal(got[0], np.array(Ns, float))
        assert np.array_equal(got[2], np.arange(len(Ns), dtype=float))
    l0, l1 = (set(np.load(f"{out}.{r}.local.npy").tolist()) for r in range(2))
    assert not (l0 & l1) and (l0 | l1) == set(range(len(Ns)))


def _bench_worker(rank, world, port, out_path):
    import torch.distributed as dist

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        Ns = [40, 4000, 128, 900, 2048, 33, 513, 3000, 64, 1500]
        res = shard.run_sharded_rounds([_FakeGP(n) for n in Ns], [float(k) for k in range(len(Ns))], rounds=3,
                                       batch_cls=_FakeBatch)
        np.save(f"{out_path}.{rank}.npy", np.array([res["values"], [g[1] for g in res["grads"]]]))
        np.save(f"{out_path}.{rank}.meta.npy", np.array([res["ranks"], res["local_problems"], res["value"],
                                                          res["max_s"], max(res["per_rank_s"])]))
    finally:
        dist.destroy_process_group()


def test_bench_sharded_rounds_over_gloo_world_2(tmp_path):
    """The bench's sharded path (shard.run_sharded_rounds): LPT shares over two
    gloo ranks, results gathered in batch order on both, the job's rate taken
    over the slower rank."""
    import torch.multiprocessing as mp

    out = str(tmp_path / "b")
    mp.spawn(_bench_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    Ns = [40, 4000, 128, 900, 2048, 33, 513, 3000, 64, 1500]
    metas = [np.load(f"{out}.{r}.meta.npy") for r in range(2)]
    for r in range(2):
        got = np.load(f"{out}.{r}.npy")
        assert np.array_equal(got[0], np.array(Ns, float))
        assert np.array_equal(got[1], np.arange(len(Ns), dtype=float))
        assert metas[r][0] == 2 and metas[r][3] == metas[r][4]
        assert metas[r][2] == pytest.approx(len(Ns) * 3 / metas[r][3])
    assert metas[0][1] + metas[1][1] == len(Ns)
    assert metas[0][3] == metas[1][3]


def test_bench_sharded_rounds_single_rank():
    Ns = [100, 2000, 300]
    res = shard.run_sharded_rounds([_FakeGP(n) for n in Ns], [0.0, 1.0, 2.0], rounds=2, rank=0, world=1,
                                   batch_cls=_FakeBatch)
    assert res["ranks"] == 1 and res["local_problems"] == 3
    assert res["values"] == [float(n) for n in Ns]

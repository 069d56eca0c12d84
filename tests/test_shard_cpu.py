"""Instance sharding of the batched workload (sdpa-gmp_gb300/shard.py): the cost-ordered
partition, its balance, and the gather of per-instance results on rank 0 in the original
order, with two gloo ranks on the CPU (the solve itself is replaced by a pure function of
the instance, so no GPU is needed)."""
import importlib
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
shard = importlib.import_module("sdpa-gmp_gb300.shard")
problems = importlib.import_module("sdpa-gmp_gb300.problems")


def test_partition_covers_and_balances():
    sizes = [problems.batch_instance_size(s) for s in range(256)]
    costs = [shard.instance_cost(m, b) for m, b in sizes]
    for world in (1, 2, 3, 4, 8):
        parts = shard.partition(costs, world)
        assert sorted(i for p in parts for i in p) == list(range(len(costs)))
        assert all(p == sorted(p) for p in parts)
        ld = shard.loads(costs, parts)
        # greedy largest-first: no rank exceeds the mean by more than the largest instance
        assert max(ld) - sum(ld) / world <= max(costs), (world, ld)
        assert shard.partition(costs, world) == parts  # deterministic on every rank


def test_instance_size_matches_generator():
    for seed in (0, 7, 1023):
        m, blocks = problems.batch_instance_size(seed)
        c, F0, F = problems.batch_instance(seed)
        assert len(c) == m
        assert [blk.shape[0] for blk in F0] == blocks


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    sh = importlib.import_module("sdpa-gmp_gb300.shard")
    instances = list(range(40))
    costs = [(17 * i) % 23 + 1 for i in instances]
    solved = []

    def solve(items):
        solved.extend(items)
        return [(i, i * i) for i in items]

    res = sh.solve_sharded(instances, costs, solve, rank, world, dist)
    out.put((rank, sorted(solved), res))
    dist.destroy_process_group()


def test_two_gloo_ranks_gather_in_order():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted((q.get(timeout=120) for _ in procs), key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, solved0, res0), (r1, solved1, res1) = results
    assert res1 is None
    assert res0 == [(i, i * i) for i in range(40)]
    # each instance solved exactly once, on the rank the partition gave it
    parts = shard.partition([(17 * i) % 23 + 1 for i in range(40)], 2)
    assert solved0 == parts[0] and solved1 == parts[1]
    assert not set(solved0) & set(solved1)

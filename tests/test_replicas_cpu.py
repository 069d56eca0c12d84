"""The multi-GPU mode of bench.py runs one independent replica per rank (the single
solve does not shard); its only cross-rank logic is the barrier and the max / sum
reductions of the timing.  Exercised here with two gloo ranks on the CPU."""
import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out):
    import importlib.util
    import sys
    os.environ.update({"RANK": str(rank), "LOCAL_RANK": str(rank), "WORLD_SIZE": str(world),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(root, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    w, r, local, dist = bench.dist_setup(world)
    bench.barrier(dist)
    mx = bench.max_over_ranks(dist, 10.0 + r)      # per-rank times: the slowest rank counts
    total = bench.sum_over_ranks(dist, 5.0)        # per-rank steps: the job's total
    out.put((r, w, local, mx, total))
    dist.destroy_process_group()


def test_two_gloo_ranks_reduce_timing():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[0] for r in results] == [0, 1]
    for r, w, local, mx, total in results:
        assert w == 2 and local == r
        assert mx == 11.0 and total == 10.0

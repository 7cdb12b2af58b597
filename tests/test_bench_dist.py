"""The bench's multi-rank path on CPU: two gloo ranks (world size 2) exchange
the max-over-ranks step time and the summed work, and each rank draws its
own source sample (replicas, weak scaling) -- everything bench.py does across
ranks, without a GPU."""
import os
import socket
import sys
import types

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        mx = d.max(float(rank + 1) * 10.0)
        sm = d.sum(float(rank + 1))
        args = types.SimpleNamespace(workload="c2", scale=10, k=64)
        _, src, k_act, _, name = bench.workload(rank, args)
        import torch.distributed as dist
        obj = [None] * world
        dist.all_gather_object(obj, sorted(int(x) for x in src))
        q.put((rank, mx, sm, k_act, name, obj))
    finally:
        d.close()


def test_two_gloo_ranks():
    world = 2
    port = _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, mx, sm, k_act, name, srcs in out:
        assert mx == 20.0 and sm == 3.0
        assert name == "rmat10_sampled_bc_k64" and 0 < k_act <= 64
        assert srcs[0] != srcs[1]  # each rank its own sample (seed 2 + rank)

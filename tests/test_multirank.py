"""The N > 1 path on CPU: bench.py's ranks are one process per GPU, joined by a gloo process group
used only for the barrier and the max/sum of the timings (the forward path has no exchange step:
points are independent). World size 2, rendezvous on 127.0.0.1, processes started with spawn."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, task, q):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    try:
        import bench

        dist = bench.Dist()
        if task == "aggregate":
            dist.barrier()
            q.put((rank, dist.max(10.0 + rank), dist.sum(100.0 * (rank + 1)), dist.world))
        else:  # each rank evaluates its own range of points with the oracle; ranks gather the rows
            import torch

            from oracle import oracle
            from qmckl_sycl_gb300 import config_small

            s = config_small(5, point_num=64)
            lo, hi = rank * s.point_num // world, (rank + 1) * s.point_num // world
            part = oracle.forward(s.with_points(s.coord[lo:hi]), want=("mo_vgl",))["mo_vgl"]
            t = torch.from_numpy(np.ascontiguousarray(part))
            parts = [torch.empty_like(t) for _ in range(world)]
            dist.pg.all_gather(parts, t)
            q.put((rank, np.concatenate([p.numpy() for p in parts]), None, dist.world))
        dist.pg.destroy_process_group()
    except Exception as e:  # reported to the parent
        q.put((rank, "error: %r" % (e,), None, None))


def _run(task, world=2):
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, task, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = [q.get(timeout=240) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    return sorted(out, key=lambda r: r[0])


def test_bench_rank_aggregation_world_size_2():
    out = _run("aggregate")
    for rank, mx, sm, world in out:
        assert not isinstance(mx, str), mx
        assert world == 2
        assert mx == 11.0  # the slowest rank's time
        assert sm == 300.0  # the units of all ranks


def test_points_shard_across_ranks_without_exchange():
    # rank r evaluates points [r P / 2, (r + 1) P / 2); the gathered rows are the single-process
    # result bit for bit (each point's AO and MO values depend on that point only)
    from oracle import oracle
    from qmckl_sycl_gb300 import config_small

    out = _run("shard")
    s = config_small(5, point_num=64)
    full = oracle.forward(s, want=("mo_vgl",))["mo_vgl"]
    for rank, rows, _, world in out:
        assert not isinstance(rows, str), rows
        assert np.array_equal(rows, full)

"""Host logic of point sharding (qmckl_sycl_gb300/sharding.py) on CPU: the ranges cover every
point once, in whole blocks, as evenly as blocks allow; and the sharded VJP's all-reduce sums the
ranks' coefficient and exponent gradients and leaves each rank its coordinates' gradients (world
size 2, gloo on 127.0.0.1, a stand-in context that returns fixed arrays, processes started with
spawn)."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from qmckl_sycl_gb300.sharding import point_range  # noqa: E402


@pytest.mark.parametrize("P,world,block", [(40960, 1, 160), (40960, 2, 160), (40960, 3, 160), (50, 4, 1),
                                           (7, 8, 1), (2048, 5, 64)])
def test_point_ranges_cover_every_point_once(P, world, block):
    ranges = [point_range(P, r, world, block) for r in range(world)]
    assert ranges[0][0] == 0 and ranges[-1][1] == P
    for (a, b), (c, d) in zip(ranges, ranges[1:]):
        assert b == c
    sizes = [b - a for a, b in ranges]
    assert all(s % block == 0 for s in sizes)
    assert max(sizes) - min(sizes) <= block


def test_point_range_rejects_bad_arguments():
    with pytest.raises(ValueError):
        point_range(10, 2, 2)
    with pytest.raises(ValueError):
        point_range(10, 0, 2, block=3)


class _FakeContext:
    """Gradients that depend on the rank, as a context holding that rank's points would give."""

    def __init__(self, rank):
        self.rank = rank

    def vjp_mo_vgl(self, w, prim_num=None):
        r = self.rank + 1.0
        return {"coef": np.full((3, 4), r), "expo": np.arange(5) * r, "coord": np.full((2, 3), -r)}


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    try:
        import torch.distributed as dist

        sys.path.insert(0, ROOT)
        from qmckl_sycl_gb300.sharding import vjp_mo_vgl_allreduce

        dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
        g = vjp_mo_vgl_allreduce(_FakeContext(rank), None, 5)
        dist.destroy_process_group()
        q.put((rank, g))
    except Exception as e:  # reported to the parent
        q.put((rank, "error: %r" % (e,)))


def test_sharded_vjp_allreduce_on_cpu():
    pytest.importorskip("torch")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=240) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
    for rank, g in out.items():
        assert not isinstance(g, str), g
        assert np.array_equal(g["coef"], np.full((3, 4), 3.0))      # 1 + 2
        assert np.array_equal(g["expo"], np.arange(5) * 3.0)
        assert np.array_equal(g["coord"], np.full((2, 3), -(rank + 1.0)))  # local, not reduced

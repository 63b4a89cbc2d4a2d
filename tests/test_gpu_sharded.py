"""Points sharded over two processes on the GPU (the replicas a multi-GPU run would place one per
GPU; here both use cuda:0, which is safe because no kernel of one rank waits on the other), joined
by a gloo process group on 127.0.0.1: each rank evaluates its contiguous range of the adjoint
workload's points through its own context. The ranks' mo_vgl rows together must equal a single
context's bit for bit (points are independent; both forms), and the sharded VJP (one all-reduce of
the coefficient and exponent gradients, coordinates local) must match the single context's
gradients within 1e-12 (only the order of some sums differs)."""
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest

from conftest import normwise_rel_err

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _weights(s):
    return np.random.default_rng(21).normal(size=(s.point_num, 5, s.mo_num))


def _rank_main(rank, world, port, q):
    try:
        import torch.distributed as dist

        sys.path.insert(0, ROOT)
        from qmckl_sycl_gb300 import Context, config_adjoint
        from qmckl_sycl_gb300.sharding import point_range, vjp_mo_vgl_allreduce

        dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
        s = config_adjoint(0)
        lo, hi = point_range(s.point_num, rank, world, block=32)
        part = s.with_points(s.coord[lo:hi])
        out = {"range": (lo, hi)}
        with Context(0) as ctx:
            ctx.load_system(part)
            for mode in (0, 1):
                ctx.set_precision(mode)
                ctx.touch()
                out["mo_vgl%d" % mode] = ctx.get_mo_vgl(hi - lo)
            out["grad"] = vjp_mo_vgl_allreduce(ctx, _weights(s)[lo:hi], s.prim_num)
        dist.destroy_process_group()
        q.put((rank, out))
    except Exception as e:  # reported to the parent
        q.put((rank, "error: %r" % (e,)))


def test_two_ranks_equal_one_context():
    pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    mpc = mp.get_context("spawn")
    q = mpc.Queue()
    port = _free_port()
    procs = [mpc.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=600) for _ in range(2))
    for p in procs:
        p.join(timeout=120)
    for r in out:
        assert not isinstance(out[r], str), out[r]

    from qmckl_sycl_gb300 import Context, config_adjoint

    s = config_adjoint(0)
    with Context(0) as ctx:
        ctx.load_system(s)
        want = {}
        for mode in (0, 1):
            ctx.set_precision(mode)
            ctx.touch()
            want[mode] = ctx.get_mo_vgl(s.point_num)
        ctx.set_precision(0)
        g = ctx.vjp_mo_vgl(_weights(s), prim_num=s.prim_num)
    for mode in (0, 1):
        rows = np.concatenate([out[r]["mo_vgl%d" % mode] for r in (0, 1)])
        assert np.array_equal(rows, want[mode]), mode
    # a point's coordinate gradient sums its nucleus chunks, whose size follows the point count
    coord = np.concatenate([out[r]["grad"]["coord"] for r in (0, 1)])
    assert normwise_rel_err(coord, g["coord"]) <= 1e-12
    for r in (0, 1):
        for k in ("coef", "expo"):
            assert normwise_rel_err(out[r]["grad"][k], g[k]) <= 1e-12, (r, k)

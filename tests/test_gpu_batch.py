"""Batched form: many molecules of uneven size evaluated by one persistent launch per stage,
replayed as a CUDA graph, with autotuned launch parameters. Every member's result must be the
single-context result bit for bit (FP64 and split-BF16 alike: the batch runs the same per-tile
arithmetic), hence within 1e-12 (FP64) or 1e-6 (split-BF16) of the oracle, whatever the tuning,
across graph replays with new points, and with members that have no points."""
import numpy as np
import pytest

from conftest import normwise_rel_err
from oracle import oracle
from qmckl_sycl_gb300 import PRECISION_FP64, PRECISION_SPLIT_BF16, Batch, Context, config_batched

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-12
MIXED_RTOL = 1e-6


def small_batch(seed=0, molecules=6, walkers=2):
    """config_batched's generators with fewer molecules and walkers (oracle-sized)."""
    return config_batched(seed, molecules=molecules, walkers=walkers)


def single(s, mode):
    with Context(0) as ctx:
        ctx.load_system(s)
        ctx.set_precision(mode)
        return ctx.get_mo_vgl(s.point_num)


def members_of(systems):
    ctxs = []
    for s in systems:
        c = Context(0)
        c.load_system(s)
        ctxs.append(c)
    return ctxs


def close_all(batch, ctxs):
    batch.close()
    for c in ctxs:
        c.close()


@pytest.mark.parametrize("mode", [PRECISION_FP64, PRECISION_SPLIT_BF16])
def test_batch_matches_single_context_and_oracle(mode):
    systems = small_batch(0)
    ctxs = members_of(systems)
    b = Batch(ctxs)
    try:
        b.set_precision(mode)
        outs = b.get_mo_vgl()
        tune = b.tuning()
        assert tune[0] >= 0 and tune[1] in (0, 1, 2) and 16 <= tune[2] <= 160
        assert b.launch_count() == 5
        for s, got in zip(systems, outs):
            assert np.array_equal(got, single(s, mode)), s.name
        tol = FP64_RTOL if mode == PRECISION_FP64 else MIXED_RTOL
        for s, got in list(zip(systems, outs))[:3]:
            ref = oracle.forward(s, want=("mo_vgl",))["mo_vgl"]
            assert normwise_rel_err(got, ref) <= tol, s.name
    finally:
        close_all(b, ctxs)


@pytest.mark.parametrize("mode", [PRECISION_FP64, PRECISION_SPLIT_BF16])
def test_every_tuning_gives_the_same_bits(mode):
    systems = small_batch(1, molecules=4)
    ctxs = members_of(systems)
    b = Batch(ctxs)
    try:
        b.set_precision(mode)
        first = None
        configs = [(0, 0, 160), (1, 1, 128), (2, 2, 96), (3, 0, 48), (30, 1, 16)]
        for params in configs:
            b.set_tuning(params)
            assert b.tuning() == params
            b.touch()
            outs = b.get_mo_vgl()
            if first is None:
                first = outs
            else:
                for x, y in zip(first, outs):
                    assert np.array_equal(x, y), params
    finally:
        close_all(b, ctxs)


@pytest.mark.parametrize("graph", [True, False])
def test_replay_with_new_points(graph):
    systems = small_batch(2, molecules=5)
    ctxs = members_of(systems)
    b = Batch(ctxs)
    try:
        b.set_graph(graph)
        b.get_mo_vgl()
        rng = np.random.default_rng(7)
        for step in range(3):
            moved = []
            for s, c in zip(systems, ctxs):
                s2 = s.with_points(s.coord + rng.normal(0.0, 0.3, size=s.coord.shape))
                c.set_point(s2.coord)
                moved.append(s2)
            outs = b.get_mo_vgl()
            for s2, got in zip(moved, outs):
                assert np.array_equal(got, single(s2, PRECISION_FP64)), (step, s2.name)
        ref = oracle.forward(moved[0], want=("mo_vgl",))["mo_vgl"]
        assert normwise_rel_err(outs[0], ref) <= FP64_RTOL
    finally:
        close_all(b, ctxs)


def test_member_without_points_and_ao_cache():
    systems = small_batch(3, molecules=3)
    systems[1] = systems[1].with_points(np.zeros((0, 3)))
    ctxs = members_of(systems)
    b = Batch(ctxs)
    try:
        b.provide_mo_vgl()
        for i in (0, 2):
            s = systems[i]
            ref = oracle.forward(s, want=("ao_vgl", "mo_vgl"))
            # the FP64 batch also leaves each member's ao_vgl current
            assert normwise_rel_err(ctxs[i].get_ao_vgl(s.point_num), ref["ao_vgl"]) <= FP64_RTOL
            assert normwise_rel_err(ctxs[i].get_mo_vgl(s.point_num), ref["mo_vgl"]) <= FP64_RTOL
    finally:
        close_all(b, ctxs)


def test_autotune_and_async():
    systems = small_batch(4, molecules=4)
    ctxs = members_of(systems)
    b = Batch(ctxs)
    try:
        b.set_precision(PRECISION_SPLIT_BF16)
        b.autotune()
        t = b.tuning()
        assert t[0] >= 0 and 16 <= t[2] <= 160
        b.set_async(True)
        b.touch()
        b.provide_mo_vgl()
        b.synchronize()
        for s, c in zip(systems, ctxs):
            assert np.array_equal(c.get_mo_vgl(s.point_num), single(s, PRECISION_SPLIT_BF16))
    finally:
        close_all(b, ctxs)


def test_profiled_stages_are_recorded():
    systems = small_batch(5, molecules=3)
    ctxs = members_of(systems)
    b = Batch(ctxs)
    try:
        ctxs[0].set_profiling(True)
        ctxs[0].reset_kernel_stats()
        b.provide_mo_vgl()
        stats = ctxs[0].kernel_stats()
        assert {"batch_point_order", "batch_ao_vgl", "batch_mo_vgl_dgemm"} <= set(stats)
        assert all(stats[k][1] > 0 for k in ("batch_ao_vgl", "batch_mo_vgl_dgemm"))
    finally:
        close_all(b, ctxs)

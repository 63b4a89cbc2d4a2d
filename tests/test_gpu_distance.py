"""Electron-nucleus and electron-electron distances (reference src/qmckl_electron.cpp:192-552)
against the oracle's restatement of their intended result, bit for bit (same operations, correctly
rounded square root), through the providers, getters and the low-level distance call."""
import ctypes

import numpy as np
import pytest

from oracle import oracle
from qmckl_sycl_gb300 import Context, config_medium, config_small

pytestmark = pytest.mark.gpu


def test_en_distance_matches_oracle_bitwise(chbrclf):
    for s in (chbrclf, config_small(1, point_num=77), config_medium(0, walkers=2, electrons=160)):
        with Context(0) as ctx:
            ctx.load_system(s)
            got = np.empty((s.point_num, s.nucl_num))
            ctx.call("get_electron_en_distance", got.ctypes.data_as(ctypes.c_void_p), got.size)
        assert np.array_equal(got, oracle.en_distance(s)), s.name


def test_ee_distance_per_walker(chbrclf, golden):
    s = chbrclf
    elec, walk = int(golden["elec_num"]), int(golden["walk_num"])
    up, dn = int(golden["elec_up_num"]), int(golden["elec_dn_num"])
    coord = s.coord[: walk * elec]
    with Context(0) as ctx:
        ctx.load_system(s, points=False)
        ctx.call("set_electron_num", up, dn)
        c = np.ascontiguousarray(coord)
        ctx.call("set_electron_coord", b"N", walk, c.ctypes.data_as(ctypes.c_void_p), c.size)
        got = np.empty((walk, elec, elec))
        ctx.call("get_electron_ee_distance", got.ctypes.data_as(ctypes.c_void_p), got.size)
    ref = oracle.ee_distance(np.ascontiguousarray(coord.T), elec, walk)
    assert np.array_equal(got, ref)
    assert np.all(np.diagonal(got, axis1=1, axis2=2) == 0.0)


@pytest.mark.parametrize("ta,tb", [("N", "N"), ("N", "T"), ("T", "N"), ("T", "T")])
def test_distance_layouts(ta, tb):
    rng = np.random.default_rng(3)
    m, n = 37, 53
    A = rng.normal(size=(m, 3)) * 4
    B = rng.normal(size=(n, 3)) * 4
    Al = np.ascontiguousarray(A.T) if ta == "T" else A
    Bl = np.ascontiguousarray(B.T) if tb == "T" else B
    lda = m if ta == "T" else 3
    ldb = n if tb == "T" else 3
    ldc = m + 3
    with Context(0) as ctx:
        dA, dB = ctx.upload(Al), ctx.upload(Bl)
        dC = ctx.buffer("C", 8 * ldc * n)
        rc = ctx.L.qmckl_distance_device(ctx.handle, ta.encode(), tb.encode(), m, n, dA.ptr, lda, dB.ptr, ldb,
                                         dC.ptr, ldc)
        assert rc == 0
        got = ctx.download(dC.ptr, (n, ldc))[:, :m]
    ref = np.zeros((n, ldc))
    oracle.lib().oracle_distance(ta.encode(), tb.encode(), m, n, np.ascontiguousarray(Al), lda,
                                 np.ascontiguousarray(Bl), ldb, ref, ldc)
    assert np.array_equal(got, ref[:, :m])
    assert np.allclose(got, np.linalg.norm(A[None, :, :] - B[:, None, :], axis=2), rtol=1e-15, atol=0)

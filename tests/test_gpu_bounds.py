"""The debug build with bounds checks on the kernels' global stores (-DQMCKL_BOUNDS_CHECK,
_lib/libqmckl_gpu_bounds.so). Every checked store tests its element index against the extent
of the array it writes; an out-of-range store is skipped and the first one recorded, with no
trap or assert. A child process loads that build (QMCKL_GB300_BOUNDS_CHECK=1) and runs the small
cases of every path (FP64 and split-BF16 AO/MO vgl and values, shell radials, ragged point
counts, centres without shells, the host-buffer chunked path, distances, the adjoint, a batch, the allocation-free
contraction); no store may have been out of range, and the results must still match the oracle.
The recording itself is checked first with the self-test kernel (an index past its extent,
nothing stored)."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import ctypes, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[1] + "/tests")
from conftest import normwise_rel_err
from oracle import oracle
from qmckl_sycl_gb300 import capi, Batch, Context, config_adjoint, config_batched, config_medium, config_small
from qmckl_sycl_gb300.systems import System, with_empty_nucleus

L = capi.lib()
assert b"bounds-check" in L.qmckl_gb300_build_info(), L.qmckl_gb300_build_info()
site, index, extent = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()


def status(reset=1):
    return L.qmckl_bounds_check_status_device(reset, ctypes.byref(site), ctypes.byref(index), ctypes.byref(extent))


with Context(0) as ctx:  # makes device 0 current
    assert status() in (0, 1)
    assert L.qmckl_bounds_check_selftest_device(5, 4) == 0
    assert status() == 1 and (site.value, index.value, extent.value) == (10, 5, 4), (site, index, extent)
    assert status() == 0  # the records were cleared

chbrclf = System.from_npz(sys.argv[1] + "/tests/golden/chbrclf.npz")
cases = [chbrclf, config_small(0), config_adjoint(0)] + [config_small(1, point_num=n) for n in (1, 33, 97)]
cases += [with_empty_nucleus(chbrclf, 0), with_empty_nucleus(config_small(2), 6)]  # centres without shells
for s in cases:
    ref = oracle.forward(s)
    for mode, tol in ((0, 1e-12), (1, 1e-6)):
        with Context(0) as ctx:
            ctx.load_system(s)
            ctx.set_precision(mode)
            P = s.point_num
            assert normwise_rel_err(ctx.get_ao_vgl(P), ref["ao_vgl"]) <= 1e-12
            assert normwise_rel_err(ctx.get_ao_value(P), ref["ao_value"]) <= 1e-12
            assert normwise_rel_err(ctx.get_mo_vgl(P), ref["mo_vgl"]) <= tol
            assert normwise_rel_err(ctx.get_mo_value(P), ref["mo_value"]) <= tol
            ctx.get_shell_vgl(P, s.shell_num)
            en = np.empty((P, s.nucl_num))
            ctx.call("get_electron_en_distance", en.ctypes.data_as(ctypes.c_void_p), en.size)
    assert status() == 0, (s.name, site.value, index.value, extent.value)

# the chunked host-buffer path (>= 16384 points, split-BF16)
s = config_medium(0, walkers=103, electrons=160)
with Context(0) as ctx:
    ctx.load_system(s)
    ctx.set_precision(1)
    ctx.get_mo_vgl(s.point_num)
assert status() == 0, ("chunked", site.value, index.value, extent.value)

# the adjoint
s = config_adjoint(0)
w = np.random.default_rng(1).normal(size=(s.point_num, 5, s.mo_num))
g = None
with Context(0) as ctx:
    ctx.load_system(s)
    g = ctx.vjp_mo_vgl(w, prim_num=s.prim_num)
gref = oracle.vjp_mo_vgl(s, w)
for k in ("coef", "expo", "coord"):
    assert normwise_rel_err(g[k], gref[k]) <= 1e-10, k
assert status() == 0, ("adjoint", site.value, index.value, extent.value)

# a batch, both forms
systems = config_batched(0, molecules=4, walkers=1)
for mode in (0, 1):
    ctxs = []
    for sy in systems:
        c = Context(0)
        c.load_system(sy)
        ctxs.append(c)
    with Batch(ctxs) as b:
        b.set_precision(mode)
        b.get_mo_vgl()
    for c in ctxs:
        c.close()
assert status() == 0, ("batch", site.value, index.value, extent.value)

# the allocation-free contraction, two chunks
s = config_medium(3, walkers=2, electrons=160)
with Context(0) as ctx:
    ctx.load_system(s)
    P, A, M = s.point_num, s.ao_num, s.mo_num
    ao = ctx.buffer("ao", 8 * 5 * P * A)
    ctx.call("get_ao_basis_ao_vgl", ctypes.c_void_p(ao.ptr), 5 * P * A)
    coef = ctx.upload(s.mo_coef)
    out = ctx.buffer("out", 8 * 5 * P * M)
    assert ctx.L.qmckl_mo_contract_split_bf16_noalloc_device(ao.ptr, 5 * P, A, coef.ptr, M, 1, out.ptr,
                                                             ctx.stream) == 0
assert status() == 0, ("noalloc", site.value, index.value, extent.value)
print("bounds-checked build: no out-of-range store")
"""


def test_bounds_checked_build_records_no_out_of_range_store():
    from qmckl_sycl_gb300 import build

    build.build(bounds=True)
    env = dict(os.environ, QMCKL_GB300_BOUNDS_CHECK="1")
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], env=env, capture_output=True, text=True, timeout=1500)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-4000:]
    assert "no out-of-range store" in r.stdout

"""Whole evaluations with the library's host code under AddressSanitizer and
UndefinedBehaviorSanitizer (_lib/libqmckl_gpu_asan.so; device code as usual), on the GPU: the
finalize that builds the packed tables, the caches and getters, both precision forms, the
host-buffer chunked path, a batch (descriptors, graph capture, autotuning), the adjoint, the
distances, the allocation-free contraction and error paths, in a child process with libasan
preloaded. Any report aborts the child; the results must still match the oracle."""
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
from qmckl_sycl_gb300 import capi, Batch, Context, QmcklError, config_adjoint, config_batched, config_medium, config_small
from qmckl_sycl_gb300.systems import System

assert capi.lib_path().endswith("libqmckl_gpu_asan.so"), capi.lib_path()
chbrclf = System.from_npz(sys.argv[1] + "/tests/golden/chbrclf.npz")
for s in (chbrclf, config_small(0), config_small(1, point_num=33)):
    ref = oracle.forward(s)
    for mode, tol in ((0, 1e-12), (1, 1e-6)):
        with Context(0) as ctx:
            ctx.load_system(s)
            ctx.set_precision(mode)
            P = s.point_num
            assert normwise_rel_err(ctx.get_ao_vgl(P), ref["ao_vgl"]) <= 1e-12
            assert normwise_rel_err(ctx.get_mo_vgl(P), ref["mo_vgl"]) <= tol
            assert normwise_rel_err(ctx.get_mo_value(P), ref["mo_value"]) <= tol
            ctx.get_shell_vgl(P, s.shell_num)
            en = np.empty((P, s.nucl_num))
            ctx.call("get_electron_en_distance", en.ctypes.data_as(ctypes.c_void_p), en.size)
            try:  # an error path: a buffer too small for the result
                ctx.call("get_mo_basis_mo_vgl", ctypes.c_void_p(0), 1)
                raise AssertionError("size check did not fire")
            except QmcklError:
                pass
s = config_medium(0, walkers=103, electrons=160)  # the host-buffer chunked path
with Context(0) as ctx:
    ctx.load_system(s)
    ctx.set_precision(1)
    ctx.get_mo_vgl(s.point_num)
s = config_adjoint(0)
w = np.random.default_rng(1).normal(size=(s.point_num, 5, s.mo_num))
with Context(0) as ctx:
    ctx.load_system(s)
    g = ctx.vjp_mo_vgl(w, prim_num=s.prim_num)
gref = oracle.vjp_mo_vgl(s, w)
for k in ("coef", "expo", "coord"):
    assert normwise_rel_err(g[k], gref[k]) <= 1e-10, k
systems = config_batched(0, molecules=4, walkers=1)
ctxs = []
for sy in systems:
    c = Context(0)
    c.load_system(sy)
    ctxs.append(c)
with Batch(ctxs) as b:
    for mode in (0, 1):
        b.set_precision(mode)
        b.get_mo_vgl()
for c in ctxs:
    c.close()
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
print("sanitized host code: no report")
"""


def test_whole_evaluations_under_address_and_undefined_behaviour_sanitizers():
    libasan = subprocess.run(["gcc", "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    if not os.path.isabs(libasan) or not os.path.exists(libasan):
        pytest.skip("libasan not available")
    from qmckl_sycl_gb300 import build

    build.build(sanitize=True)
    env = dict(os.environ, LD_PRELOAD=libasan, QMCKL_GB300_SANITIZE="1",
               ASAN_OPTIONS="detect_leaks=0:halt_on_error=1:protect_shadow_gap=0",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1")
    r = subprocess.run([sys.executable, "-c", CHILD, ROOT], env=env, capture_output=True, text=True, timeout=1500)
    assert r.returncode == 0 and "no report" in r.stdout, r.stdout[-3000:] + r.stderr[-6000:]

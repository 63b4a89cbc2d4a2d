"""The allocation-free split-BF16 contraction (qmckl_mo_contract_split_bf16_noalloc_device).

It serves callers that must not have device memory allocated for them (their own pool owns
the GPU's memory, or an allocation would synchronise the device); its scratch is a device
array compiled into the library. Its results must equal those of the context's split-BF16
path within the precision form's tolerance, on two calls in a row (the second reuses the
array the first left behind). This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from conftest import normwise_rel_err
from qmckl_sycl_gb300 import PRECISION_SPLIT_BF16, Context, config_medium

pytestmark = pytest.mark.gpu

MIXED_RTOL = 1e-6


def _nan_fill(ctx, buf, n):
    ctx.check(ctx.L.qmckl_memcpy_H2D(ctx.handle, buf.ptr, np.full(n, np.nan).ctypes.data_as(ctypes.c_void_p), 8 * n),
              "qmckl_memcpy_H2D")


def test_noalloc_contraction_matches_context_path():
    # 320 points -> 1600 vgl rows: more than one chunk of the scratch array
    s = config_medium(3, walkers=2, electrons=160)
    P, A, M = s.point_num, s.ao_num, s.mo_num
    with Context(0) as ctx:
        ctx.load_system(s)
        ctx.set_precision(PRECISION_SPLIT_BF16)
        want_vgl = ctx.get_mo_vgl(P)
        want_val = ctx.get_mo_value(P)
        ao_vgl = ctx.buffer("ao_vgl", 8 * 5 * P * A)
        ctx.call("get_ao_basis_ao_vgl", ctypes.c_void_p(ao_vgl.ptr), 5 * P * A)
        ao_val = ctx.buffer("ao_val", 8 * P * A)
        ctx.call("get_ao_basis_ao_value", ctypes.c_void_p(ao_val.ptr), P * A)
        coef = ctx.upload(s.mo_coef)
        out = ctx.buffer("out", 8 * 5 * P * M)
        f = ctx.L.qmckl_mo_contract_split_bf16_noalloc_device
        for call in range(2):
            _nan_fill(ctx, out, 5 * P * M)
            rc = f(ao_vgl.ptr, 5 * P, A, coef.ptr, M, 1, out.ptr, ctx.stream)
            assert rc == 0, "call %d returned %d" % (call, rc)
            got = ctx.download(out.ptr, (P, 5, M))
            assert np.isfinite(got).all()
            assert normwise_rel_err(got, want_vgl) <= MIXED_RTOL
        _nan_fill(ctx, out, P * M)
        assert f(ao_val.ptr, P, A, coef.ptr, M, 0, out.ptr, ctx.stream) == 0
        got = ctx.download(out.ptr, (P, M))
        assert normwise_rel_err(got, want_val) <= MIXED_RTOL


def test_noalloc_at_its_largest_shape_with_a_partial_chunk():
    # ao_num = 2048 and mo_num = 1024 fill the array up to the job descriptor; 1285 vgl rows are one
    # full chunk of 1280 and a partial one of 5 (one point); checked against an FP64 product on the
    # host with the reference's zero-value skip (src/qmckl_mo_sycl.cpp:40)
    rng = np.random.default_rng(11)
    P, A, M = 257, 2048, 1024
    ao = rng.normal(size=(P, 5, A))
    ao[:, 0, ::7] = 0.0  # AOs whose value is zero: their derivative rows are dropped too
    coef = rng.normal(size=(M, A)) / np.sqrt(A)
    masked = ao.copy()
    masked[:, 1:, :] *= (ao[:, :1, :] != 0.0)
    want = np.einsum("pca,ma->pcm", masked, coef)
    with Context(0) as ctx:
        d_ao, d_coef = ctx.upload(ao), ctx.upload(coef)
        out = ctx.buffer("out", 8 * 5 * P * M)
        f = ctx.L.qmckl_mo_contract_split_bf16_noalloc_device
        for call in range(2):
            _nan_fill(ctx, out, 5 * P * M)
            assert f(d_ao.ptr, 5 * P, A, d_coef.ptr, M, 1, out.ptr, ctx.stream) == 0
            got = ctx.download(out.ptr, (P, 5, M))
            assert np.isfinite(got).all()
            errs = [normwise_rel_err(got[:, c:c + 1], want[:, c:c + 1]) for c in range(5)]
            assert max(errs) <= MIXED_RTOL, "call %d: %s" % (call, errs)


FIRST_CALLS_FROM_TWO_THREADS = r"""
import sys, threading
import numpy as np
sys.path.insert(0, sys.argv[1])
from qmckl_sycl_gb300 import Context
rng = np.random.default_rng(5)
rows, A, M = 640, 300, 96
ao = rng.normal(size=(rows, A))
coef = rng.normal(size=(M, A))
want = ao @ coef.T
ctx = Context(0)  # holds the test's own buffers only
d_ao, d_coef = ctx.upload(ao), ctx.upload(coef)
d_out = ctx.buffer("out", 8 * rows * M)
f = ctx.L.qmckl_mo_contract_split_bf16_noalloc_device
go = threading.Barrier(2)
rc = [None, None]
def run(i):
    go.wait()
    # identical inputs and output, one chunk: the two calls write the same values into the shared array
    rc[i] = f(d_ao.ptr, rows, A, d_coef.ptr, M, 0, d_out.ptr, None)
ts = [threading.Thread(target=run, args=(i,)) for i in range(2)]
for t in ts: t.start()
for t in ts: t.join()
got = ctx.download(d_out.ptr, (rows, M))
err = np.abs(got - want).max() / np.abs(want).max()
print("rc", rc, "err %.2e" % err)
sys.exit(0 if rc == [0, 0] and err <= 1e-6 else 1)
"""


def test_noalloc_first_calls_from_two_threads():
    # a fresh process, so that both threads make the library's first split-BF16 call (the
    # run-time resolution of the tensor-map encoder and the array's address happen then)
    import os
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", FIRST_CALLS_FROM_TWO_THREADS, root], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr


def test_noalloc_rejects_sizes_beyond_its_array():
    with Context(0) as ctx:
        buf = ctx.buffer("b", 64)
        f = ctx.L.qmckl_mo_contract_split_bf16_noalloc_device
        assert f(buf.ptr, 5, 4096, buf.ptr, 8, 1, buf.ptr, ctx.stream) == 3  # ao_num > 2048
        assert f(buf.ptr, 5, 8, buf.ptr, 2000, 1, buf.ptr, ctx.stream) == 5  # mo_num > 1024
        assert f(buf.ptr, 7, 8, buf.ptr, 8, 1, buf.ptr, ctx.stream) == 2  # vgl rows not a multiple of 5
        assert f(None, 5, 8, buf.ptr, 8, 1, buf.ptr, ctx.stream) == 1

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


def test_noalloc_rejects_sizes_beyond_its_array():
    with Context(0) as ctx:
        buf = ctx.buffer("b", 64)
        f = ctx.L.qmckl_mo_contract_split_bf16_noalloc_device
        assert f(buf.ptr, 5, 4096, buf.ptr, 8, 1, buf.ptr, ctx.stream) == 3  # ao_num > 2048
        assert f(buf.ptr, 5, 8, buf.ptr, 2000, 1, buf.ptr, ctx.stream) == 5  # mo_num > 1024
        assert f(buf.ptr, 7, 8, buf.ptr, 8, 1, buf.ptr, ctx.stream) == 2  # vgl rows not a multiple of 5
        assert f(None, 5, 8, buf.ptr, 8, 1, buf.ptr, ctx.stream) == 1

"""Adjoint form on the GPU: gradients of L = sum(W * mo_vgl) with respect to the MO
coefficients, the primitive exponents and the point coordinates through
qmckl_vjp_mo_vgl_device, against the oracle's FP64 reference gradient (normwise 1e-10: both
are FP64, summed in different orders) and against central differences of the oracle's forward
path (h = 1e-5, normwise 1e-7)."""

import numpy as np
import pytest

from oracle import oracle
from qmckl_sycl_gb300 import PRECISION_SPLIT_BF16, Context, config_adjoint, config_small
from qmckl_sycl_gb300.systems import make_system

pytestmark = pytest.mark.gpu

REF_RTOL = 1e-10
FD_RTOL = 1e-7
H = 1e-5


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def gpu_vjp(s, w, **kw):
    with Context(0) as ctx:
        ctx.load_system(s)
        return ctx.vjp_mo_vgl(w, prim_num=s.prim_num, **kw)


def weights(s, seed=0):
    return np.random.default_rng(seed).normal(size=(s.point_num, 5, s.mo_num))


def loss_per_point(s, w):
    return (w * oracle.forward(s, want=("mo_vgl",))["mo_vgl"]).sum(axis=(1, 2))


def replace(s, **kw):
    return s.__class__(**{**s.__dict__, **kw})


@pytest.fixture(scope="module")
def adjoint_case():
    s = config_adjoint(0)
    return s, weights(s, 5)


def test_adjoint_config_matches_reference_gradient(adjoint_case):
    s, w = adjoint_case
    g = gpu_vjp(s, w)
    ref = oracle.vjp_mo_vgl(s, w)
    for k in ("coef", "expo", "coord"):
        print("%s: rel err vs FP64 reference gradient %.2e" % (k, rel(g[k], ref[k])))
        assert rel(g[k], ref[k]) <= REF_RTOL, k


def test_adjoint_config_matches_central_differences(adjoint_case):
    s, w = adjoint_case
    g = gpu_vjp(s, w)
    fd = np.zeros_like(g["coord"])
    for j in range(3):  # each point's loss depends on its own coordinates only
        e = np.zeros(3)
        e[j] = H
        fd[:, j] = (loss_per_point(s.with_points(s.coord + e), w) -
                    loss_per_point(s.with_points(s.coord - e), w)) / (2 * H)
    assert rel(g["coord"], fd) <= FD_RTOL
    # exponents: every primitive, on a 128-point subset (2 x prim_num forward passes)
    idx = np.arange(0, s.point_num, 16)
    sub = s.with_points(s.coord[idx])
    wsub = np.ascontiguousarray(w[idx])
    ge = gpu_vjp(sub, wsub, want=("expo",))["expo"]
    fde = np.zeros(s.prim_num)
    for k in range(s.prim_num):
        ep = s.exponent.copy()
        ep[k] += H
        em = s.exponent.copy()
        em[k] -= H
        fde[k] = (loss_per_point(replace(sub, exponent=ep), wsub).sum() -
                  loss_per_point(replace(sub, exponent=em), wsub).sum()) / (2 * H)
    assert rel(ge, fde) <= FD_RTOL
    # coefficients (L is linear in C) and all exponents along random directions, full size
    rng = np.random.default_rng(9)
    d = rng.normal(size=g["coef"].shape)
    dl = (loss_per_point(replace(s, mo_coef=s.mo_coef + H * d), w).sum() -
          loss_per_point(replace(s, mo_coef=s.mo_coef - H * d), w).sum()) / (2 * H)
    assert abs(dl - (g["coef"] * d).sum()) <= FD_RTOL * np.abs(g["coef"] * d).sum()
    d = rng.normal(size=s.prim_num)
    dl = (loss_per_point(replace(s, exponent=s.exponent + H * d), w).sum() -
          loss_per_point(replace(s, exponent=s.exponent - H * d), w).sum()) / (2 * H)
    assert abs(dl - (g["expo"] * d).sum()) <= FD_RTOL * np.abs(g["expo"] * d).sum()


@pytest.mark.parametrize("name", ["chbrclf", "small_on_nucleus", "g_shells"])
def test_other_bases_match_reference_gradient(name, chbrclf):
    if name == "chbrclf":
        s = chbrclf
    elif name == "small_on_nucleus":
        s = config_small(2, point_num=40)
        coord = s.coord.copy()
        coord[0] = s.nucl_coord[:, 0]  # p/d components vanish there: the zero-value skip acts
        coord[1] = s.nucl_coord[:, 1]
        s = s.with_points(coord)
    else:  # l up to 5: the adjoint's run-time-exponent path
        s = make_system(11, 5, 8, 5.0, 40, (0.3, 0.2, 0.2, 0.1, 0.1, 0.1), 4, (0.1, 20.0), 30, 96, 1.5, name="g")
    w = weights(s, 1)
    g = gpu_vjp(s, w)
    ref = oracle.vjp_mo_vgl(s, w)
    for k in ("coef", "expo", "coord"):
        assert rel(g[k], ref[k]) <= REF_RTOL, (name, k, rel(g[k], ref[k]))


def test_deterministic_and_independent_of_precision_mode(adjoint_case):
    s, w = adjoint_case
    with Context(0) as ctx:
        ctx.load_system(s)
        a = ctx.vjp_mo_vgl(w, prim_num=s.prim_num)
        b = ctx.vjp_mo_vgl(w, prim_num=s.prim_num)
        ctx.set_precision(PRECISION_SPLIT_BF16)
        c = ctx.vjp_mo_vgl(w, prim_num=s.prim_num)
    for k in a:
        assert np.array_equal(a[k], b[k]) and np.array_equal(a[k], c[k]), k


def test_device_pointers_and_partial_requests(adjoint_case):
    s, w = adjoint_case
    with Context(0) as ctx:
        ctx.load_system(s)
        host = ctx.vjp_mo_vgl(w, prim_num=s.prim_num)
        wd = ctx.upload(w)
        dc = ctx.buffer("dc", 8 * s.mo_num * s.ao_num)
        de = ctx.buffer("de", 8 * s.prim_num)
        dx = ctx.buffer("dx", 8 * 3 * s.point_num)
        ctx.call("vjp_mo_vgl", wd.ptr, w.size, dc.ptr, s.mo_num * s.ao_num, de.ptr, s.prim_num, dx.ptr,
                 3 * s.point_num)
        dev = dict(coef=ctx.download(dc.ptr, (s.mo_num, s.ao_num)), expo=ctx.download(de.ptr, (s.prim_num,)),
                   coord=ctx.download(dx.ptr, (s.point_num, 3)))
        only = ctx.vjp_mo_vgl(w, want=("expo",), prim_num=s.prim_num)
        # argument checks
        with pytest.raises(Exception) as e:
            ctx.call("vjp_mo_vgl", wd.ptr, w.size - 1, dc.ptr, s.mo_num * s.ao_num, None, 0, None, 0)
        assert e.value.code == 3
        with pytest.raises(Exception) as e:
            ctx.call("vjp_mo_vgl", wd.ptr, w.size, None, 0, de.ptr, s.prim_num - 1, None, 0)
        assert e.value.code == 7
    for k in host:
        assert np.array_equal(host[k], dev[k]), k
    assert np.array_equal(only["expo"], host["expo"])


def test_ao_level_vjp_equals_mo_level_without_mask(adjoint_case):
    s, w = adjoint_case
    with Context(0) as ctx:
        ctx.load_system(s)
        # AO values that are exactly zero here are screened ones, whose derivatives vanish too,
        # so the MO kernel's zero-value mask changes nothing on this workload
        gbar = np.einsum("plm,ma->pla", w, s.mo_coef)
        a = ctx.vjp_ao_vgl(gbar, prim_num=s.prim_num)
        m = ctx.vjp_mo_vgl(w, want=("expo", "coord"), prim_num=s.prim_num)
    for k in a:
        assert rel(a[k], m[k]) <= 1e-12, k

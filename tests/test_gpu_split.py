"""Precision form: MO contraction as a split-BF16 product on the tcgen05 tensor cores
(three BF16 terms per FP64 operand, six cross products, FP32 accumulation). Target:
MO vgl within 1e-6 relative of the FP64 oracle, normwise per component; the AO arrays
(FP64 throughout) stay within the FP64 tolerance."""
import numpy as np
import pytest

from conftest import normwise_rel_err
from oracle import oracle
from qmckl_sycl_gb300 import PRECISION_FP64, PRECISION_SPLIT_BF16, Context, config_adjoint, config_medium, config_small

pytestmark = pytest.mark.gpu

MIXED_RTOL = 1e-6


def run(s, mode):
    with Context(0) as ctx:
        ctx.load_system(s)
        ctx.set_precision(mode)
        P = s.point_num
        return dict(ao_vgl=ctx.get_ao_vgl(P), mo_vgl=ctx.get_mo_vgl(P), mo_value=ctx.get_mo_value(P))


def _replace(s, **kw):
    return s.__class__(**{**s.__dict__, **kw})


def _unfoldable():
    # a coefficient outside the folded evaluation's range (binary exponent beyond +-64): the planes
    # kernel evaluates the radials like the FP64 form
    s = config_small(6, point_num=200)
    c = s.coefficient.copy()
    c[3] = 1e-300
    return _replace(s, coefficient=c)


def _signed():
    # negative and zero coefficients (the folded evaluation's sign bit and never-active entries)
    s = config_small(8, point_num=200)
    c = s.coefficient.copy()
    c[1::3] *= -1.0
    c[::11] = 0.0
    return _replace(s, coefficient=c)


@pytest.mark.parametrize("name", ["chbrclf", "small", "adjoint", "medium_sub", "unfoldable", "signed"])
def test_split_mo_vgl_within_1e6(name, chbrclf):
    s = {"chbrclf": lambda: chbrclf, "small": lambda: config_small(0), "adjoint": lambda: config_adjoint(0),
         "medium_sub": lambda: config_medium(0, walkers=8, electrons=160), "unfoldable": _unfoldable,
         "signed": _signed}[name]()
    ref = oracle.forward(s, want=("ao_vgl", "mo_vgl", "mo_value"))
    out = run(s, PRECISION_SPLIT_BF16)
    assert normwise_rel_err(out["ao_vgl"], ref["ao_vgl"]) <= 1e-12
    errs = [normwise_rel_err(out["mo_vgl"][:, c:c + 1], ref["mo_vgl"][:, c:c + 1]) for c in range(5)]
    print("%s split-BF16 mo_vgl normwise rel err per component: %s" % (name, " ".join("%.2e" % e for e in errs)))
    assert max(errs) <= MIXED_RTOL
    assert normwise_rel_err(out["mo_value"], ref["mo_value"]) <= MIXED_RTOL


def test_split_respects_zero_value_skip():
    s = config_small(4, point_num=8)
    coord = s.coord.copy()
    coord[:, 0] = s.nucl_coord[0, 0]
    s = s.with_points(coord)
    ref = oracle.forward(s, want=("mo_vgl",))
    out = run(s, PRECISION_SPLIT_BF16)
    assert normwise_rel_err(out["mo_vgl"], ref["mo_vgl"]) <= MIXED_RTOL


def test_split_tiny_displacements():
    # Displacements below 2^-340 can underflow the FP64 polynomial x^a (y^b z^c), which the
    # reference's zero-value skip tests (src/qmckl_mo_sycl.cpp:40); the split form then decides
    # that skip from the FP64 product itself (a warp-uniform branch) instead of the displacements'
    # zero tests. Nucleus 0 sits on the plane x = 0 so that the displacements are the points' own
    # tiny coordinates: 1e-200, 3e-300 and a subnormal one, mixed with ordinary points in one warp.
    s = config_small(4, point_num=64)
    nc = s.nucl_coord.copy()
    nc[0, 0] = 0.0
    coord = s.coord.copy()
    coord[:16, 0] = 1e-200
    coord[16:24, 0] = -3e-300
    coord[24:28, 0] = 5e-320
    coord[28:32, 0] = 0.0
    s = _replace(s, nucl_coord=nc).with_points(coord)
    ref = oracle.forward(s, want=("ao_vgl", "mo_vgl", "mo_value"))
    plain = run(s, PRECISION_FP64)
    assert np.array_equal(plain["ao_vgl"] == 0.0, ref["ao_vgl"] == 0.0)
    assert normwise_rel_err(plain["mo_vgl"], ref["mo_vgl"]) <= 1e-12
    out = run(s, PRECISION_SPLIT_BF16)
    errs = [normwise_rel_err(out["mo_vgl"][:, c:c + 1], ref["mo_vgl"][:, c:c + 1]) for c in range(5)]
    assert max(errs) <= MIXED_RTOL
    assert normwise_rel_err(out["mo_value"], ref["mo_value"]) <= MIXED_RTOL


def test_mode_switch_recomputes(chbrclf):
    s = chbrclf
    with Context(0) as ctx:
        ctx.load_system(s)
        a = ctx.get_mo_vgl(s.point_num)
        ctx.set_precision(PRECISION_SPLIT_BF16)
        b = ctx.get_mo_vgl(s.point_num)
        ctx.set_precision(PRECISION_FP64)
        c = ctx.get_mo_vgl(s.point_num)
    assert not np.array_equal(a, b)  # the split product rounds differently
    assert np.array_equal(a, c)
    assert normwise_rel_err(b, a) <= MIXED_RTOL


@pytest.mark.parametrize("mo_num", [1, 17, 160, 161, 333])
def test_split_tile_edges(mo_num):
    s = config_small(9, point_num=77)
    rng = np.random.default_rng(mo_num)
    s = s.__class__(**{**s.__dict__, "mo_num": mo_num, "mo_coef": rng.normal(0, 1 / np.sqrt(s.ao_num),
                                                                              size=(mo_num, s.ao_num))})
    ref = oracle.forward(s, want=("mo_vgl",))
    out = run(s, PRECISION_SPLIT_BF16)
    assert normwise_rel_err(out["mo_vgl"], ref["mo_vgl"]) <= MIXED_RTOL


def test_host_getter_overlaps_copies_bitwise():
    # >= 16384 points and a host buffer: computed in point-range chunks whose rows are copied to
    # the host while the next chunk computes; the result must equal the one-pass device result
    import ctypes

    s = config_medium(0, walkers=104, electrons=160)  # 16640 points
    with Context(0) as ctx:
        ctx.load_system(s)
        ctx.set_precision(PRECISION_SPLIT_BF16)
        P, M = s.point_num, s.mo_num
        host = ctx.get_mo_vgl(P)  # pipelined path (numpy buffer is host memory)
        dev = ctx.buffer("mo", 8 * 5 * P * M)
        ctx.call("get_mo_basis_mo_vgl_inplace", dev.ptr, 5 * P * M)  # one pass, device buffer
        one_pass = ctx.download(dev.ptr, (P, 5, M))
        again = ctx.get_mo_vgl(P)  # cached: plain copy
    assert np.array_equal(host, one_pass)
    assert np.array_equal(again, host)
    idx = np.arange(0, P, 97)
    ref = oracle.forward(s.with_points(s.coord[idx]), want=("mo_vgl",))["mo_vgl"]
    assert normwise_rel_err(host[idx], ref) <= MIXED_RTOL


@pytest.mark.parametrize("mo_num, point_num", [(161, 16411), (97, 20003), (333, 16416)])
def test_host_getter_wave_sized_ranges_bitwise(mo_num, point_num):
    # the host-buffer path's ranges are sized by the contraction's tile waves, which depend on the
    # MO count's column tiles (161: two of 96; 97: one; 333: three of 112); a point count that is
    # not a multiple of 32 leaves a ragged last range. Every layout gives the one-pass bits.
    import ctypes

    from qmckl_sycl_gb300.systems import SPDF_WEIGHTS, make_system

    s = make_system(5, 12, 10, 9.0, 160, SPDF_WEIGHTS, 5, (0.05, 60.0), mo_num, point_num, 2.0, name="waves")
    with Context(0) as ctx:
        ctx.load_system(s)
        ctx.set_precision(PRECISION_SPLIT_BF16)
        P, M = s.point_num, s.mo_num
        host = ctx.get_mo_vgl(P)
        dev = ctx.buffer("mo", 8 * 5 * P * M)
        ctx.call("get_mo_basis_mo_vgl_inplace", dev.ptr, 5 * P * M)
        one_pass = ctx.download(dev.ptr, (P, 5, M))
    assert np.array_equal(host, one_pass)
    idx = np.arange(0, P, 211)
    ref = oracle.forward(s.with_points(s.coord[idx]), want=("mo_vgl",))["mo_vgl"]
    assert normwise_rel_err(host[idx], ref) <= MIXED_RTOL


def test_split_zero_and_tiny_mo_columns():
    # an MO whose coefficients are all zero gives exact zeros (the epilogue's float-to-double
    # conversion of zeros), an MO scaled by 1e-20 keeps its own relative accuracy (the BF16 terms
    # carry FP32's exponent range), and a 17-column tail checks the ragged last tile
    s = config_small(3, point_num=300)
    c = s.mo_coef.copy()
    c[0] = 0.0
    c[1] *= 1e-20
    c[2] *= -3e12
    s = _replace(s, mo_coef=np.ascontiguousarray(c))
    ref = oracle.forward(s, want=("mo_vgl",))["mo_vgl"]
    got = run(s, PRECISION_SPLIT_BF16)["mo_vgl"]
    assert np.all(ref[:, :, 0] == 0.0)
    assert np.array_equal(got[:, :, 0], np.zeros_like(got[:, :, 0]))
    for m in (1, 2, 3):
        for comp in range(5):
            assert normwise_rel_err(got[:, comp, m], ref[:, comp, m]) <= MIXED_RTOL, (m, comp)

"""Parity of the CUDA path (through the C ABI) with the CPU oracle and the reference's
golden data. Tolerance: the FP64 form must match within 1e-12 relative, normwise per
vgl component (max |gpu - oracle| / max |oracle| over each of value, d/dx, d/dy, d/dz,
Laplacian), with identical screening decisions (identical zero patterns)."""
import ctypes

import numpy as np
import pytest

from conftest import normwise_rel_err
from oracle import oracle
from qmckl_sycl_gb300 import Context, QmcklError, config_adjoint, config_medium, config_small
from qmckl_sycl_gb300.systems import with_empty_nucleus

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def run_all(s, inplace=False):
    with Context(0) as ctx:
        ctx.load_system(s)
        P = s.point_num
        out = dict(ao_vgl=ctx.get_ao_vgl(P, inplace), ao_value=ctx.get_ao_value(P, inplace),
                   mo_vgl=ctx.get_mo_vgl(P, inplace), mo_value=ctx.get_mo_value(P, inplace))
    return out


def check(out, ref, keys=("ao_vgl", "ao_value", "mo_vgl", "mo_value")):
    for k in keys:
        assert out[k].shape == ref[k].shape, k
        err = normwise_rel_err(out[k], ref[k])
        assert err <= RTOL, "%s normwise rel err %.3e" % (k, err)
    for k in ("ao_vgl", "ao_value"):
        if k in keys:
            assert np.array_equal(out[k] == 0.0, ref[k] == 0.0), "%s screening pattern differs" % k


@pytest.mark.parametrize("name", ["chbrclf", "small", "adjoint", "medium_sub", "small_empty_nucleus"])
def test_forward_matches_oracle(name, chbrclf):
    s = {"chbrclf": lambda: chbrclf, "small": lambda: config_small(0), "adjoint": lambda: config_adjoint(0),
         "medium_sub": lambda: config_medium(0, walkers=16, electrons=160),
         "small_empty_nucleus": lambda: with_empty_nucleus(config_small(0), 3)}[name]()
    ref = oracle.forward(s)
    check(run_all(s), ref)


def test_golden_mo_vgl_and_known_answers(chbrclf, golden):
    out = run_all(chbrclf)
    ref = golden["mo_vgl_ref"]
    # the reference's own check (tests/test_qmckl_mo.cpp:401) is 1e-14 absolute with its
    # sequential sum; a tensor-core sum in a different order stays within a few ulps.
    worst = np.abs(out["mo_vgl"] - ref).max()
    print("golden mo_vgl: max abs difference %.3e over %d values (bound 5e-14)" % (worst, ref.size))
    assert worst <= 5e-14
    assert normwise_rel_err(out["mo_vgl"], ref) <= RTOL
    for p, c, a, v in golden["kat_ao_vgl"]:
        assert abs(out["ao_vgl"][int(p), int(c), int(a)] - v) <= float(golden["kat_ao_vgl_tol"])
    for p, a, v in golden["kat_ao_value"]:
        assert abs(out["ao_value"][int(p), int(a)] - v) <= float(golden["kat_ao_value_tol"])
    assert np.abs(out["mo_value"] - out["mo_vgl"][:, 0, :]).max() <= 1e-12


def test_inplace_getters_match(chbrclf):
    a = run_all(chbrclf)
    b = run_all(chbrclf, inplace=True)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_shell_vgl_matches_oracle(chbrclf):
    ref = oracle.shell_vgl(chbrclf)
    with Context(0) as ctx:
        ctx.load_system(chbrclf)
        got = ctx.get_shell_vgl(chbrclf.point_num, chbrclf.shell_num)
    assert normwise_rel_err(got, ref) <= RTOL
    assert np.array_equal(got == 0, ref == 0)


@pytest.mark.parametrize("P", [1, 31, 33, 97])
def test_ragged_point_counts(P):
    s = config_small(1, point_num=P)
    check(run_all(s), oracle.forward(s))


def test_points_far_away_are_screened_to_zero():
    s = config_small(2, point_num=40)
    coord = s.coord.copy()
    coord[::2] += 500.0  # every nucleus screened for these points
    s = s.with_points(coord)
    out = run_all(s)
    ref = oracle.forward(s)
    check(out, ref)
    assert np.all(out["ao_vgl"][::2] == 0.0) and np.all(out["mo_vgl"][::2] == 0.0)


@pytest.mark.parametrize("mode", [0, 1])
def test_nan_coordinates_propagate_like_the_reference(mode):
    # The reference's screening tests are false for a NaN r2, so it screens nothing for a NaN
    # coordinate and every AO (and hence every MO) of that point is NaN
    # (src/qmckl_ao_sycl.cpp:53,72-75; src/qmckl_mo_sycl.cpp:40 keeps NaN values); the other
    # points are unaffected. Both precision forms, and the shell radials' getter.
    from test_oracle_golden import nan_points

    s = nan_points(config_small(9, point_num=40))
    ref = oracle.forward(s)
    ref["shell_vgl"] = oracle.shell_vgl(s)
    with Context(0) as ctx:
        ctx.load_system(s)
        ctx.set_precision(mode)
        P = s.point_num
        out = dict(ao_vgl=ctx.get_ao_vgl(P), ao_value=ctx.get_ao_value(P), mo_vgl=ctx.get_mo_vgl(P),
                   mo_value=ctx.get_mo_value(P), shell_vgl=ctx.get_shell_vgl(P, s.shell_num))
    for k in out:
        assert np.array_equal(np.isnan(out[k]), np.isnan(ref[k])), k
        tol = RTOL if mode == 0 or k in ("ao_vgl", "ao_value", "shell_vgl") else 1e-6
        assert normwise_rel_err(np.nan_to_num(out[k]), np.nan_to_num(ref[k])) <= tol, k
    assert np.isnan(out["mo_vgl"][[3, 7, 12]]).all()
    assert np.array_equal(out["ao_vgl"] == 0.0, ref["ao_vgl"] == 0.0)


def _g_shells():
    # angular momenta up to 5: the fused kernels' generic (run-time exponent) path. The reference
    # built on the host corrupts its heap on l >= 4 inputs, so the oracle alone pins this case.
    from qmckl_sycl_gb300.systems import make_system

    return make_system(11, 5, 8, 5.0, 40, (0.3, 0.2, 0.2, 0.1, 0.1, 0.1), 4, (0.1, 20.0), 30, 96, 1.5, name="g")


@pytest.mark.parametrize("name", ["g_shells", "g_shells_nan", "zero_prim", "zero_prim_nan"])
@pytest.mark.parametrize("mode", [0, 1])
def test_high_l_and_zero_primitive_shells(name, mode):
    from test_oracle_golden import nan_points, zero_prim_shells

    s = _g_shells() if name.startswith("g_shells") else zero_prim_shells(config_small(12, point_num=64))
    if name.endswith("_nan"):
        s = nan_points(s)
    ref = oracle.forward(s)
    with Context(0) as ctx:
        ctx.load_system(s)
        ctx.set_precision(mode)
        P = s.point_num
        out = dict(ao_vgl=ctx.get_ao_vgl(P), ao_value=ctx.get_ao_value(P), mo_vgl=ctx.get_mo_vgl(P),
                   mo_value=ctx.get_mo_value(P))
    for k in out:
        assert np.array_equal(np.isnan(out[k]), np.isnan(ref[k])), k
        tol = RTOL if mode == 0 or k.startswith("ao") else 1e-6
        assert normwise_rel_err(np.nan_to_num(out[k]), np.nan_to_num(ref[k])) <= tol, (k, name)
    assert np.array_equal(out["ao_vgl"] == 0.0, ref["ao_vgl"] == 0.0)


def test_mo_skips_zero_valued_aos_like_the_reference():
    # A point on the plane x = X_n of a nucleus makes that nucleus' p_x value exactly 0
    # while its x-derivative is not; the reference drops such AOs from the MO sum for all
    # components (src/qmckl_mo_sycl.cpp:40).
    s = config_small(4, point_num=8)
    coord = s.coord.copy()
    coord[:, 0] = s.nucl_coord[0, 0]
    coord[:, 1] = s.nucl_coord[1, 1]
    s = s.with_points(coord)
    ref = oracle.forward(s)
    out = run_all(s)
    check(out, ref)
    zero_val = (ref["ao_vgl"][:, 0, :] == 0) & (np.abs(ref["ao_vgl"][:, 1:, :]).max(axis=1) > 0)
    assert zero_val.any()  # the case is exercised


def test_set_point_resizes_and_recomputes(chbrclf):
    s1 = config_small(5, point_num=64)
    s2 = config_small(5, point_num=200)
    with Context(0) as ctx:
        ctx.load_system(s1)
        m1 = ctx.get_mo_vgl(64)
        ctx.set_point(s2.coord)
        m2 = ctx.get_mo_vgl(200)
        ctx.set_point(s1.coord[:10], transp="N", host=True)
        m3 = ctx.get_mo_vgl(10)
        ctx.set_point(np.ascontiguousarray(s1.coord[:10].T), transp="T")
        m4 = ctx.get_mo_vgl(10)
    assert normwise_rel_err(m1, oracle.forward(s1)["mo_vgl"]) <= RTOL
    assert normwise_rel_err(m2, oracle.forward(s2)["mo_vgl"]) <= RTOL
    assert np.array_equal(m3, m1[:10]) and np.array_equal(m4, m1[:10])


def test_cache_dates(chbrclf):
    with Context(0) as ctx:
        ctx.load_system(chbrclf)
        ctx.get_mo_vgl(chbrclf.point_num)
        n0 = ctx.launch_count()
        ctx.get_mo_vgl(chbrclf.point_num)  # cached: no kernel
        assert ctx.launch_count() == n0
        ctx.touch()
        ctx.get_mo_vgl(chbrclf.point_num)
        assert ctx.launch_count() > n0
        n1 = ctx.launch_count()
        ctx.get_mo_value(chbrclf.point_num)  # copied from the fresh mo_vgl (src/qmckl_mo.cpp:232)
        assert ctx.launch_count() == n1 + 1


def test_electron_walker_api(chbrclf):
    ec = chbrclf.coord.reshape(2, 68, 3)
    with Context(0) as ctx:
        ctx.load_system(chbrclf, points=False)
        ctx.call("set_electron_num", 34, 34)
        d = ctx.upload(ec)
        ctx.call("set_electron_coord", b"N", 2, d.ptr, 3 * 136)
        mo = ctx.get_mo_vgl(136)
        back = np.empty((136, 3))
        ctx.call("get_electron_coord", b"N", back.ctypes.data_as(ctypes.c_void_p), back.size)
    assert np.array_equal(back, chbrclf.coord)
    assert normwise_rel_err(mo, oracle.forward(chbrclf)["mo_vgl"]) <= RTOL


def test_getters_round_trip(chbrclf):
    s = chbrclf
    with Context(0) as ctx:
        ctx.load_system(s)
        e = np.empty(s.prim_num)
        ctx.call("get_ao_basis_exponent", e.ctypes.data_as(ctypes.c_void_p), s.prim_num)
        assert np.array_equal(e, s.exponent)
        li = np.empty(s.shell_num, np.int32)
        ctx.call("get_ao_basis_shell_ang_mom", li.ctypes.data_as(ctypes.c_void_p), s.shell_num)
        assert np.array_equal(li, s.shell_ang_mom)
        nc = np.empty((s.nucl_num, 3))
        ctx.call("get_nucleus_coord", b"N", nc.ctypes.data_as(ctypes.c_void_p), nc.size)
        assert np.array_equal(nc, s.nucl_coord.T)
        fin = oracle.finalize(s)
        nr = np.empty(s.nucl_num)
        ctx.call("get_ao_basis_nucleus_range", nr.ctypes.data_as(ctypes.c_void_p), s.nucl_num)
        assert np.array_equal(nr, fin["nucleus_range"])
        cn = np.empty(s.prim_num)
        ctx.call("get_ao_basis_coefficient_normalized", cn.ctypes.data_as(ctypes.c_void_p), s.prim_num)
        assert np.array_equal(cn, fin["coefficient_normalized"])
        mm = np.empty(s.nucl_num, np.int32)
        ctx.call("get_ao_basis_nucleus_max_ang_mom", mm.ctypes.data_as(ctypes.c_void_p), s.nucl_num)
        assert np.array_equal(mm, fin["nucleus_max_ang_mom"])


def test_device_errors_and_size_checks(chbrclf):
    s = chbrclf
    with Context(0) as ctx:
        ctx.load_system(s)
        small = np.empty(10)
        with pytest.raises(QmcklError) as e:
            ctx.call("get_mo_basis_mo_vgl", small.ctypes.data_as(ctypes.c_void_p), 10)
        assert e.value.code == 3
        with pytest.raises(QmcklError) as e:
            ctx.call("get_ao_basis_ao_vgl_inplace", small.ctypes.data_as(ctypes.c_void_p), 10)
        assert e.value.code == 3
        with pytest.raises(QmcklError) as e:
            ctx.call("set_mo_basis_mo_num", 5)
        assert e.value.code == 108
        with pytest.raises(QmcklError) as e:
            ctx.call("set_nucleus_coord", b"T", ctx.upload(s.nucl_coord).ptr, 3 * s.nucl_num)
        assert e.value.code == 108


def test_inconsistent_ao_num_is_rejected(chbrclf):
    s = chbrclf
    with Context(0) as ctx:
        ctx.set_nucleus(s)
        bad = s.__class__(**{**s.__dict__, "ao_num": s.ao_num + 1, "ao_factor": np.ones(s.ao_num + 1)})
        with pytest.raises(QmcklError) as e:
            ctx.set_ao_basis(bad)
        assert e.value.code == 101


def test_allocation_failure_hook(chbrclf):
    with Context(0) as ctx:
        ctx.load_system(chbrclf)
        ctx.call("set_allocation_failure", 1)  # the next device allocation fails
        out = np.empty((chbrclf.point_num, 5, chbrclf.ao_num))
        with pytest.raises(QmcklError) as e:
            ctx.call("get_ao_basis_ao_vgl", out.ctypes.data_as(ctypes.c_void_p), out.size)
        assert e.value.code == 104
        ao = ctx.get_ao_vgl(chbrclf.point_num)  # recovers
    assert normwise_rel_err(ao, oracle.forward(chbrclf, want=("ao_vgl",))["ao_vgl"]) <= RTOL


def test_select_mo(chbrclf):
    s = chbrclf
    keep = np.zeros(s.mo_num, np.int32)
    keep[::3] = 1
    with Context(0) as ctx:
        ctx.load_system(s)
        full = ctx.get_mo_vgl(s.point_num)
        failed = ctx.L.qmckl_mo_basis_select_mo_device(ctx.handle, keep.ctypes.data_as(ctypes.c_void_p), s.mo_num)
        assert not failed
        assert ctx.mo_num == int(keep.sum())
        ctx.touch()
        sub = ctx.get_mo_vgl(s.point_num)
    assert normwise_rel_err(sub, full[:, :, ::3]) <= RTOL


def test_empty_point_set(chbrclf):
    with Context(0) as ctx:
        ctx.load_system(chbrclf, points=False)
        dummy = np.zeros(3)
        ctx.call("set_point", b"N", 0, dummy.ctypes.data_as(ctypes.c_void_p), 0)
        out = np.zeros(1)
        ctx.call("get_mo_basis_mo_vgl", out.ctypes.data_as(ctypes.c_void_p), 0)


def _ulps(a, b):
    # distance in units in the last place, for positive doubles (integer arithmetic on the
    # bit patterns: a float64 cast of ~2^62-sized integers would round to multiples of 512)
    return np.abs(np.ascontiguousarray(a).view(np.int64) - np.ascontiguousarray(b).view(np.int64))


def test_kernel_exponential_against_cuda_and_libm(chbrclf):
    # the fused AO kernel's table-driven e^-x on the screened range [0, 27.7]
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.uniform(0.0, 27.7, 1 << 20), np.linspace(0.0, 27.7, 4097), [0.0, 1e-300, 27.631021115928547]])
    with Context(0) as ctx:
        ctx.load_system(chbrclf, mo=False, points=False)
        dx = ctx.upload(x)
        out = ctx.buffer("exp_out", 16 * x.size)
        ctx.call("exp_check", ctypes.c_void_p(dx.ptr), x.size, ctypes.c_void_p(out.ptr))
        got = ctx.download(out.ptr, (x.size, 2))
    ours, cuda = got[:, 0], got[:, 1]
    libm = np.exp(-x)
    for name, other in (("cuda", cuda), ("libm", libm)):
        u = _ulps(ours, other)
        bad = np.argsort(u)[-5:]
        print("vs %s: max %d ulp; worst x %s ours %s other %s" % (
            name, u.max(), x[bad].tolist(), ours[bad].tolist(), other[bad].tolist()))
        print("   cuda vs libm at those x:", _ulps(cuda[bad], libm[bad]).tolist())
    assert _ulps(ours, cuda).max() <= 2
    assert _ulps(ours, libm).max() <= 2
    assert ours[x.size - 3] == 1.0


def test_point_order_does_not_change_results():
    # results depend only on each point, not on which points share a warp
    s = config_small(11, point_num=300)
    perm = np.random.default_rng(1).permutation(s.point_num)
    a = run_all(s)
    b = run_all(s.with_points(s.coord[perm]))
    for k in a:
        assert np.array_equal(a[k][perm], b[k]), k


def _prim_values(s, r2):
    with Context(0) as ctx:
        ctx.load_system(s, mo=False, points=False)
        d = ctx.upload(r2)
        out = ctx.buffer("prim_out", 8 * r2.size * s.prim_num)
        ctx.call("prim_value_check", ctypes.c_void_p(d.ptr), r2.size, ctypes.c_void_p(out.ptr), r2.size * s.prim_num)
        return ctx.download(out.ptr, (r2.size, s.prim_num))


def _replace(s, **kw):
    return s.__class__(**{**s.__dict__, **kw})


@pytest.mark.parametrize("name", ["chbrclf", "medium", "signs_and_zeros", "extreme_coefficient"])
def test_split_form_primitive_values(name, chbrclf):
    # the split-BF16 form's AO kernel evaluates coef * e^(-expo r2) with the coefficient folded
    # into the exponential, in FP32 pair arithmetic; its values against long double, and its
    # screening against the reference's test expo * r2 > 27.631021115928547 (bit-identical zero
    # pattern)
    s = chbrclf if name == "chbrclf" else config_small(3) if name != "medium" else config_medium(0, 1, 2)
    if name == "signs_and_zeros":
        c = s.coefficient.copy()
        c[::7] = 0.0
        c[1::5] *= -1.0
        s = _replace(s, coefficient=c)
    elif name == "extreme_coefficient":  # outside the folded range: the FP64 form's evaluation
        c = s.coefficient.copy()
        c[2] = 1e-300
        s = _replace(s, coefficient=c)
    rng = np.random.default_rng(4)
    rmax = 27.7 / s.exponent.min()
    r2 = np.concatenate([rng.uniform(0.0, rmax, 1000), np.exp(rng.uniform(-12, np.log(rmax), 1000)), [0.0]])
    got = _prim_values(s, r2)
    cn = oracle.finalize(s)["coefficient_normalized"]
    ar2 = s.exponent[None, :] * r2[:, None]
    screened = ar2 > 27.631021115928547
    # long double reference (x87 extended or IEEE quad, depending on the host)
    exact = (cn.astype(np.longdouble)[None, :] * np.exp(-(s.exponent.astype(np.longdouble)[None, :] *
                                                            r2.astype(np.longdouble)[:, None])))
    want = np.where(screened, 0.0, exact.astype(np.float64))
    assert np.array_equal(got == 0.0, want == 0.0)
    ok = np.abs(want) > 1e-290  # normal results
    rel = (np.abs(got[ok] - exact[ok]) / np.abs(exact[ok])).astype(np.float64)
    # folded evaluation in FP32 pair arithmetic (~44 significant bits): within 2e-10 relative; the
    # FP64 form's evaluation (a coefficient outside the folded range): the argument's rounding
    # (|expo r2| ulp / 2) plus a few units of 1e-16
    bound = 1.2e-16 * ar2[ok] + 6e-16 if name == "extreme_coefficient" else np.full(rel.shape, 2e-10)
    print("%s: max rel err %.2e, max err / bound %.2f" % (name, rel.max(), (rel / bound).max()))
    assert (rel <= bound).all()


def _hpc_case(name, chbrclf):
    if name == "chbrclf":
        return chbrclf
    s = config_small(2 if name == "shared_exponents" else 3)
    if name == "shared_exponents":  # many equal exponents within nuclei and within shells
        return _replace(s, exponent=np.round(s.exponent) + 1.0)
    nsh, nidx = s.nucleus_shell_num.copy(), s.nucleus_index.copy()  # nucleus 1 without shells
    nsh[0] += nsh[1]
    nsh[1] = 0
    nidx[1] = nidx[2]
    return _replace(s, nucleus_shell_num=nsh, nucleus_index=nidx)


@pytest.mark.parametrize("name", ["chbrclf", "shared_exponents", "empty_nucleus"])
def test_finalize_hpc_tables_match_oracle(name, chbrclf):
    # per-nucleus exponent tables (src/qmckl_ao_sycl.cpp:855-1065), bit for bit
    s = _hpc_case(name, chbrclf)
    ref = oracle.finalize_hpc(s)
    N = s.nucl_num
    with Context(0) as ctx:
        ctx.load_system(s, mo=False, points=False)
        for rep in range(2):  # built by the finalize, then rebuilt by the explicit call
            pm, sm = ctypes.c_int64(0), ctypes.c_int64(0)
            ctx.call("get_ao_basis_hpc_dims", ctypes.byref(pm), ctypes.byref(sm))
            pm, sm = pm.value, sm.value
            num = np.zeros(N, np.int32)
            ex = np.zeros(N * pm)
            co = np.zeros(N * sm * pm)
            ctx.call("get_ao_basis_prim_num_per_nucleus", num.ctypes.data_as(ctypes.c_void_p), N)
            ctx.call("get_ao_basis_expo_per_nucleus", ex.ctypes.data_as(ctypes.c_void_p), ex.size)
            ctx.call("get_ao_basis_coef_per_nucleus", co.ctypes.data_as(ctypes.c_void_p), co.size)
            assert np.array_equal(num, ref["prim_num_per_nucleus"])
            assert np.array_equal(ex.reshape(N, pm), ref["expo_per_nucleus"])
            assert np.array_equal(co.reshape(N, sm, pm), ref["coef_per_nucleus"])
            ctx.call("finalize_ao_basis_hpc")
        with pytest.raises(QmcklError) as e:
            ctx.call("get_ao_basis_expo_per_nucleus", ex.ctypes.data_as(ctypes.c_void_p), ex.size - 1)
        assert e.value.code == 3

"""Shared exponentials of the fused AO kernels (the per-nucleus distinct-exponent layout of
qmckl_finalize_ao_basis_hpc_device, src/qmckl_ao_sycl.cpp:855-1065, used by the kernels): on
contracted bases each distinct exponential is evaluated once per point and nucleus. The FP64
results must be bit-identical with sharing on and off, the split-BF16 ones within the form's
tolerance of the oracle, and the batched form must give each member's single-context bits."""
import numpy as np
import pytest

from conftest import normwise_rel_err
from oracle import oracle
from qmckl_sycl_gb300 import (PRECISION_FP64, PRECISION_SPLIT_BF16, SHARED_EXP_AUTO, SHARED_EXP_OFF, SHARED_EXP_ON,
                              Batch, Context, QmcklError, config_medium, config_small)
from qmckl_sycl_gb300.systems import config_contracted, make_system

pytestmark = pytest.mark.gpu


def replace(s, **kw):
    return s.__class__(**{**s.__dict__, **kw})


def rounded_exponents(s):
    return replace(s, exponent=np.round(s.exponent) + 1.0)


def g_shells():
    # l up to 5 (the generic path) with repeated exponents
    s = make_system(11, 5, 8, 5.0, 40, (0.3, 0.2, 0.2, 0.1, 0.1, 0.1), 4, (0.1, 20.0), 30, 96, 1.5, name="g")
    return rounded_exponents(s)


def chbrclf_points(chbrclf, n, seed=0):
    rng = np.random.default_rng(seed)
    nuc = chbrclf.nucl_coord.T[rng.integers(0, chbrclf.nucl_num, n)]
    return chbrclf.with_points(nuc + rng.normal(scale=1.5, size=(n, 3)))


def run(s, mode, precision=PRECISION_FP64):
    with Context(0) as ctx:
        ctx.load_system(s)
        ctx.set_shared_exponentials(mode)
        ctx.set_precision(precision)
        active = ctx.shared_exponentials()
        out = dict(mo_vgl=ctx.get_mo_vgl(s.point_num))
        if precision == PRECISION_FP64:
            out["ao_vgl"] = ctx.get_ao_vgl(s.point_num)
            out["ao_value"] = ctx.get_ao_value(s.point_num)
            ctx.touch()
            out["mo_value"] = ctx.get_mo_value(s.point_num)
        return active, out


def test_auto_selection(chbrclf):
    # CHBrClF repeats exponents (133 distinct for 297 primitives), but mostly steep ones that
    # are screened for most points: the automatic choice leaves sharing off there
    assert not run(chbrclf, SHARED_EXP_AUTO)[0]
    # generally contracted: shared for the FP64 outputs, not for the split-BF16 planes
    assert run(config_contracted(0, 64, nucl_num=3), SHARED_EXP_AUTO)[0]
    assert not run(config_contracted(0, 64, nucl_num=3), SHARED_EXP_AUTO, PRECISION_SPLIT_BF16)[0]
    assert run(rounded_exponents(config_small(0)), SHARED_EXP_AUTO)[0]
    assert not run(config_small(0), SHARED_EXP_AUTO)[0]  # random exponents: nothing shared
    assert not run(config_medium(0, 1, 2), SHARED_EXP_AUTO)[0]
    assert not run(config_medium(0, 1, 2), SHARED_EXP_ON)[0]  # over 64 distinct exponents on a nucleus
    assert run(config_small(0), SHARED_EXP_ON)[0]  # forced on
    assert not run(chbrclf, SHARED_EXP_OFF)[0]


@pytest.mark.parametrize("name", ["chbrclf", "rounded_small", "g_shells", "small_forced", "contracted"])
def test_fp64_bit_identical_on_and_off(name, chbrclf):
    s = {"chbrclf": lambda: chbrclf_points(chbrclf, 700), "rounded_small": lambda: rounded_exponents(config_small(4, 300)),
         "g_shells": g_shells, "small_forced": lambda: config_small(7, 300),
         "contracted": lambda: config_contracted(1, 300, nucl_num=4, mo_num=60)}[name]()
    a_on, on = run(s, SHARED_EXP_ON)
    a_off, off = run(s, SHARED_EXP_OFF)
    assert a_on and not a_off
    for k in on:
        assert np.array_equal(on[k], off[k]), k
    ref = oracle.forward(s, want=("ao_vgl", "mo_vgl"))
    assert normwise_rel_err(on["mo_vgl"], ref["mo_vgl"]) <= 1e-12
    assert normwise_rel_err(on["ao_vgl"], ref["ao_vgl"]) <= 1e-12


def test_golden_mo_vgl_with_sharing(chbrclf, golden):
    # the reference's own golden values (1e-14 absolute) through the shared path
    active, out = run(chbrclf, SHARED_EXP_ON)
    assert active
    assert np.abs(out["mo_vgl"] - golden["mo_vgl_ref"]).max() <= 1e-14


@pytest.mark.parametrize("name", ["chbrclf", "rounded_small", "g_shells", "contracted"])
def test_split_form_with_sharing(name, chbrclf):
    s = {"chbrclf": lambda: chbrclf_points(chbrclf, 700), "rounded_small": lambda: rounded_exponents(config_small(4, 300)),
         "g_shells": g_shells, "contracted": lambda: config_contracted(1, 300, nucl_num=4, mo_num=60)}[name]()
    ref = oracle.forward(s, want=("mo_vgl",))["mo_vgl"]
    on = run(s, SHARED_EXP_ON, PRECISION_SPLIT_BF16)[1]["mo_vgl"]
    off = run(s, SHARED_EXP_OFF, PRECISION_SPLIT_BF16)[1]["mo_vgl"]
    e_on, e_off = normwise_rel_err(on, ref), normwise_rel_err(off, ref)
    print("%s: split-BF16 error with sharing %.2e, without %.2e" % (name, e_on, e_off))
    assert e_on <= 1e-6 and e_off <= 1e-6


@pytest.mark.parametrize("precision", [PRECISION_FP64, PRECISION_SPLIT_BF16])
def test_batch_members_match_single_contexts(precision, chbrclf):
    systems = [chbrclf_points(chbrclf, 300, 1), rounded_exponents(config_small(5, 200)), config_small(6, 150)]
    want = [run(s, SHARED_EXP_AUTO, precision)[1]["mo_vgl"] for s in systems]
    ctxs = []
    for s in systems:
        c = Context(0)
        c.load_system(s)
        ctxs.append(c)
    with Batch(ctxs) as b:
        b.set_precision(precision)
        got = b.get_mo_vgl()
    for c in ctxs:
        c.close()
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_mode_argument_checked(chbrclf):
    with Context(0) as ctx:
        ctx.load_system(chbrclf)
        with pytest.raises(QmcklError) as e:
            ctx.set_shared_exponentials(2)
        assert e.value.code == 2

"""Pins the CPU oracle (oracle/qmckl_oracle.c) before it is trusted as the checker:
against the reference's own golden file and known answers, and bit for bit against the
unmodified reference built on this host (when the reference checkout is present)."""
import numpy as np
import pytest

from oracle import oracle
from qmckl_sycl_gb300.systems import config_adjoint, config_medium, config_small, with_empty_nucleus


def test_oracle_matches_golden_mo_vgl(chbrclf, golden):
    # tests/test_qmckl_mo.cpp:382-405 of the reference: every mo_vgl value at 1e-14 absolute
    out = oracle.forward(chbrclf, want=("mo_vgl",))
    ref = golden["mo_vgl_ref"]
    assert out["mo_vgl"].shape == ref.shape
    assert np.abs(out["mo_vgl"] - ref).max() <= 1e-14


def test_oracle_known_answers(chbrclf, golden):
    # ao_value[26][219..222] on walker 0 (tests/test_qmckl_ao.cpp:440-448)
    s0 = chbrclf.with_points(chbrclf.coord[:68])
    out = oracle.forward(s0, want=("ao_value",))
    for p, a, v in golden["kat_ao_value"]:
        assert abs(out["ao_value"][int(p), int(a)] - v) <= float(golden["kat_ao_value_tol"])
    # ao_vgl[26][0..4][219] on both walkers (tests/test_qmckl_mo.cpp:250-259)
    out = oracle.forward(chbrclf, want=("ao_vgl",))
    for p, c, a, v in golden["kat_ao_vgl"]:
        assert abs(out["ao_vgl"][int(p), int(c), int(a)] - v) <= float(golden["kat_ao_vgl_tol"])


def test_oracle_mo_value_consistent_with_mo_vgl(chbrclf):
    # tests/test_qmckl_mo.cpp:301-356: mo_value == mo_vgl[:, 0, :] within 1e-12
    out = oracle.forward(chbrclf, want=("mo_vgl", "mo_value"))
    assert np.abs(out["mo_value"] - out["mo_vgl"][:, 0, :]).max() <= 1e-12


@pytest.mark.parametrize("name", ["chbrclf", "small", "adjoint", "medium64", "chbrclf_empty_nucleus"])
def test_oracle_bitwise_equal_to_reference(name, chbrclf):
    if oracle.reference_lib() is None:
        pytest.skip("reference library not built on this machine (needs the reference checkout)")
    s = {"chbrclf": lambda: chbrclf, "small": lambda: config_small(0), "adjoint": lambda: config_adjoint(0),
         "medium64": lambda: config_medium(0, walkers=1, electrons=64),
         "chbrclf_empty_nucleus": lambda: with_empty_nucleus(chbrclf, 2)}[name]()
    want = ("ao_vgl", "ao_value", "mo_vgl", "mo_value")
    r = oracle.reference_forward(s, want=want)
    o = oracle.forward(s, want=want)
    for k in want:
        assert np.array_equal(r[k], o[k]), k


@pytest.mark.parametrize("at", [0, 2, 5])
def test_oracle_centre_without_shells(chbrclf, at):
    # a centre that owns no shell (nucleus_shell_num 0) changes no AO or MO value
    want = ("ao_vgl", "ao_value", "mo_vgl", "mo_value")
    a = oracle.forward(chbrclf, want=want)
    b = oracle.forward(with_empty_nucleus(chbrclf, at), want=want)
    for k in want:
        assert np.array_equal(a[k], b[k]), k


def test_oracle_nan_coordinates_equal_to_reference():
    # NaN coordinates: the reference screens nothing for them (its `>` tests are false for NaN)
    # and every output of the point is NaN; the oracle must give the same bits elsewhere and
    # NaN in the same places
    if oracle.reference_lib() is None:
        pytest.skip("reference library not built on this machine (needs the reference checkout)")
    s = nan_points(config_small(9, point_num=40))
    want = ("ao_vgl", "ao_value", "mo_vgl", "mo_value")
    r = oracle.reference_forward(s, want=want)
    o = oracle.forward(s, want=want)
    for k in want:
        assert np.array_equal(np.isnan(r[k]), np.isnan(o[k])), k
        assert np.array_equal(np.nan_to_num(r[k]), np.nan_to_num(o[k])), k
    assert np.isnan(o["mo_vgl"][7]).all() and not np.isnan(o["mo_vgl"][0]).any()


def zero_prim_shells(s, shells=(3, 10, 25)):
    """The system with some shells given no primitives (their radial sums are zero)."""
    spn = s.shell_prim_num.copy()
    spn[list(shells)] = 0
    return s.__class__(**{**s.__dict__, "shell_prim_num": spn})


@pytest.mark.parametrize("with_nan", [False, True])
def test_oracle_zero_primitive_shells_equal_to_reference(with_nan):
    # shells without primitives contribute zero radials; with NaN coordinates their AOs are 0 or
    # NaN depending on the polynomial's factors, like the reference's
    if oracle.reference_lib() is None:
        pytest.skip("reference library not built on this machine (needs the reference checkout)")
    s = zero_prim_shells(config_small(12, point_num=64))
    if with_nan:
        s = nan_points(s)
    want = ("ao_vgl", "ao_value", "mo_vgl", "mo_value")
    r = oracle.reference_forward(s, want=want)
    o = oracle.forward(s, want=want)
    for k in want:
        assert np.array_equal(np.isnan(r[k]), np.isnan(o[k])), k
        assert np.array_equal(np.nan_to_num(r[k]), np.nan_to_num(o[k])), k


def nan_points(s):
    """The system with NaN in some coordinates: point 3 (x), point 7 (x, y, z), point 12 (z)."""
    coord = s.coord.copy()
    coord[3, 0] = np.nan
    coord[7, :] = np.nan
    coord[12, 2] = np.nan
    return s.with_points(coord)


def test_oracle_shell_vgl_matches_reference_layout(chbrclf):
    sv = oracle.shell_vgl(chbrclf)
    assert sv.shape == (chbrclf.point_num, 5, chbrclf.shell_num)
    # s shells contribute their radial value directly to their AO value (ao_factor 1)
    ao = oracle.forward(chbrclf, want=("ao_vgl",))["ao_vgl"]
    assert np.array_equal(sv[:, 0, 0] * chbrclf.ao_factor[0], ao[:, 0, 0])


def test_oracle_threads_do_not_change_bits():
    s = config_small(3, point_num=200)
    a = oracle.forward(s, threads=1)
    b = oracle.forward(s, threads=4)
    for k in a:
        assert np.array_equal(a[k], b[k]), k

"""TREXIO reader on the GPU (reference: src/qmckl_trexio.cpp:960-1021, qmckl_trexio_read_device):
the CHBrClF molecule written in TREXIO's layout (per-shell nucleus index, per-primitive shell
index, coordinates [nucleus][3], MO coefficients [mo][ao]) and read through the C ABI gives the
same context as the setters: the same per-nucleus and per-shell tables, bit-identical AO and MO
values, and the reference's golden MO values (tests/mo_reference.txt of the reference). libtrexio
is not installed on these machines, so the test double of its API in tests/trexio_double serves
the file."""
import ctypes
import os
import shutil
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from trexio_double import files  # noqa: E402

from qmckl_sycl_gb300 import Context, QmcklError  # noqa: E402
from qmckl_sycl_gb300.systems import with_empty_nucleus  # noqa: E402

pytestmark = [pytest.mark.gpu, pytest.mark.skipif(shutil.which("gcc") is None, reason="no host C compiler")]


@pytest.fixture(scope="module")
def double_lib(tmp_path_factory):
    return files.build(str(tmp_path_factory.mktemp("trexio")))


@pytest.fixture
def use_double(double_lib, monkeypatch):
    monkeypatch.setenv("QMCKL_TREXIO_LIBRARY", double_lib)


def outputs(ctx, P):
    return dict(ao_vgl=ctx.get_ao_vgl(P), ao_value=ctx.get_ao_value(P), mo_vgl=ctx.get_mo_vgl(P),
                mo_value=ctx.get_mo_value(P))


def get_i64(ctx, name, n):
    a = np.zeros(n, np.int64)
    ctx.call(name, a.ctypes.data_as(ctypes.c_void_p), n)
    return a


@pytest.mark.parametrize("back_end", ["T", "H"])
def test_chbrclf_from_trexio_equals_setters(use_double, chbrclf, golden, tmp_path, back_end):
    path = tmp_path / "chbrclf.trexio"
    up, dn = int(golden["elec_up_num"]), int(golden["elec_dn_num"])
    files.write(str(path), files.records_of(chbrclf, up, dn), back_end=back_end)
    P = chbrclf.point_num
    with Context(0) as a, Context(0) as b:
        a.read_trexio(path)
        a.set_point(chbrclf.coord)
        b.load_system(chbrclf)
        n = ctypes.c_int64(0)
        a.call("get_electron_num", ctypes.byref(n))
        assert n.value == up + dn
        S, N = chbrclf.shell_num, chbrclf.nucl_num
        assert (get_i64(a, "get_ao_basis_nucleus_index", N) == chbrclf.nucleus_index).all()
        assert (get_i64(a, "get_ao_basis_nucleus_shell_num", N) == chbrclf.nucleus_shell_num).all()
        assert (get_i64(a, "get_ao_basis_shell_prim_index", S) == chbrclf.shell_prim_index).all()
        assert (get_i64(a, "get_ao_basis_shell_prim_num", S) == chbrclf.shell_prim_num).all()
        got, want = outputs(a, P), outputs(b, P)
        for k in want:
            assert np.array_equal(got[k], want[k]), k
        worst = np.abs(got["mo_vgl"] - golden["mo_vgl_ref"]).max()
        print("TREXIO-loaded CHBrClF: golden mo_vgl max abs difference %.3e" % worst)
        assert worst <= 5e-14


def test_nucleus_without_shells(use_double, chbrclf, tmp_path):
    # a sixth centre (a bare charge) owns no shell: its first-shell entry is 0 and its count 0,
    # and the AO and MO values are those of the five-nucleus molecule
    six = with_empty_nucleus(chbrclf, 5)
    path = tmp_path / "six.trexio"
    files.write(str(path), files.records_of(six, 3, 2))
    P = chbrclf.point_num
    with Context(0) as a, Context(0) as b:
        a.read_trexio(path)
        a.set_point(six.coord)
        assert get_i64(a, "get_ao_basis_nucleus_index", 6)[5] == 0
        assert get_i64(a, "get_ao_basis_nucleus_shell_num", 6)[5] == 0
        b.load_system(chbrclf)
        got, want = outputs(a, P), outputs(b, P)
        for k in want:
            assert np.array_equal(got[k], want[k]), k


def test_missing_mo_group_keeps_the_basis(use_double, chbrclf, golden, tmp_path):
    path = tmp_path / "no_mo.trexio"
    files.write(str(path), files.records_of(chbrclf, 2, 1, mo=False))
    P = chbrclf.point_num
    with Context(0) as a, Context(0) as b:
        with pytest.raises(QmcklError) as e:
            a.read_trexio(path)
        assert (e.value.code, e.value.function, e.value.message) == (101, "qmckl_trexio_omp_read", "Error reading MOs")
        a.set_point(chbrclf.coord)
        b.load_system(chbrclf, mo=False)
        assert np.array_equal(a.get_ao_vgl(P), b.get_ao_vgl(P))

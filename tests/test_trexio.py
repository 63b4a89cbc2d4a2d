"""TREXIO reader checks that need no GPU (reference: src/qmckl_trexio.cpp): the library binds
libtrexio at run time and reports its absence; files open with the text back end first, then
HDF5; the electron group is read; per-shell nucleus indices and per-primitive shell indices that
are out of range or not contiguous are refused before anything reaches the device. libtrexio is
not installed here, so a test double of its API (tests/trexio_double) stands in for it."""
import ctypes
import os
import shutil
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
from trexio_double import files  # noqa: E402

from qmckl_sycl_gb300 import capi  # noqa: E402

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="no host C compiler")

FAILURE, INVALID_ARG_2, INVALID_CONTEXT = 101, 2, 103


@pytest.fixture(scope="module")
def double_lib(tmp_path_factory):
    return files.build(str(tmp_path_factory.mktemp("trexio")))


@pytest.fixture
def use_double(double_lib, monkeypatch):
    monkeypatch.setenv("QMCKL_TREXIO_LIBRARY", double_lib)
    return ctypes.CDLL(double_lib)  # the same handle the library binds: its call counters


@pytest.fixture
def ctx():
    L = capi.lib()
    c = L.qmckl_context_create_device(0)
    yield c
    L.qmckl_context_destroy_device(c)


def error_of(c):
    code = ctypes.c_int32(0)
    fn = ctypes.create_string_buffer(256)
    msg = ctypes.create_string_buffer(1024)
    capi.lib().qmckl_get_error_device(c, ctypes.byref(code), fn, 256, msg, 1024)
    return code.value, fn.value.decode(), msg.value.decode()


def read(c, path):
    name = os.fsencode(str(path))
    return capi.lib().qmckl_trexio_read_device(c, name, len(name))


def test_missing_library_is_reported(ctx, monkeypatch, tmp_path):
    monkeypatch.setenv("QMCKL_TREXIO_LIBRARY", str(tmp_path / "no_such_libtrexio.so"))
    assert read(ctx, tmp_path / "x.trexio") == FAILURE
    code, fn, msg = error_of(ctx)
    assert (code, fn) == (FAILURE, "qmckl_trexio_read_device")
    assert msg.startswith("libtrexio could not be loaded")
    rc = ctypes.c_int32(0)
    assert capi.lib().qmckl_trexio_open_X_device(b"x", ctypes.byref(rc)) is None
    assert rc.value == FAILURE


def test_null_context_and_arguments(use_double, ctx, tmp_path):
    L = capi.lib()
    assert L.qmckl_trexio_read_device(0, b"x", 1) == INVALID_CONTEXT
    assert L.qmckl_trexio_read_device(ctx, None, 1) == INVALID_ARG_2
    assert L.qmckl_trexio_read_device(ctx, b"x", -1) == 3
    assert L.qmckl_trexio_read_electron_X_device(ctx, None) == INVALID_ARG_2
    assert L.qmckl_trexio_read_ao_X_device(0, None) == INVALID_CONTEXT


def test_open_tries_text_then_hdf5(use_double, ctx, tmp_path):
    calls = use_double.trexio_double_calls
    calls.restype = ctypes.c_int64
    before = [calls(i) for i in range(3)]
    assert read(ctx, tmp_path / "absent.trexio") == INVALID_ARG_2
    assert [calls(i) - b for i, b in zip(range(3), before)] == [1, 1, 0]

    files.write(str(tmp_path / "h.trexio"), {"electron_up_num": np.int64(3)}, back_end="H")
    rc = ctypes.c_int32(-1)
    L = capi.lib()
    f = L.qmckl_trexio_open_X_device(os.fsencode(str(tmp_path / "h.trexio")), ctypes.byref(rc))
    assert f and rc.value == 0
    assert [calls(i) - b for i, b in zip(range(3), before)] == [2, 2, 0]
    close = use_double.trexio_close
    close.argtypes = [ctypes.c_void_p]
    assert close(f) == 0


def test_file_name_is_cut_at_size_max(use_double, ctx, tmp_path):
    path = tmp_path / "e.trexio"
    files.write(str(path), {"electron_up_num": np.int64(5), "electron_dn_num": np.int64(4)})
    name = os.fsencode(str(path))
    # the name's first len(name) characters open the file; the trailing garbage is not read
    assert capi.lib().qmckl_trexio_read_device(ctx, name + b"garbage", len(name)) == FAILURE
    code, fn, msg = error_of(ctx)
    assert (fn, msg) == ("qmckl_trexio_read_device", "Error reading nucleus")
    num = ctypes.c_int64(0)
    assert capi.lib().qmckl_get_electron_num_device(ctx, ctypes.byref(num)) == 0
    assert num.value == 9


def _open(path):
    rc = ctypes.c_int32(-1)
    f = capi.lib().qmckl_trexio_open_X_device(os.fsencode(str(path)), ctypes.byref(rc))
    assert f and rc.value == 0
    return f


def _basis_file(tmp_path, shell_nucleus, prim_shell, name="b.trexio", **extra):
    r = {"nucleus_num": np.int64(2), "basis_type": "Gaussian", "basis_shell_num": np.int64(len(shell_nucleus)),
         "basis_prim_num": np.int64(len(prim_shell)), "ao_num": np.int64(4),
         "basis_nucleus_index": np.asarray(shell_nucleus, np.int64),
         "basis_shell_index": np.asarray(prim_shell, np.int64),
         "basis_shell_ang_mom": np.zeros(len(shell_nucleus), np.int32)}
    r.update(extra)
    files.write(str(tmp_path / name), r)
    return tmp_path / name


@pytest.mark.parametrize("shell_nucleus, prim_shell, what", [
    ([0, 1, 2, 1], [0, 1, 2, 3], "trexio_read_basis_nucleus_index"),   # nucleus 2 of 2
    ([0, 1, 0, 1], [0, 1, 2, 3], "trexio_read_basis_nucleus_index"),   # nucleus 0's shells split
    ([-1, 0, 1, 1], [0, 1, 2, 3], "trexio_read_basis_nucleus_index"),
])
def test_irrelevant_nucleus_index_is_refused(use_double, ctx, tmp_path, shell_nucleus, prim_shell, what):
    L = capi.lib()
    f = _open(_basis_file(tmp_path, shell_nucleus, prim_shell))
    assert L.qmckl_set_nucleus_num_device(ctx, 2) == 0
    assert L.qmckl_trexio_read_ao_X_device(ctx, f) == FAILURE
    assert error_of(ctx) == (FAILURE, what, "Irrelevant data in TREXIO file")
    # nothing of the per-nucleus tables was set
    assert L.qmckl_get_ao_basis_nucleus_index_device(ctx, (ctypes.c_int64 * 2)(), 2) == 106
    use_double.trexio_close.argtypes = [ctypes.c_void_p]
    use_double.trexio_close(f)


def test_basis_type_and_missing_data(use_double, ctx, tmp_path):
    L = capi.lib()
    L.qmckl_set_nucleus_num_device(ctx, 2)
    f = _open(_basis_file(tmp_path, [0, 1], [0, 1], basis_type="Slater"))
    assert L.qmckl_trexio_read_ao_X_device(ctx, f) == FAILURE
    assert error_of(ctx) == (FAILURE, "trexio_read_basis_type", "Invalid basis type")
    g = _open(_basis_file(tmp_path, [0, 1], [0, 1], name="c.trexio",
                          basis_nucleus_index=np.array([0, 1, 1], np.int64)))
    # basis_nucleus_index holds 3 values where shell_num says 2: the size-checked read refuses it
    code = L.qmckl_trexio_read_ao_X_device(ctx, g)
    assert code == FAILURE
    assert error_of(ctx)[1:] == ("trexio_read_basis_nucleus_index", "Incorrect array dimensions")
    use_double.trexio_close.argtypes = [ctypes.c_void_p]
    use_double.trexio_close(f)
    use_double.trexio_close(g)


def test_group_conversion_matches_the_fixture(chbrclf):
    # the file form of CHBrClF inverts back to the reference's per-nucleus and per-shell tables
    r = files.records_of(chbrclf, 34, 33)
    sn = r["basis_nucleus_index"]
    assert (np.bincount(sn, minlength=chbrclf.nucl_num) == chbrclf.nucleus_shell_num).all()
    assert all(int(np.argmax(sn == k)) == chbrclf.nucleus_index[k] for k in range(chbrclf.nucl_num))
    ps = r["basis_shell_index"]
    assert (np.bincount(ps, minlength=chbrclf.shell_num) == chbrclf.shell_prim_num).all()


def test_absurd_sizes_fail_cleanly(use_double, ctx, tmp_path):
    # a file that declares 10^15 shells: the reader reports an allocation failure instead of
    # throwing across the C ABI
    L = capi.lib()
    L.qmckl_set_nucleus_num_device(ctx, 2)
    f = _open(_basis_file(tmp_path, [0, 1], [0, 1], name="big.trexio", basis_shell_num=np.int64(10**15),
                          basis_prim_num=np.int64(10**15), ao_num=np.int64(10**15)))
    assert L.qmckl_trexio_read_ao_X_device(ctx, f) == 104
    assert error_of(ctx)[:2] == (104, "qmckl_trexio_read_ao_X_device")
    use_double.trexio_close.argtypes = [ctypes.c_void_p]
    use_double.trexio_close(f)

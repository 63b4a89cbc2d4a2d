"""C ABI checks that need no GPU: the library loads, exports every function
include/qmckl_gpu.h declares, and the host-side argument checks, masks and exit codes
follow the reference (contexts create their CUDA stream lazily, so everything up to the
first device copy runs on a machine without a GPU)."""
import ctypes
import subprocess

import pytest

from qmckl_sycl_gb300 import capi

L = None


def setup_module(_):
    global L
    L = capi.lib()


def test_library_exports_every_declared_symbol():
    declared = capi.declared_functions()
    assert len(declared) >= 100
    out = subprocess.check_output(["nm", "-D", "--defined-only", capi.lib_path()]).decode()
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    missing = [f for f in declared if f not in exported]
    assert missing == []


def test_reference_entry_points_are_declared():
    # the call set of the reference's tests (tests/test_qmckl_ao.cpp, tests/test_qmckl_mo.cpp)
    needed = """context_create context_destroy context_touch malloc free memcpy_H2D memcpy_D2H
        set_point set_electron_num set_electron_coord set_nucleus_num set_nucleus_coord set_nucleus_charge
        set_ao_basis_type set_ao_basis_shell_num set_ao_basis_prim_num set_ao_basis_nucleus_index
        set_ao_basis_nucleus_shell_num set_ao_basis_shell_ang_mom set_ao_basis_shell_factor
        set_ao_basis_shell_prim_num set_ao_basis_shell_prim_index set_ao_basis_exponent set_ao_basis_coefficient
        set_ao_basis_prim_factor set_ao_basis_ao_num set_ao_basis_ao_factor get_ao_basis_ao_vgl
        get_ao_basis_ao_value set_mo_basis_mo_num set_mo_basis_coefficient get_mo_basis_mo_value
        get_mo_basis_mo_vgl ao_basis_provided mo_basis_provided nucleus_provided electron_provided""".split()
    declared = set(capi.declared_functions())
    for n in needed:
        name = "qmckl_%s_device" % n if not n.startswith("memcpy") else "qmckl_" + n
        assert name in declared, name


def test_null_context_codes():
    assert L.qmckl_context_check_device(0) == 0
    assert L.qmckl_context_destroy_device(0) == 103
    assert L.qmckl_context_touch_device(0) == 103
    assert L.qmckl_set_nucleus_num_device(0, 3) == 103
    assert L.qmckl_malloc_device(0, 16) is None
    assert not L.qmckl_ao_basis_provided_device(0)
    assert L.qmckl_string_of_error_device(103) == b"Invalid context"


def test_batch_argument_checks():
    # creation rejects empty, invalid and duplicated member lists before touching a GPU
    assert L.qmckl_batch_create_device(None, 0) == 0
    bad = (ctypes.c_int64 * 2)(0, 0)
    assert L.qmckl_batch_create_device(bad, 2) == 0
    c = L.qmckl_context_create_device(0)
    dup = (ctypes.c_int64 * 2)(c, c)
    assert L.qmckl_batch_create_device(dup, 2) == 0
    assert L.qmckl_context_destroy_device(c) == 0
    for f in ("destroy", "touch", "provide_mo_vgl", "synchronize", "autotune"):
        assert getattr(L, "qmckl_batch_%s_device" % f)(0) == 103
    assert L.qmckl_batch_set_precision_mode_device(0, 1) == 103
    assert L.qmckl_batch_get_launch_count_device(0) == 0


def test_distance_argument_checks():
    c = L.qmckl_context_create_device(0)
    v = ctypes.c_void_p(1)  # never dereferenced: the checks fail first
    assert L.qmckl_distance_device(c, b"T", b"T", 0, 4, v, 4, v, 4, v, 4) == 4
    assert L.qmckl_distance_device(c, b"T", b"T", 4, 0, v, 4, v, 4, v, 4) == 5
    assert L.qmckl_distance_device(c, b"X", b"T", 4, 4, v, 4, v, 4, v, 4) == 1
    assert L.qmckl_distance_device(c, b"T", b"N", 4, 4, v, 3, v, 3, v, 4) == 7
    assert L.qmckl_distance_device(c, b"N", b"T", 4, 4, v, 3, v, 3, v, 4) == 9
    assert L.qmckl_distance_device(c, b"N", b"N", 4, 4, v, 3, v, 3, v, 3) == 11
    assert L.qmckl_compute_en_distance_device(c, 0, 2, v, v, v) == 2
    assert L.qmckl_compute_ee_distance_device(c, 2, 0, v, v) == 3
    assert L.qmckl_distance_device(0, b"T", b"T", 4, 4, v, 4, v, 4, v, 4) == 103
    assert L.qmckl_string_of_error_device(11) == b"Invalid argument 11"
    assert L.qmckl_context_destroy_device(c) == 0


def test_error_record_and_strings():
    c = L.qmckl_context_create_device(0)
    assert L.qmckl_context_check_device(c) == c
    assert L.qmckl_failwith_device(c, 104, b"f", b"m") == 104
    code = ctypes.c_int32()
    fn = ctypes.create_string_buffer(64)
    msg = ctypes.create_string_buffer(64)
    L.qmckl_get_error_device(c, ctypes.byref(code), fn, 64, msg, 64)
    assert (code.value, fn.value, msg.value) == (104, b"f", b"m")
    for k in (0, 1, 2, 3, 101, 102, 103, 104, 105, 106, 107, 108, 109):
        assert L.qmckl_string_of_error_device(k) not in (b"", None)
    assert L.qmckl_context_destroy_device(c) == 0


def test_nucleus_and_electron_masks():
    c = L.qmckl_context_create_device(0)
    n = ctypes.c_int64()
    assert L.qmckl_get_nucleus_num_device(c, ctypes.byref(n)) == 106  # not provided
    assert L.qmckl_set_nucleus_num_device(c, 0) == 2
    assert L.qmckl_set_nucleus_num_device(c, 4) == 0
    assert L.qmckl_set_nucleus_num_device(c, 4) == 108  # src/qmckl_nucleus.cpp:522-526
    assert L.qmckl_get_nucleus_num_device(c, ctypes.byref(n)) == 0 and n.value == 4
    assert not L.qmckl_nucleus_provided_device(c)
    assert L.qmckl_set_nucleus_coord_device(c, b"T", None, 5) == 4  # array too small -> arg 4
    assert L.qmckl_set_nucleus_charge_device(c, None, 4) == 2
    assert L.qmckl_set_electron_num_device(c, 0, 1) == 2
    assert L.qmckl_set_electron_num_device(c, 2, -1) == 3
    assert L.qmckl_set_electron_num_device(c, 2, 1) == 0
    assert L.qmckl_electron_provided_device(c)
    assert L.qmckl_set_electron_num_device(c, 2, 1) == 108
    assert L.qmckl_get_electron_num_device(c, ctypes.byref(n)) == 0 and n.value == 3
    L.qmckl_context_destroy_device(c)


def test_point_argument_checks():
    c = L.qmckl_context_create_device(0)
    assert L.qmckl_set_point_device(c, b"N", 10, None, 29) == 4  # size_max < 3*num
    assert L.qmckl_set_point_device(c, b"X", 10, None, 30) == 2  # bad transp
    assert L.qmckl_set_point_device(c, b"N", 10, None, 30) == 3  # NULL coord
    buf = (ctypes.c_double * 3)()
    assert L.qmckl_get_point_device(c, b"N", buf, 3) == 106  # no points yet
    L.qmckl_context_destroy_device(c)


def test_ao_scalar_setters_follow_reference_order_checks():
    c = L.qmckl_context_create_device(0)
    v = ctypes.c_int64()
    assert L.qmckl_set_ao_basis_type_device(c, b"X") == 2
    assert L.qmckl_set_ao_basis_type_device(c, b"G") == 0
    assert L.qmckl_set_ao_basis_prim_num_device(c, 10) == 101  # shell_num not set
    assert L.qmckl_set_ao_basis_ao_num_device(c, 10) == 2  # shell_num not set
    assert L.qmckl_set_ao_basis_shell_num_device(c, 0) == 2
    assert L.qmckl_set_ao_basis_shell_num_device(c, 5) == 0
    assert L.qmckl_set_ao_basis_prim_num_device(c, 4) == 2  # prim_num < shell_num
    assert L.qmckl_set_ao_basis_prim_num_device(c, 9) == 0
    assert L.qmckl_set_ao_basis_shell_num_device(c, 10) == 2  # shell_num > prim_num
    assert L.qmckl_set_ao_basis_ao_num_device(c, 4) == 2  # ao_num < shell_num
    assert L.qmckl_set_ao_basis_ao_num_device(c, 7) == 0
    assert L.qmckl_get_ao_basis_shell_num_device(c, ctypes.byref(v)) == 0 and v.value == 5
    assert L.qmckl_get_ao_basis_prim_num_device(c, ctypes.byref(v)) == 0 and v.value == 9
    assert L.qmckl_get_ao_basis_ao_num_device(c, ctypes.byref(v)) == 0 and v.value == 7
    t = ctypes.create_string_buffer(1)
    assert L.qmckl_get_ao_basis_type_device(c, t) == 0 and t.raw == b"G"
    # array setters check their governing count before touching memory
    assert L.qmckl_set_ao_basis_nucleus_index_device(c, None, 3) == 101  # nucl_num not set
    assert L.qmckl_set_ao_basis_exponent_device(c, None, 8) == 3  # size_max < prim_num
    assert L.qmckl_set_ao_basis_shell_ang_mom_device(c, None, 4) == 3
    assert L.qmckl_set_ao_basis_ao_factor_device(c, None, 6) == 3
    # getters of unset arrays: not provided
    a = (ctypes.c_double * 16)()
    assert L.qmckl_get_ao_basis_exponent_device(c, a, 16) == 106
    assert not L.qmckl_ao_basis_provided_device(c)
    L.qmckl_context_destroy_device(c)


def test_mo_setters_masks():
    c = L.qmckl_context_create_device(0)
    v = ctypes.c_int64()
    assert L.qmckl_get_mo_basis_mo_num_device(c, ctypes.byref(v)) == 106
    assert L.qmckl_set_mo_basis_mo_num_device(c, 0) == 2
    assert L.qmckl_set_mo_basis_mo_num_device(c, 3) == 0
    assert L.qmckl_set_mo_basis_mo_num_device(c, 3) == 108
    assert L.qmckl_set_mo_basis_coefficient_device(c, None) == 101  # ao_num not set
    assert not L.qmckl_mo_basis_provided_device(c)
    assert L.qmckl_get_mo_basis_mo_vgl_device(c, None, 0) == 106
    assert L.qmckl_set_precision_mode_device(c, 7) == 2
    assert L.qmckl_set_precision_mode_device(c, 1) == 0
    m = ctypes.c_int32()
    assert L.qmckl_get_precision_mode_device(c, ctypes.byref(m)) == 0 and m.value == 1
    L.qmckl_context_destroy_device(c)


def test_host_allocation_registry():
    c = L.qmckl_context_create_device(0)
    info = capi.MemoryInfo(64, None)
    p = L.qmckl_malloc_host(c, info)
    assert p
    assert L.qmckl_free_host(c, p) == 0
    assert L.qmckl_free_host(c, p) == 2  # not registered any more
    assert L.qmckl_free_device(c, ctypes.c_void_p(12345)) == 101  # src/qmckl_memory.cpp:201-208
    L.qmckl_context_destroy_device(c)


def test_split_wait_test_hook_argument_checks():
    assert L.qmckl_set_split_wait_test_device(0, 1000, 1) == 103
    c = L.qmckl_context_create_device(0)
    assert L.qmckl_set_split_wait_test_device(c, -1, 0) == 2
    assert L.qmckl_set_split_wait_test_device(c, 1000, 2) == 3
    assert L.qmckl_set_split_wait_test_device(c, 1000, 1) == 0
    assert L.qmckl_set_split_wait_test_device(c, 0, 0) == 0
    L.qmckl_context_destroy_device(c)


def test_normal_build_has_no_bounds_checks():
    assert L.qmckl_bounds_check_status_device(0, None, None, None) == -1
    assert L.qmckl_bounds_check_selftest_device(5, 4) == -1
    assert b"bounds-check" not in L.qmckl_gb300_build_info()


def test_lock_is_recursive():
    c = L.qmckl_context_create_device(0)
    L.qmckl_lock_device(c)
    L.qmckl_lock_device(c)
    L.qmckl_unlock_device(c)
    L.qmckl_unlock_device(c)
    L.qmckl_context_destroy_device(c)


def test_library_does_not_need_the_driver_library():
    # the library must load on machines without a GPU driver (driver entry points are
    # resolved at run time through the CUDA runtime)
    out = subprocess.check_output(["readelf", "-d", capi.LIB_PATH]).decode()
    needed = [line.split("[")[-1].rstrip("]") for line in out.splitlines() if "(NEEDED)" in line]
    assert not any(n.startswith("libcuda.so") for n in needed), needed

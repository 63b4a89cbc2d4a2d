"""ctypes loader for the CPU oracle (qmckl_oracle.c) and, when it was built here, the
unmodified reference library (oracle/_ref/libqmckl_ref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the CPU
baseline legs of bench.py, as the checker or the timed CPU baseline. The product
(qmckl_sycl_gb300) never imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
ASAN_LIB_PATH = os.path.join(HERE, "_build", "liboracle_asan.so")
REF_PATH = os.path.join(HERE, "_ref", "libqmckl_ref.so")


def reference_dir():
    """The reference checkout's location (QMCKL_REFERENCE_DIR, else the default of the recipe
    oracle/Makefile.ref), or None when no checkout is there."""
    d = os.environ.get("QMCKL_REFERENCE_DIR")
    if not d:
        try:
            d = subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile.ref"), "print-reference"],
                               capture_output=True, text=True, timeout=30).stdout.strip()
        except (OSError, subprocess.SubprocessError):
            d = ""
    return d if d and os.path.isdir(os.path.join(d, "src")) else None


_f64 = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_vp = ctypes.c_void_p
_I = ctypes.c_int64


def build_oracle(force=False, sanitize=False):
    """Compiles qmckl_oracle.c (no FP contraction, OpenMP) into _build/liboracle.so, or with
    AddressSanitizer and UndefinedBehaviorSanitizer into _build/liboracle_asan.so (sanitize)."""
    src = os.path.join(HERE, "qmckl_oracle.c")
    out = ASAN_LIB_PATH if sanitize else LIB_PATH
    if not force and os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(src):
        return out
    os.makedirs(os.path.dirname(out), exist_ok=True)
    tmp = out + ".tmp%d" % os.getpid()
    extra = ["-fsanitize=address,undefined", "-fno-sanitize-recover=all", "-fno-omit-frame-pointer", "-g"] \
        if sanitize else []
    subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared",
                           "-std=c11"] + extra + [src, "-o", tmp, "-lm"])
    os.replace(tmp, out)
    return out


def build_reference(ref_dir=None):
    """Builds oracle/_ref/libqmckl_ref.so from the reference sources where they lie.
    Returns the path, or None when the reference checkout is not present."""
    ref = ref_dir or reference_dir()
    if not ref or not os.path.isdir(os.path.join(ref, "src")):
        return None
    subprocess.check_call(["make", "-s", "-j8", "-f", os.path.join(HERE, "Makefile.ref"),
                           "REFERENCE=" + ref], cwd=os.path.dirname(HERE))
    return REF_PATH


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        # QMCKL_ORACLE_SANITIZE=1: the sanitizer build (the process must preload libasan)
        L = ctypes.CDLL(build_oracle(sanitize=os.environ.get("QMCKL_ORACLE_SANITIZE") == "1"))
        L.oracle_num_threads.restype = ctypes.c_int
        L.oracle_set_num_threads.argtypes = [ctypes.c_int]
        L.oracle_forward.restype = ctypes.c_int
        L.oracle_forward.argtypes = [_I, _f64, _I, _I, _I, _i64, _i64, _i32, _i64, _i64, _f64, _f64, _f64, _f64,
                                     _f64, _I, _f64, _I, _f64, _vp, _vp, _vp, _vp]
        L.oracle_finalize_ao.argtypes = [_I, _I, _I, _i64, _i64, _i32, _i64, _i64, _f64, _f64, _f64, _f64,
                                         _i64, _f64, _i32, _f64]
        L.oracle_shell_vgl.argtypes = [_I, _I, _I, _i64, _i64, _f64, _i64, _i64, _f64, _f64, _f64, _f64, _f64]
        L.oracle_mo_vgl.argtypes = [_I, _I, _I, _f64, _f64, _f64]
        L.oracle_mo_value.argtypes = [_I, _I, _I, _f64, _f64, _f64]
        L.oracle_distance.argtypes = [ctypes.c_char, ctypes.c_char, _I, _I, _f64, _I, _f64, _I, _f64, _I]
        L.oracle_hpc_dims.argtypes = [_I, _i64, _i64, _i64, ctypes.POINTER(ctypes.c_int64),
                                      ctypes.POINTER(ctypes.c_int64)]
        L.oracle_finalize_hpc.argtypes = [_I, _i64, _i64, _i64, _i64, _f64, _f64, _I, _I, _i32, _f64, _f64]
        L.oracle_vjp_mo_vgl.restype = ctypes.c_int
        L.oracle_vjp_mo_vgl.argtypes = [_I, _f64, _I, _I, _I, _i64, _i64, _i32, _i64, _i64, _f64, _f64, _f64, _f64,
                                        _f64, _I, _f64, _I, _f64, _f64, _vp, _vp, _vp]
        _lib = L
    return _lib


def reference_lib():
    """The unmodified reference built on the host, or None if unavailable."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PATH):
            return None
        L = ctypes.CDLL(REF_PATH)
        argt = [_I, _f64, _f64, _I, _I, _I, _i64, _i64, _i32, _i64, _i64, _f64, _f64, _f64, _f64, _f64, _I,
                _f64, _I, _f64]
        L.ref_run.restype = ctypes.c_int
        L.ref_run.argtypes = argt + [_vp, _vp, _vp, _vp]
        L.ref_time_mo_vgl.restype = ctypes.c_int
        L.ref_time_mo_vgl.argtypes = argt + [ctypes.c_int, _f64]
        L.ref_hpc.restype = ctypes.c_int
        L.ref_hpc.argtypes = argt[:16] + [_i64, _i32, _f64, _f64, _I]
        _ref = L
    return _ref


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _basis_args(s):
    return (s.nucl_num, s.nucl_coord, s.shell_num, s.prim_num, s.ao_num, s.nucleus_index, s.nucleus_shell_num,
            s.shell_ang_mom, s.shell_prim_num, s.shell_prim_index, s.shell_factor, s.exponent, s.coefficient,
            s.prim_factor, s.ao_factor)


def forward(s, coord_soa=None, want=("ao_vgl", "ao_value", "mo_vgl", "mo_value"), threads=0):
    """Runs the oracle on a System `s` (see qmckl_sycl_gb300.synth). coord_soa is [3][P];
    defaults to s.coord (which is [P][3]). Returns a dict of the requested arrays."""
    L = lib()
    if threads:
        L.oracle_set_num_threads(int(threads))
    if coord_soa is None:
        coord_soa = np.ascontiguousarray(s.coord.T)
    P = coord_soa.shape[1]
    out = {}
    if "ao_vgl" in want:
        out["ao_vgl"] = np.zeros((P, 5, s.ao_num))
    if "ao_value" in want:
        out["ao_value"] = np.zeros((P, s.ao_num))
    if "mo_vgl" in want:
        out["mo_vgl"] = np.zeros((P, 5, s.mo_num))
    if "mo_value" in want:
        out["mo_value"] = np.zeros((P, s.mo_num))
    rc = L.oracle_forward(*_basis_args(s), s.mo_num, s.mo_coef, P, np.ascontiguousarray(coord_soa),
                          _ptr(out.get("ao_vgl")), _ptr(out.get("ao_value")), _ptr(out.get("mo_vgl")),
                          _ptr(out.get("mo_value")))
    assert rc == 0
    return out


def vjp_mo_vgl(s, w, want=("coef", "expo", "coord"), coord_soa=None, threads=0):
    """FP64 reference gradient of L = sum(w * mo_vgl) for System s: dL/dC [M][A], dL/dexponent
    [K] and dL/dcoord [P][3]. w is [P][5][M]."""
    L = lib()
    if threads:
        L.oracle_set_num_threads(int(threads))
    if coord_soa is None:
        coord_soa = np.ascontiguousarray(s.coord.T)
    P = coord_soa.shape[1]
    out = {}
    if "coef" in want:
        out["coef"] = np.zeros((s.mo_num, s.ao_num))
    if "expo" in want:
        out["expo"] = np.zeros(s.prim_num)
    if "coord" in want:
        out["coord"] = np.zeros((P, 3))
    rc = L.oracle_vjp_mo_vgl(*_basis_args(s), s.mo_num, s.mo_coef, P, np.ascontiguousarray(coord_soa),
                             np.ascontiguousarray(w, dtype=np.float64), _ptr(out.get("coef")), _ptr(out.get("expo")),
                             _ptr(out.get("coord")))
    assert rc == 0
    return out


def en_distance(s, coord_soa=None):
    """en_distance[point][nucleus] (the reference's call: distance('T', 'T', N, P, nucl_coord, N,
    coord, P, C, N))."""
    L = lib()
    if coord_soa is None:
        coord_soa = np.ascontiguousarray(s.coord.T)
    P = coord_soa.shape[1]
    out = np.zeros((P, s.nucl_num))
    L.oracle_distance(b"T", b"T", s.nucl_num, P, np.ascontiguousarray(s.nucl_coord), s.nucl_num,
                      np.ascontiguousarray(coord_soa), P, out, s.nucl_num)
    return out


def ee_distance(coord_soa, elec_num, walk_num):
    """ee_distance[walker][j][i] from the points [3][walk_num * elec_num]."""
    L = lib()
    out = np.zeros((walk_num, elec_num, elec_num))
    ld = elec_num * walk_num
    c = np.ascontiguousarray(coord_soa)
    for k in range(walk_num):
        sub = np.ascontiguousarray(c[:, k * elec_num:(k + 1) * elec_num])
        blk = np.zeros((elec_num, elec_num))
        L.oracle_distance(b"T", b"T", elec_num, elec_num, sub, elec_num, sub, elec_num, blk, elec_num)
        out[k] = blk
    del ld
    return out


def finalize(s):
    L = lib()
    npi = np.zeros(s.nucl_num + 1, np.int64)
    cn = np.zeros(s.prim_num)
    nmax = np.zeros(s.nucl_num, np.int32)
    nr = np.zeros(s.nucl_num)
    L.oracle_finalize_ao(s.nucl_num, s.shell_num, s.prim_num, s.nucleus_index, s.nucleus_shell_num,
                         s.shell_ang_mom, s.shell_prim_index, s.shell_prim_num, s.exponent, s.coefficient,
                         s.prim_factor, s.shell_factor, npi, cn, nmax, nr)
    return dict(nucleus_prim_index=npi, coefficient_normalized=cn, nucleus_max_ang_mom=nmax, nucleus_range=nr)


def finalize_hpc(s):
    """Per-nucleus sorted, merged exponent tables (qmckl_finalize_ao_basis_hpc_device):
    prim_num_per_nucleus [N] int32, expo_per_nucleus [N][prim_max], coef_per_nucleus
    [N][shell_max][prim_max]."""
    L = lib()
    pm, sm = ctypes.c_int64(0), ctypes.c_int64(0)
    L.oracle_hpc_dims(s.nucl_num, s.nucleus_index, s.nucleus_shell_num, s.shell_prim_num, ctypes.byref(pm),
                      ctypes.byref(sm))
    pm, sm = pm.value, sm.value
    cn = finalize(s)["coefficient_normalized"]
    num = np.zeros(s.nucl_num, np.int32)
    ex = np.zeros((s.nucl_num, pm))
    co = np.zeros((s.nucl_num, sm, pm))
    L.oracle_finalize_hpc(s.nucl_num, s.nucleus_index, s.nucleus_shell_num, s.shell_prim_index, s.shell_prim_num,
                          s.exponent, cn, pm, sm, num, ex, co)
    return dict(prim_num_per_nucleus=num, expo_per_nucleus=ex, coef_per_nucleus=co)


def reference_hpc(s):
    """The same tables read out of the unmodified reference's context after its finalize;
    None if the reference build is unavailable."""
    R = reference_lib()
    if R is None:
        return None
    dims = np.zeros(2, np.int64)
    cap = max(1, s.nucl_num * s.prim_num * max(1, s.shell_num))
    num = np.zeros(s.nucl_num, np.int32)
    ex = np.zeros(cap)
    co = np.zeros(cap)
    rc = R.ref_hpc(s.nucl_num, s.charge, *_basis_args(s)[1:], dims, num, ex, co, cap)
    assert rc == 0, rc
    pm, sm = int(dims[0]), int(dims[1])
    return dict(prim_num_per_nucleus=num, expo_per_nucleus=ex[:s.nucl_num * pm].reshape(s.nucl_num, pm),
                coef_per_nucleus=co[:s.nucl_num * sm * pm].reshape(s.nucl_num, sm, pm))


def shell_vgl(s, coord_soa=None):
    L = lib()
    fin = finalize(s)
    if coord_soa is None:
        coord_soa = np.ascontiguousarray(s.coord.T)
    P = coord_soa.shape[1]
    out = np.zeros((P, 5, s.shell_num))
    L.oracle_shell_vgl(P, s.nucl_num, s.shell_num, s.nucleus_index, s.nucleus_shell_num, fin["nucleus_range"],
                       s.shell_prim_index, s.shell_prim_num, np.ascontiguousarray(coord_soa), s.nucl_coord,
                       s.exponent, fin["coefficient_normalized"], out)
    return out


def reference_forward(s, want=("ao_vgl", "ao_value", "mo_vgl", "mo_value")):
    """Runs the unmodified reference (host build) through its own API; None if absent.
    Points are passed as [P][3] with transp 'N', nuclei as [3][N] with 'T'."""
    R = reference_lib()
    if R is None:
        return None
    P = s.coord.shape[0]
    out = {}
    if "ao_vgl" in want:
        out["ao_vgl"] = np.zeros((P, 5, s.ao_num))
    if "ao_value" in want:
        out["ao_value"] = np.zeros((P, s.ao_num))
    if "mo_vgl" in want:
        out["mo_vgl"] = np.zeros((P, 5, s.mo_num))
    if "mo_value" in want:
        out["mo_value"] = np.zeros((P, s.mo_num))
    rc = R.ref_run(s.nucl_num, s.charge, *_basis_args(s)[1:], s.mo_num, s.mo_coef, P, np.ascontiguousarray(s.coord),
                   _ptr(out.get("ao_vgl")), _ptr(out.get("ao_value")), _ptr(out.get("mo_vgl")),
                   _ptr(out.get("mo_value")))
    assert rc == 0, rc
    return out


def reference_time_mo_vgl(s, reps):
    R = reference_lib()
    if R is None:
        return None
    secs = np.zeros(reps)
    rc = R.ref_time_mo_vgl(s.nucl_num, s.charge, *_basis_args(s)[1:], s.mo_num, s.mo_coef, s.coord.shape[0],
                           np.ascontiguousarray(s.coord), reps, secs)
    assert rc == 0, rc
    return secs

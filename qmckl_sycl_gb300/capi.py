"""ctypes binding of the C ABI declared in include/qmckl_gpu.h.

The prototypes are read from the header itself, so every function the header declares
is bound with its exact argument and return types. Loading fails loudly when the native
library has not been built: there is no Python or CPU fallback for any computation.
"""
import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
HEADER = os.path.join(ROOT, "include", "qmckl_gpu.h")
LIB_PATH = os.path.join(HERE, "_lib", "libqmckl_gpu.so")
# the debug build with bounds checks on the kernels' stores (python -m qmckl_sycl_gb300.build --bounds)
BOUNDS_LIB_PATH = os.path.join(HERE, "_lib", "libqmckl_gpu_bounds.so")
# host code under AddressSanitizer/UndefinedBehaviorSanitizer (python -m qmckl_sycl_gb300.build --sanitize)
ASAN_LIB_PATH = os.path.join(HERE, "_lib", "libqmckl_gpu_asan.so")


def lib_path():
    """The library this process loads: the bounds-checked build when QMCKL_GB300_BOUNDS_CHECK=1,
    the sanitizer build when QMCKL_GB300_SANITIZE=1, else the normal one."""
    if os.environ.get("QMCKL_GB300_BOUNDS_CHECK") == "1":
        return BOUNDS_LIB_PATH
    if os.environ.get("QMCKL_GB300_SANITIZE") == "1":
        return ASAN_LIB_PATH
    return LIB_PATH


class MemoryInfo(ctypes.Structure):
    _fields_ = [("size", ctypes.c_size_t), ("pointer", ctypes.c_void_p)]


class Vector(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("size", ctypes.c_int64)]


class Matrix(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("size", ctypes.c_int64 * 2)]


class Tensor(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("order", ctypes.c_int64), ("size", ctypes.c_int64 * 16)]


_SCALARS = {
    "void": None,
    "qmckl_exit_code_device": ctypes.c_int32,
    "qmckl_context_device": ctypes.c_int64,
    "qmckl_batch_device": ctypes.c_int64,
    "int64_t": ctypes.c_int64,
    "int32_t": ctypes.c_int32,
    "uint64_t": ctypes.c_uint64,
    "size_t": ctypes.c_size_t,
    "char": ctypes.c_char,
    "bool": ctypes.c_bool,
    "double": ctypes.c_double,
    "qmckl_memory_info_struct_device": MemoryInfo,
    "qmckl_vector_device": Vector,
    "qmckl_matrix_device": Matrix,
    "qmckl_tensor_device": Tensor,
}


def _ctype(decl):
    """Maps a C parameter/return declaration (without name) to a ctypes type."""
    d = decl.replace("const", " ").strip()
    ptr = d.count("*")
    base = d.replace("*", " ").split()[0] if d.replace("*", " ").split() else "void"
    if ptr:
        if base == "char" and ptr == 1:
            return ctypes.c_char_p
        if base in ("qmckl_vector_device", "qmckl_matrix_device", "qmckl_tensor_device"):
            return ctypes.POINTER(_SCALARS[base])
        return ctypes.c_void_p
    return _SCALARS[base]


def parse_header(path=HEADER):
    """Returns {name: (restype, [argtypes])} for every function the header declares."""
    src = open(path).read()
    src = re.sub(r"/\*.*?\*/", " ", src, flags=re.S)
    src = re.sub(r"//[^\n]*", " ", src)
    src = re.sub(r"^\s*#[^\n]*", " ", src, flags=re.M)
    src = re.sub(r"typedef\s+struct\s+\w*\s*\{.*?\}\s*\w+\s*;", " ", src, flags=re.S)
    src = re.sub(r"typedef[^;]*;", " ", src)
    src = src.replace('extern "C" {', " ").replace("}", " ")
    out = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(qmckl_\w+)\s*\(([^;{]*?)\)\s*;", src, flags=re.S):
        ret, name, args = m.group(1), m.group(2), m.group(3)
        ret = ret.strip().split("\n")[-1]
        argtypes = []
        if args.strip() not in ("", "void"):
            for a in args.split(","):
                a = " ".join(a.split())
                # drop the parameter name (last identifier)
                t = re.sub(r"\b\w+\s*$", "", a) if re.search(r"[\w\*]\s+\w+\s*$", a) or "*" in a else a
                if t.strip() == "" or t.strip() in ("const",):
                    t = a
                argtypes.append(_ctype(t))
        out[name] = (_ctype(ret), argtypes)
    return out


_lib = None


def lib():
    """The loaded native library with every header prototype bound."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            raise RuntimeError(
                "qmckl_sycl_gb300 native library not found at %s; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (there is no CPU fallback)" % path)
        L = ctypes.CDLL(path)
        for name, (res, args) in parse_header().items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def declared_functions():
    return sorted(parse_header().keys())

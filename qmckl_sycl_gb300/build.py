"""Build recipe for the in-tree native library qmckl_sycl_gb300/_lib/libqmckl_gpu.so.

Every source under csrc/ is compiled by nvcc for sm_103a only (one -gencode), in parallel,
and linked into one shared library exporting the C ABI of include/qmckl_gpu.h. Host code
is compiled without floating-point contraction so that host-side table arithmetic rounds
like the reference.

    python -m qmckl_sycl_gb300.build [--force] [--verbose] [--bounds | --sanitize]

--bounds builds the debug variant _lib/libqmckl_gpu_bounds.so instead (objects in _build_bounds/),
compiled with -DQMCKL_BOUNDS_CHECK: every checked global store of the kernels tests its index
against the array's extent and records the first violation (qmckl_bounds_check_status_device).
--sanitize builds _lib/libqmckl_gpu_asan.so (objects in _build_asan/): host code with
AddressSanitizer and UndefinedBehaviorSanitizer, for the tests of the host code (argument paths
on the CPU, whole evaluations on the GPU); load it with libasan preloaded.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "libqmckl_gpu.so")
BOUNDS_LIB = os.path.join(LIBDIR, "libqmckl_gpu_bounds.so")
ASAN_LIB = os.path.join(LIBDIR, "libqmckl_gpu_asan.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
          "-I" + os.path.join(ROOT, "include"), "-DQMCKL_GB300_BUILD"]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def sources():
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cpp")):
            out.append(os.path.join(CSRC, f))
    return out


def _headers_mtime():
    m = os.path.getmtime(os.path.join(ROOT, "include", "qmckl_gpu.h"))
    for f in os.listdir(CSRC):
        if f.endswith((".hpp", ".h", ".cuh")):
            m = max(m, os.path.getmtime(os.path.join(CSRC, f)))
    return m


def _compile(src, verbose, build_dir=BUILD, extra=()):
    obj = os.path.join(build_dir, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), _headers_mtime()):
        return obj
    flags = ARCH + COMMON + list(extra)
    cmd = [nvcc()] + flags + ["-c", src, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "cu"] + flags + ["-c", src, "-o", obj]
    if verbose:
        cmd += ["-Xptxas", "-v"]
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if verbose and r.stderr:
        print(r.stderr, file=sys.stderr)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
    return obj


# Host code under AddressSanitizer and UndefinedBehaviorSanitizer (device code as usual), for the
# tests of the C ABI's host code: argument paths on the CPU, whole evaluations on the GPU.
SANITIZE = ["-Xcompiler", "-fsanitize=address,-fsanitize=undefined,-fno-sanitize-recover=all,-fno-omit-frame-pointer,-g"]


def build(force=False, verbose=False, jobs=None, bounds=False, sanitize=False):
    build_dir = BUILD + ("_bounds" if bounds else "_asan" if sanitize else "")
    lib = BOUNDS_LIB if bounds else (ASAN_LIB if sanitize else LIB)
    extra = ["-DQMCKL_BOUNDS_CHECK"] if bounds else (SANITIZE if sanitize else [])
    os.makedirs(build_dir, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sources()
    if force:
        for f in os.listdir(build_dir):
            if f.endswith(".o"):
                os.remove(os.path.join(build_dir, f))
    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, build_dir, extra), srcs))
    if (not force and os.path.exists(lib)
            and os.path.getmtime(lib) >= max(os.path.getmtime(o) for o in objs)):
        return lib
    tmp = lib + ".tmp%d" % os.getpid()
    cmd = [nvcc()] + ARCH + (SANITIZE if sanitize else []) + ["-shared", "-o", tmp] + objs + ["-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv, bounds="--bounds" in sys.argv,
                sanitize="--sanitize" in sys.argv))

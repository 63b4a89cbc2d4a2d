"""Host code under AddressSanitizer and UndefinedBehaviorSanitizer (CPU only; compute-sanitizer is
not available for the device side, whose stores the bounds-checked build covers instead):

- the oracle (oracle/qmckl_oracle.c) built with -fsanitize=address,undefined runs the CHBrClF
  molecule, the small and adjoint systems, NaN coordinates, the per-nucleus tables, distances and
  the FP64 reference gradient, and must give the normal build's bits;
- the C ABI's host-side argument paths (tests/test_capi.py: NULL and invalid contexts, bad sizes,
  setter order, masks, registries, test hooks; tests/test_trexio.py: the TREXIO reader's binding,
  file opening and table conversion) run against the library whose host code is built with the
  same sanitizers.

Each runs in a child process with libasan preloaded; any report aborts the child."""
import os
import shutil
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="no host C compiler")


def _asan_env(**extra):
    libasan = subprocess.run(["gcc", "-print-file-name=libasan.so"], capture_output=True, text=True).stdout.strip()
    if not os.path.isabs(libasan) or not os.path.exists(libasan):
        pytest.skip("libasan not available")
    env = dict(os.environ, LD_PRELOAD=libasan, ASAN_OPTIONS="detect_leaks=0:halt_on_error=1:protect_shadow_gap=0:allocator_may_return_null=1",
               UBSAN_OPTIONS="halt_on_error=1:print_stacktrace=1", **extra)
    return env


ORACLE_CHILD = r"""
import sys
import numpy as np
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[1] + "/tests")
from oracle import oracle
from qmckl_sycl_gb300.systems import System, config_adjoint, config_small
from test_oracle_golden import nan_points

chbrclf = System.from_npz(sys.argv[1] + "/tests/golden/chbrclf.npz")
sub = config_adjoint(0)
sub = sub.with_points(sub.coord[:96])
out = {}
for name, s in (("chbrclf", chbrclf), ("small", config_small(0)), ("adjoint96", sub),
                ("nan", nan_points(config_small(9, point_num=40)))):
    for k, v in oracle.forward(s).items():
        out["%s_%s" % (name, k)] = v
    out[name + "_shell_vgl"] = oracle.shell_vgl(s)
    out[name + "_en"] = oracle.en_distance(s)
hpc = oracle.finalize_hpc(chbrclf)
for k in hpc:
    out["hpc_" + k] = np.asarray(hpc[k])
w = np.random.default_rng(2).normal(size=(sub.point_num, 5, sub.mo_num))
for k, v in oracle.vjp_mo_vgl(sub, w, threads=1).items():  # one thread: a fixed summation order
    out["vjp_" + k] = v
np.savez(sys.argv[2], **out)
print("oracle ok")
"""


def test_oracle_under_address_and_undefined_behaviour_sanitizers(tmp_path):
    sys.path.insert(0, ROOT)
    from oracle import oracle

    oracle.build_oracle(sanitize=True)
    oracle.build_oracle()
    san, plain = tmp_path / "san.npz", tmp_path / "plain.npz"
    r = subprocess.run([sys.executable, "-c", ORACLE_CHILD, ROOT, str(san)], capture_output=True, text=True,
                       timeout=600, env=_asan_env(QMCKL_ORACLE_SANITIZE="1"))
    assert r.returncode == 0 and "oracle ok" in r.stdout, r.stdout[-3000:] + r.stderr[-6000:]
    r = subprocess.run([sys.executable, "-c", ORACLE_CHILD, ROOT, str(plain)], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    import numpy as np

    a, b = np.load(san), np.load(plain)
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        assert np.array_equal(a[k], b[k], equal_nan=True), k


def test_c_abi_argument_paths_under_address_and_undefined_behaviour_sanitizers():
    from qmckl_sycl_gb300 import build

    build.build(sanitize=True)
    build.build()
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-p", "no:cacheprovider",
                        os.path.join(ROOT, "tests", "test_capi.py"), os.path.join(ROOT, "tests", "test_trexio.py")],
                       capture_output=True, text=True, timeout=900,
                       cwd=ROOT, env=_asan_env(QMCKL_GB300_SANITIZE="1"))
    assert r.returncode == 0 and " passed" in r.stdout, r.stdout[-4000:] + r.stderr[-4000:]

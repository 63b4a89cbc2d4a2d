"""Error bounds of the split-BF16 AO kernel's FP32 pair arithmetic, checked on the CPU.

tests/pair_emulation.c restates that kernel's primitive evaluation and radial sums in binary32 C
(fmaf, no other contraction) and compares them with long double on the test bases: every primitive
value within 2e-10 relative (the bound the GPU test test_split_form_primitive_values applies to
the kernel itself), and the shell quantities R, the radial gradient factor and the Laplacian's radial
part within the FP32 rounding of their results against the sum of their terms' magnitudes (the
Laplacian's cancellation costs nothing beyond that rounding)."""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from oracle import oracle
from qmckl_sycl_gb300.systems import System, config_contracted, config_medium, config_small

HERE = os.path.dirname(os.path.abspath(__file__))
PRIM_BOUND = 2e-10
SHELL_BOUND = 6.5e-8  # FP32 rounding of the result: 2^-24 = 5.96e-8 of its magnitude, plus the pair's own error


@pytest.fixture(scope="module")
def emulator(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = str(tmp_path_factory.mktemp("pair") / "pair_emulation")
    subprocess.run([cc, "-O2", "-ffp-contract=off", "-o", exe, os.path.join(HERE, "pair_emulation.c"), "-lm"],
                   check=True)
    return exe


def _bases():
    return {"chbrclf": System.from_npz(os.path.join(HERE, "golden", "chbrclf.npz")), "medium": config_medium(0, 1, 2),
            "small": config_small(3), "contracted": config_contracted(0, 64)}


@pytest.mark.parametrize("name", ["chbrclf", "medium", "small", "contracted"])
def test_pair_arithmetic_error_bounds(name, emulator):
    s = _bases()[name]
    cn = oracle.finalize(s)["coefficient_normalized"]
    data = np.stack([s.exponent, cn]).T.astype(np.float64)
    blob = struct.pack("<q", data.shape[0]) + data.tobytes()
    out = subprocess.run([emulator], input=blob, capture_output=True, check=True).stdout.decode()
    fields = {line.split()[0]: [float(x) for x in line.split()[1:]] for line in out.splitlines()}
    prim_err, evals = fields["prim"]
    r_err, g_err, rt_err = fields["shell"]
    print("%s: primitive max rel err %.2e over %d values; shell R %.2e, 2G %.2e, Rt %.2e" % (
        name, prim_err, evals, r_err, g_err, rt_err))
    assert evals > 1000
    assert prim_err <= PRIM_BOUND
    assert max(r_err, g_err, rt_err) <= SHELL_BOUND

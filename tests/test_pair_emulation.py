"""Error bounds of the split-BF16 AO kernel's FP32 pair arithmetic, checked on the CPU.

tests/pair_emulation.c restates that kernel's primitive evaluation and radial sums in binary32 C
(fmaf, no other contraction) and compares them with long double on the test bases: every primitive
value within 2e-10 relative (the bound the GPU test test_split_form_primitive_values applies to
the kernel itself), and the shell quantities R, the radial gradient factor and the Laplacian's radial
part within the FP32 rounding of their results against the sum of their terms' magnitudes (the
Laplacian's cancellation costs nothing beyond that rounding). A numpy float32 emulation of the
kernel's FP32 assembly of each AO's Laplacian bounds what that assembly adds, normwise, at AO level
and after the contraction with the MO coefficients."""
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


def _laplacians(s, npts):
    """The AO Laplacian rows of the first npts points: FP64 (the FP64 form's formulas) and as the
    split-BF16 planes kernel assembles them in FP32 (powers, P, and lap = fma(P, Rt, e(e-1) R m)
    from R and Rt rounded once to FP32; the kernel forms Rt in pair arithmetic, to ~2^-44, before that
    rounding). fma is emulated in float64 (exact products of floats)."""
    f32 = np.float32
    cn = oracle.finalize(s)["coefficient_normalized"]
    co = s.coord[:npts]
    shell_nuc = np.repeat(np.arange(s.nucl_num), s.nucleus_shell_num)
    cols64, cols32 = [], []
    for si in range(s.shell_num):
        n, l = shell_nuc[si], int(s.shell_ang_mom[si])
        d = co - s.nucl_coord[:, n][None, :]
        r2 = (d * d).sum(1)
        p0, pn = s.shell_prim_index[si], s.shell_prim_num[si]
        a, c = s.exponent[p0:p0 + pn], cn[p0:p0 + pn]
        ar2 = a[None, :] * r2[:, None]
        v = np.where(ar2 > 27.631021115928547, 0.0, c[None, :] * np.exp(-ar2))
        R = v.sum(1)
        Rt = (v * (4 * a[None, :] ** 2 * r2[:, None] - 2 * a[None, :] * (3 + 2 * l))).sum(1)
        Rf, Rtf = R.astype(f32), Rt.astype(f32)
        X64, X32 = d.T, d.T.astype(f32)
        for ea in range(l, -1, -1):
            for eb in range(l - ea, -1, -1):
                e = (ea, eb, l - ea - eb)
                P = X64[0] ** e[0] * X64[1] ** e[1] * X64[2] ** e[2]
                pw = [(X32[k] ** e[k]).astype(f32) for k in range(3)]
                Pf = pw[0] * (pw[1] * pw[2])
                lap = P * Rt
                term = None
                for k in range(3):
                    if e[k] > 1:
                        others = [j for j in range(3) if j != k]
                        lap = lap + e[k] * (e[k] - 1) * R * X64[k] ** (e[k] - 2) * X64[others[0]] ** e[others[0]] * \
                            X64[others[1]] ** e[others[1]]
                        m = (X32[k] ** (e[k] - 2)).astype(f32) * (pw[others[0]] * pw[others[1]])
                        term = (f32(e[k] * (e[k] - 1)) * Rf) * m
                lapf = Pf * Rtf if term is None else (Pf.astype(np.float64) * Rtf + term).astype(f32)
                cols64.append(lap)
                cols32.append(lapf.astype(np.float64))
    return np.stack(cols64, 1), np.stack(cols32, 1)


@pytest.mark.parametrize("name", ["chbrclf", "medium", "small", "contracted"])
def test_fp32_laplacian_assembly_error(name):
    # the planes kernel assembles each AO's Laplacian in FP32; normwise against the FP64 assembly it
    # adds about 1e-7 at most, at AO level and after the FP64 contraction with the MO coefficients
    s = _bases()[name]
    lap64, lap32 = _laplacians(s, 1024)
    C = s.mo_coef.T
    ao_err = np.linalg.norm(lap32 - lap64) / np.linalg.norm(lap64)
    mo_err = np.linalg.norm((lap32 - lap64) @ C) / np.linalg.norm(lap64 @ C)
    print("%s: FP32 Laplacian assembly, normwise AO %.2e, MO %.2e" % (name, ao_err, mo_err))
    assert ao_err <= 2e-7 and mo_err <= 2e-7

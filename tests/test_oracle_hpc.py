"""Pins the oracle's restatement of the reference's per-nucleus exponent tables
(qmckl_finalize_ao_basis_hpc_device, src/qmckl_ao_sycl.cpp:855-1065): against the tables the
unmodified reference leaves in its context for CHBrClF (tests/golden/chbrclf_hpc.npz, made by
tests/golden/make_golden_hpc.py), and bit for bit against the reference built on this host on
bases with merged exponents and an empty nucleus (when the reference checkout is present)."""
import os

import numpy as np
import pytest

from oracle import oracle
from qmckl_sycl_gb300.systems import config_small

HPC_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "chbrclf_hpc.npz")
KEYS = ("prim_num_per_nucleus", "expo_per_nucleus", "coef_per_nucleus")


def replace(s, **kw):
    return s.__class__(**{**s.__dict__, **kw})


def shared_exponents(seed):
    # exponents on a coarse grid: many repeat within a nucleus and within a shell
    s = config_small(seed)
    return replace(s, exponent=np.round(s.exponent) + 1.0)


def empty_nucleus(seed):
    # the shells of nucleus 1 moved to nucleus 0 (same AO order), nucleus 1 left without shells
    s = config_small(seed)
    nsh = s.nucleus_shell_num.copy()
    nidx = s.nucleus_index.copy()
    nsh[0] += nsh[1]
    nsh[1] = 0
    nidx[1] = nidx[2]
    return replace(s, nucleus_shell_num=nsh, nucleus_index=nidx)


def test_oracle_hpc_matches_reference_golden(chbrclf):
    got = oracle.finalize_hpc(chbrclf)
    ref = np.load(HPC_GOLDEN)
    for k in KEYS:
        assert got[k].dtype == ref[k].dtype and np.array_equal(got[k], ref[k]), k
    # CHBrClF's contracted shells share exponents: 297 primitives, 133 distinct per nucleus
    assert got["prim_num_per_nucleus"].tolist() == [22, 11, 22, 31, 47]


@pytest.mark.parametrize("case", ["chbrclf", "small", "shared_exponents", "empty_nucleus"])
def test_oracle_hpc_matches_reference_build(case, chbrclf):
    if oracle.reference_lib() is None:
        pytest.skip("reference build not available on this host")
    s = {"chbrclf": lambda: chbrclf, "small": lambda: config_small(1), "shared_exponents": lambda: shared_exponents(2),
         "empty_nucleus": lambda: empty_nucleus(3)}[case]()
    got = oracle.finalize_hpc(s)
    ref = oracle.reference_hpc(s)
    for k in KEYS:
        assert got[k].shape == ref[k].shape and np.array_equal(got[k], ref[k]), (case, k)
    if case == "shared_exponents":
        assert (got["prim_num_per_nucleus"] < np.bincount(
            np.repeat(np.arange(s.nucl_num), s.nucleus_shell_num), weights=s.shell_prim_num,
            minlength=s.nucl_num)).all()
    if case == "empty_nucleus":
        assert got["prim_num_per_nucleus"][1] == 1  # the reference reports one (zero) entry


def test_hpc_tables_reproduce_the_radials(chbrclf):
    # the merged tables describe the same functions: sum over entries of coef * e^(-a r2) per
    # shell equals the sum over the shell's own primitives
    t = oracle.finalize_hpc(chbrclf)
    cn = oracle.finalize(chbrclf)["coefficient_normalized"]
    r2 = np.array([0.0, 0.3, 1.7, 4.0])
    for n in range(chbrclf.nucl_num):
        u = t["prim_num_per_nucleus"][n]
        e = np.exp(-np.outer(r2, t["expo_per_nucleus"][n, :u]))
        for j in range(chbrclf.nucleus_shell_num[n]):
            sh = chbrclf.nucleus_index[n] + j
            p = slice(chbrclf.shell_prim_index[sh], chbrclf.shell_prim_index[sh] + chbrclf.shell_prim_num[sh])
            direct = (cn[p][None, :] * np.exp(-np.outer(r2, chbrclf.exponent[p]))).sum(axis=1)
            merged = e @ t["coef_per_nucleus"][n, j, :u]
            assert np.allclose(merged, direct, rtol=1e-13, atol=1e-300)

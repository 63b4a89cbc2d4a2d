"""Builds tests/golden/chbrclf_hpc.npz: the per-nucleus exponent tables that the unmodified
reference (built on the host by oracle/Makefile.ref) leaves in its context after finalizing the
CHBrClF basis of tests/golden/chbrclf.npz (qmckl_finalize_ao_basis_hpc_device,
src/qmckl_ao_sycl.cpp:855-1065): prim_num_per_nucleus, expo_per_nucleus, coef_per_nucleus.

    python tests/golden/make_golden_hpc.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main():
    from oracle import oracle
    from qmckl_sycl_gb300.systems import System

    if oracle.build_reference() is None:
        sys.exit("the reference checkout is needed to build the reference library")
    s = System.from_npz(os.path.join(HERE, "chbrclf.npz"))
    t = oracle.reference_hpc(s)
    np.savez_compressed(os.path.join(HERE, "chbrclf_hpc.npz"), **t)
    print({k: v.shape for k, v in t.items()})


if __name__ == "__main__":
    main()

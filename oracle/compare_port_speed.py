"""Times the oracle port (oracle/qmckl_oracle.c) against the unmodified reference built on this
host (oracle/_ref/libqmckl_ref.so, oracle/Makefile.ref) on the same inputs and thread count, to
show whether the port is a fair stand-in for the reference's speed where the reference cannot be
built (the GPU machine): the reference's timed call is qmckl_context_touch_device +
qmckl_get_mo_basis_mo_vgl_device (src/qmckl_mo.cpp:295), the port's the same recompute
(shell radials, polynomials, assembly, MO contraction). Prints a markdown table.

TEST INFRASTRUCTURE: runs the oracle and the reference build, nothing of the product.

    OMP_NUM_THREADS=<n> python oracle/compare_port_speed.py [walkers ...]
"""
import os
import platform
import statistics
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path[0] = os.path.dirname(HERE)  # the repository root, not oracle/ (whose oracle.py would shadow the package)

from oracle import oracle  # noqa: E402
from qmckl_sycl_gb300.systems import config_medium  # noqa: E402


def cpu_model():
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def main(walkers):
    if oracle.reference_lib() is None:
        sys.exit("the reference build (oracle/_ref/libqmckl_ref.so) is not available on this machine")
    threads = oracle.lib().oracle_num_threads()
    print("| points | AOs | MOs | reference s (median of 3) | port s (median of 3) | port / reference time |")
    print("|---|---|---|---|---|---|")
    for w in walkers:
        s = config_medium(0, walkers=w, electrons=160)
        ref = oracle.reference_time_mo_vgl(s, 3)
        port = []
        for _ in range(3):
            t0 = time.perf_counter()
            oracle.forward(s, want=("mo_vgl",))
            port.append(time.perf_counter() - t0)
        r, p = statistics.median(ref), statistics.median(port)
        print("| %d | %d | %d | %.3f | %.3f | %.2f |" % (s.point_num, s.ao_num, s.mo_num, r, p, p / r))
        sys.stdout.flush()
    print()
    print("%d threads (OpenMP) on %s, %s; medium workload's basis (seed 0), the first walkers' points" % (
        threads, cpu_model(), platform.machine()))
    assert np.isfinite(r)


if __name__ == "__main__":
    main([int(x) for x in sys.argv[1:]] or [4, 16])

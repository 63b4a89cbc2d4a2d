"""Large point sets: 1,048,576 points of the medium basis (25.6 times the benchmarked workload;
47.5 GB of FP64 ao_vgl and 36.5 GB of BF16 planes on the device, 12.6 GB of mo_vgl in host memory),
both forms, through the host-buffer getter (the split-BF16 form's chunked path). Points are
independent, so a random sample of 2048 of them, evaluated by the oracle on their own, checks the
rows at those points: FP64 within 1e-12, split-BF16 within 1e-6 normwise per component."""
import numpy as np
import pytest

from conftest import normwise_rel_err
from oracle import oracle
from qmckl_sycl_gb300 import PRECISION_FP64, PRECISION_SPLIT_BF16, Context, config_medium

pytestmark = pytest.mark.gpu


def _available_gb():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) / 1e6
    except OSError:
        pass
    return 0.0


@pytest.mark.skipif(_available_gb() < 64.0, reason="less than 64 GB of host memory available")
@pytest.mark.parametrize("mode,tol", [(PRECISION_SPLIT_BF16, 1e-6), (PRECISION_FP64, 1e-12)])
def test_million_points_sampled_against_oracle(mode, tol):
    s = config_medium(0, walkers=6554, electrons=160)  # 1,048,640 points
    P = s.point_num
    sample = np.sort(np.random.default_rng(17).choice(P, size=2048, replace=False))
    ref = oracle.forward(s.with_points(s.coord[sample]), want=("mo_vgl",))["mo_vgl"]
    with Context(0) as ctx:
        ctx.load_system(s)
        ctx.set_precision(mode)
        got = ctx.get_mo_vgl(P)[sample]
    errs = [normwise_rel_err(got[:, c:c + 1], ref[:, c:c + 1]) for c in range(5)]
    print("%d points, mode %d: sampled normwise error per component %s" % (P, mode, " ".join("%.2e" % e for e in errs)))
    assert max(errs) <= tol

"""Device-side failure handling of the split-BF16 contraction, exercised without faulting the
GPU: every mbarrier wait of that kernel is bounded, and on expiry the kernel records an error
word, releases its tensor memory and returns; the host reports QMCKL_FAILURE_DEVICE. The test
hook qmckl_set_split_wait_test_device gives the kernel a short wait limit and a producer that
issues no loads, so that the consumers wait on a barrier that nothing completes. (The
reference has error codes only: src/qmckl_basic_functions.cpp:51.) The same context must then
compute the right result: the abort path left nothing behind (tensor memory released, no
sticky CUDA error)."""
import numpy as np
import pytest

from conftest import normwise_rel_err
from oracle import oracle
from qmckl_sycl_gb300 import FAILURE, PRECISION_SPLIT_BF16, Context, QmcklError, config_medium, config_small

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("points", [50, 20000])
def test_split_wait_runs_out_then_context_recovers(points):
    # 50 points: one tile; 20000 points through a host buffer: the chunked path with its copy stream
    s = config_small(0) if points == 50 else config_medium(0, walkers=125, electrons=160)
    ref = oracle.forward(s, want=("mo_vgl",))["mo_vgl"]
    P = s.point_num
    with Context(0) as ctx:
        ctx.load_system(s)
        ctx.set_precision(PRECISION_SPLIT_BF16)
        ctx.call("set_split_wait_test", 200000, 1)  # ~0.1 ms at 2 GHz; no operand loads
        for _ in range(2):
            with pytest.raises(QmcklError) as e:
                ctx.get_mo_vgl(P)
            assert e.value.code == FAILURE
            assert "timed out" in e.value.message
        # a limit long enough for the real pipeline: the kernel completes normally
        ctx.call("set_split_wait_test", 20000000, 0)
        got = ctx.get_mo_vgl(P)
        assert normwise_rel_err(got, ref) <= 1e-6
        ctx.call("set_split_wait_test", 0, 0)
        ctx.touch()
        again = ctx.get_mo_vgl(P)
        assert np.array_equal(again, got)

"""Failure detection without a GPU fault: every device-side wait of the tcgen05
kernels is bounded and reports CORR_ERR_DEVICE_TIMEOUT to the host.  The
diagnostic entry point makes one such wait run out (an mbarrier phase that
nothing completes) and the same context must keep working afterwards."""
import time

import pytest

from corr_gb300._lib import CorrError
from oracle import oracle as O

pytestmark = pytest.mark.gpu

CORR_ERR_DEVICE_TIMEOUT = 4


@pytest.mark.parametrize("limit_ms", [20, 200])
def test_bounded_wait_times_out_and_context_survives(ctx, limit_ms):
    t0 = time.perf_counter()
    with pytest.raises(CorrError) as err:
        ctx.selftest_wait_timeout(limit_ms)
    dt = time.perf_counter() - t0
    assert err.value.status == CORR_ERR_DEVICE_TIMEOUT
    assert limit_ms * 1e-3 <= dt < limit_ms * 1e-3 + 5.0
    # the context (stream, workspace, result block) is still usable
    o, v, X = 4, 130, 70
    B, eps = O.synth_rimp2(o, v, X, 9)
    ref = O.rimp2_energy(B, eps, o, v)
    for prec in ("fp64", "split_fp16"):
        e = ctx.rimp2_energy(B, eps, o, v, X, prec)
        assert abs(e.e_total - ref[2]) <= 1e-6 * abs(ref[2])

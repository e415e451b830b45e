"""GPU test of hc_ctx_wait, the bounded wait for device work (HC_ERR_TIMEOUT).

The work waited for is torch's bounded spin kernel (a fixed number of clock
cycles, about 0.5 s), so the first wait runs out and the second one, without
a limit, returns once the kernel has ended. Nothing faults or hangs.
"""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

HC_ERR_TIMEOUT = -3021


def test_wait_times_out_then_completes():
    import torch
    from hicops_gb300 import dslim, synthetic as S
    ix = dslim.Index(S.SearchParams(maxz=2))
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        torch.cuda._sleep(1_000_000_000)  # ~0.5 s at 2 GHz
    rc = ix.lib.hc_ctx_wait(ix.ctx, C.c_void_p(s.cuda_stream), 0.01)
    assert rc == HC_ERR_TIMEOUT
    assert b"deadline" in ix.lib.hc_last_error(ix.ctx)
    assert ix.lib.hc_ctx_wait(ix.ctx, C.c_void_p(s.cuda_stream), -1.0) == 0
    assert s.query()
    # an idle stream returns at once, also with a zero limit
    assert ix.lib.hc_ctx_wait(ix.ctx, None, 0.0) == 0
    ix.close()

"""vta_sma_batch_device_noalloc: the SMA sweep without device allocation.

Called through the C ABI and compared with vta_sma_batch_device (the
allocating entry point) on three consecutive calls with different series,
lengths and sweeps, so the second call runs on scratch the first one left
behind.  Both run the same kernels, so the results are expected to agree
bit for bit; the test allows 1e-6 relative.  Collected last on purpose: it
must pass both in a fresh process and after every other GPU test.
"""
import ctypes as C
import re

import numpy as np
import pytest

from vectorta_gb300 import _native as N
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu

_HDR = open(N.HEADER).read()
MAX_LEN = int(re.search(r"#define VTA_NOALLOC_MAX_LEN (\d+)", _HDR).group(1))
MAX_COMBOS = int(re.search(r"#define VTA_NOALLOC_MAX_COMBOS (\d+)", _HDR).group(1))
RTOL = 1e-6


def _sweep(start, end, step):
    s = N.SWEEPS["period"]()
    s.period = N.RangeUsize(start, end, step)
    return s


def _noalloc(ctx, d_x, n, first, sweep, d_out):
    L = N.lib()
    return L.vta_sma_batch_device_noalloc(ctx.handle, d_x.data_ptr(), n, first, C.byref(sweep),
                                          d_out.data_ptr())


def _case(seed, n, lead):
    x = datagen.random_walk(n, seed=seed).astype(np.float32)
    x[:lead] = np.nan
    return x, lead


def test_noalloc_matches_allocating_entry_point_on_consecutive_calls():
    import torch

    ref_ctx = V.Context(0)
    ctx = V.Context(0)
    sma = V.CudaSma(0, ctx=ref_ctx)
    # the third case sweeps a descending range (300, 293, ..., 20)
    cases = [(_case(11, 200_000, 7), (5, 400, 5)), (_case(12, 150_001, 0), (2, 1000, 37)),
             (_case(13, 50_000, 3), (300, 20, 7))]
    for i, ((x, first), rng) in enumerate(cases):
        n = x.size
        sweep = _sweep(*rng)
        rows = len(sma.expand_grid({"period": rng}))
        d_x = torch.from_numpy(x).cuda()
        d_ref = torch.empty(rows, n, device="cuda")
        d_got = torch.full((rows, n), 7.0, device="cuda")
        sma.batch_device([d_x], n, first, {"period": rng}, [d_ref])
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        N.check(_noalloc(ctx, d_x, n, first, sweep, d_got))
        free_after = torch.cuda.mem_get_info()[0]
        if i > 0:
            assert free_after == free_before, "device memory changed during the call"
        assert ctx.scratch_bytes == 0
        assert ctx.last_kernel == "sma_noalloc"
        ref = d_ref.cpu().numpy()
        got = d_got.cpu().numpy()
        assert np.array_equal(np.isnan(got), np.isnan(ref)), f"call {i + 1}: NaN positions differ"
        m = ~np.isnan(ref)
        np.testing.assert_allclose(got[m], ref[m], rtol=RTOL, atol=0, err_msg=f"call {i + 1}")
    ctx.close()
    ref_ctx.close()


def test_noalloc_rejects_sizes_beyond_its_limits():
    import torch

    ctx = V.Context(0)
    n = MAX_LEN + 1
    d_x = torch.zeros(n, device="cuda")
    d_out = torch.empty(n, device="cuda")
    st = _noalloc(ctx, d_x, n, 0, _sweep(5, 5, 0), d_out)
    assert st == 4  # VTA_ERR_INVALID_INPUT
    assert "VTA_NOALLOC_MAX_LEN" in N.lib().vta_last_error().decode()

    n = 5000
    d_x = torch.ones(n, device="cuda")
    d_out = torch.empty(MAX_COMBOS + 4, n, device="cuda")
    st = _noalloc(ctx, d_x, n, 0, _sweep(1, MAX_COMBOS + 4, 1), d_out)
    assert st == 4
    assert "VTA_NOALLOC_MAX_COMBOS" in N.lib().vta_last_error().decode()
    # a huge sweep is refused from its count, before anything is expanded
    st = _noalloc(ctx, d_x, n, 0, _sweep(1, 10**15, 1), d_out)
    assert st == 4
    assert "VTA_NOALLOC_MAX_COMBOS" in N.lib().vta_last_error().decode()
    ctx.close()

"""*_batch_into_host_f32 with output buffers in vta_pinned_alloc memory: the
kernels store into them directly (policy host_out=direct, the default); the
values must equal the staged path's (device buffer + copy) bit for bit, for
one- and three-output indicators, and for a buffer at an offset inside a
pinned block.  Buffers in ordinary (pageable) memory take the staged path."""
import numpy as np
import pytest

from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu

N = 50_000


def inputs(name):
    x = datagen.random_walk(N, seed=61, nan_lead=9).astype(np.float32)
    h, l = datagen.high_low(x.astype(np.float64), seed=62)
    h, l = h.astype(np.float32), l.astype(np.float32)
    return {"willr": [h, l, x], "donchian": [h, l], "adx": [h, l, x]}.get(name, [x])


SWEEPS = {
    "ema": {"period": (2, 120, 1)}, "rsi": {"period": (2, 90, 1)}, "stddev": {"period": (5, 60, 5)},
    "willr": {"period": (5, 80, 5)}, "donchian": {"period": (5, 80, 5)}, "adx": {"period": (2, 60, 2)},
}


@pytest.mark.parametrize("name", ["ema", "rsi", "stddev", "willr", "donchian", "adx"])
def test_direct_equals_staged(name):
    ind = V.CLASSES[name](0)
    ins = inputs(name)
    sw = SWEEPS[name]
    if name == "stddev":
        sw = dict(sw, nbdev=(1.0, 1.0, 0.0))
    rows = len(ind.expand_grid(sw))
    ind.set_policy("host_out", "copy")
    ref, r, c = ind.batch_into_host_f32(*ins, sweep=sw)
    ref = ref if isinstance(ref, tuple) else (ref,)
    outs = [V.pinned_empty((rows, N)) for _ in ref]
    for o in outs:
        o.fill(12345.0)
    ind.set_policy("host_out", "direct")
    got, r2, c2 = ind.batch_into_host_f32(*ins, sweep=sw, out=outs)
    got = got if isinstance(got, tuple) else (got,)
    assert (r2, c2) == (r, c) == (rows, N)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b, equal_nan=True), name


def test_offset_and_partial_buffers():
    ind = V.CLASSES["ema"](0)
    (x,) = inputs("ema")
    sw = {"period": (3, 40, 1)}
    rows = len(ind.expand_grid(sw))
    ref, _, _ = ind.batch_into_host_f32(x, sweep=sw)
    # a view at an offset inside one pinned block
    blk = V.pinned_empty(rows * N + 1000)
    view = blk[1000:].reshape(rows, N)
    got, _, _ = ind.batch_into_host_f32(x, sweep=sw, out=[view])
    assert np.array_equal(got, ref, equal_nan=True)
    # ordinary (pageable) memory: staged
    plain = np.empty((rows, N), np.float32)
    got3, _, _ = ind.batch_into_host_f32(x, sweep=sw, out=[plain])
    assert np.array_equal(got3, ref, equal_nan=True)

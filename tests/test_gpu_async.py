"""The device-pointer entry points return once their work is queued (like the
crate's x_batch_device): several calls back to back on one context, each with
a different period list (so each stages a fresh upload through the context's
pinned buffer), must give the outputs of the same calls made one at a time,
once the context is synchronised; and a stream switch must order work across
the streams."""
import numpy as np
import pytest

from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu


def test_back_to_back_device_calls_equal_single_calls():
    import torch

    n = 120_000
    x = datagen.random_walk(n, seed=91, nan_lead=11).astype(np.float32)
    d_x = torch.from_numpy(x).cuda()
    sweeps = [{"period": (2 + k, 300 + 7 * k, 1 + k % 3)} for k in range(6)]
    names = ["ema", "sma", "rsi", "dema", "stddev", "willr"]
    torch.cuda.synchronize()
    ctx = V.Context(0)
    inds = {nm: V.CLASSES[nm](0, ctx=ctx) for nm in names}
    hi, lo = datagen.high_low(x.astype(np.float64), seed=92)
    d_h = torch.from_numpy(hi.astype(np.float32)).cuda()
    d_l = torch.from_numpy(lo.astype(np.float32)).cuda()
    ins = {"willr": [d_h, d_l, d_x]}
    outs, exp = [], []
    for nm, sw in zip(names, sweeps):
        if nm == "stddev":
            sw = dict(sw, nbdev=(1.0, 1.0, 0.0))
        rows = len(inds[nm].expand_grid(sw))
        o = torch.empty(rows, n, device="cuda")
        inds[nm].batch_device(ins.get(nm, [d_x]), n, 11, sw, [o])  # no wait between the calls
        outs.append(o)
        ref_in = [a.cpu().numpy() for a in ins.get(nm, [d_x])]
        exp.append((nm, sw, ref_in))
    ctx.synchronize()
    for o, (nm, sw, ref_in) in zip(outs, exp):
        single = V.CLASSES[nm](0).batch_dev(*ref_in, sweep=sw).to_host()
        assert np.array_equal(o.cpu().numpy(), single, equal_nan=True), nm


def test_stream_switch_orders_the_work():
    import torch

    n = 200_000
    x = datagen.random_walk(n, seed=93, nan_lead=0).astype(np.float32)
    d_x = torch.from_numpy(x).cuda()
    ctx = V.Context(0)
    ema = V.CLASSES["ema"](0, ctx=ctx)
    sw = {"period": (2, 400, 1)}
    o = torch.empty(len(ema.expand_grid(sw)), n, device="cuda")
    torch.cuda.synchronize()
    ema.batch_device([d_x], n, 0, sw, [o])
    s = torch.cuda.Stream()
    ctx.set_stream(s.cuda_stream)  # waits for the work queued on the old stream
    with torch.cuda.stream(s):
        got = o.cpu().numpy()
    ref = V.CLASSES["ema"](0).batch_dev(x, sweep=sw).to_host()
    assert np.array_equal(got, ref, equal_nan=True)

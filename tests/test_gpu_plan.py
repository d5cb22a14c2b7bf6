"""Many-series work-list plans (vta_tm_plan_*) through the C ABI.

* Ragged OHLCV series (uneven lengths and NaN leads, NaN tail past each end):
  ATR(14), ADX(14), SuperTrend(10, 3.0) and percentile(50, 50%) in one plan,
  each series checked against the FP64 oracle over its own length with the
  tolerances of the many-series parity tests.
* The chunked run (warm restarts verified on the device) is bit-identical to a
  one-chunk-per-series run, also when the warm restart is made too short to
  converge so that the fix-up pass has to repair chunks.
* Cells past a series' length are not written; replaying the graph after
  rewriting the inputs in place gives the results of the new data.
* On full-length series the sequential plan equals the sequential many-series
  kernels of ADX and SuperTrend bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as O
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu

TOL = {"atr": 1e-4, "adx": 3e-2, "supertrend": 7e-4, "percentile_nearest_rank": 1e-4}
SENTINEL = 12345.0
JOBS = [("atr", 14, 0.0), ("adx", 14, 0.0), ("supertrend", 10, 3.0), ("percentile_nearest_rank", 50, 50.0)]


def assert_close(gpu, cpu, tol, what):
    gpu = np.asarray(gpu, dtype=np.float64)
    cpu = np.asarray(cpu, dtype=np.float64)
    gn, cn = np.isnan(gpu), np.isnan(cpu)
    bad = np.argwhere(gn != cn)
    assert bad.size == 0, f"{what}: NaN mask differs at {bad[:5].tolist()}"
    m = ~cn
    diff = np.abs(gpu[m] - cpu[m])
    lim = tol + tol * np.maximum(np.abs(gpu[m]), np.abs(cpu[m]))
    assert diff.size == 0 or np.all(diff <= lim), f"{what}: max excess {np.max(diff - lim):.3g}"


@pytest.fixture(scope="module")
def ragged():
    d, lens, leads = datagen.ragged_many_series(70, seed=5, min_len=300, max_len=3000, max_nan_lead=60)
    return d, lens, leads


def make_plan(torch, d, lens, ctx=None, chunk=None, warm=None):
    rows, cols = d["close"].shape
    ctx = ctx or V.Context(0)
    if chunk is not None:
        ctx.set_policy("tm_chunk", str(chunk))
    if warm is not None:
        ctx.set_policy("tm_warm", str(warm))
    ins = [torch.from_numpy(np.ascontiguousarray(d[k])).cuda() for k in ("high", "low", "close")]
    outs, jobs = [], []
    for kind, p, prm in JOBS:
        o0 = torch.full((rows, cols), SENTINEL, device="cuda")
        o1 = torch.full((rows, cols), SENTINEL, device="cuda") if kind == "supertrend" else None
        outs.append((o0, o1))
        jobs.append({"kind": kind, "period": p, "param": prm, "out0": o0, "out1": o1})
    plan = V.TmPlan(*ins, cols, rows, lens, jobs, ctx=ctx)
    return plan, ins, outs


def host(outs):
    return [(o0.cpu().numpy(), None if o1 is None else o1.cpu().numpy()) for o0, o1 in outs]


def test_plan_matches_oracle_on_ragged_series(ragged):
    import torch

    d, lens, _ = ragged
    plan, ins, outs = make_plan(torch, d, lens)
    plan.run()
    got = host(outs)
    for j in range(d["close"].shape[1]):
        L = int(lens[j])
        h, l, c = (d[k][:L, j].astype(np.float64) for k in ("high", "low", "close"))
        exp = {"atr": [O.atr(h, l, c, 14)], "adx": [O.adx(h, l, c, 14)],
               "supertrend": list(O.supertrend(h, l, c, 10, 3.0)),
               "percentile_nearest_rank": [O.percentile_nearest_rank(c, 50, 50.0)]}
        for q, (kind, _, _) in enumerate(JOBS):
            for k, e in enumerate(exp[kind]):
                g = got[q][k][:L, j]
                tol = 1e-6 if (kind == "supertrend" and k == 1) else TOL[kind]
                assert_close(g, e, tol, f"{kind}[{k}] series {j} (len {L})")
                assert np.all(got[q][k][L:, j] == SENTINEL), f"{kind}: wrote past the end of series {j}"
    info = plan.info()
    assert info["n_items"] > 0
    plan.close()


def test_chunked_equals_sequential_bitwise(ragged):
    import torch

    d, lens, _ = ragged
    seq, _, o_seq = make_plan(torch, d, lens, chunk="sequential")
    seq.run()
    ref = host(o_seq)
    for chunk, warm in ((256, None), (300, 2)):
        plan, _, outs = make_plan(torch, d, lens, chunk=chunk, warm=warm)
        plan.run()
        got = host(outs)
        for q, (kind, _, _) in enumerate(JOBS):
            for k in range(2):
                if ref[q][k] is None:
                    continue
                assert np.array_equal(got[q][k], ref[q][k], equal_nan=True), \
                    f"{kind}[{k}] chunk={chunk} warm={warm}: differs from the sequential run"
        info = plan.info()
        assert info["chunk"][0] == chunk
        if warm == 2:
            assert info["fixups"] > 0  # a 2-step warm restart cannot converge: the fix-up pass repaired chunks
        plan.close()
    seq.close()


def test_graph_replay_on_new_data(ragged):
    import torch

    d, lens, _ = ragged
    plan, ins, outs = make_plan(torch, d, lens, chunk=512)
    plan.run()
    d2 = {k: (v * np.float32(1.5)).astype(np.float32) for k, v in d.items()}
    for t, k in zip(ins, ("high", "low", "close")):
        t.copy_(torch.from_numpy(np.ascontiguousarray(d2[k])))
    plan.run()
    fresh, _, o2 = make_plan(torch, d2, lens, chunk="sequential")
    fresh.run()
    for q, (a, b) in enumerate(zip(host(outs), host(o2))):
        assert np.array_equal(a[0], b[0], equal_nan=True), JOBS[q][0]
    plan.close()
    fresh.close()


def test_sequential_plan_equals_many_series_kernels():
    import torch

    rows, cols = 1500, 40
    d, lens, _ = datagen.ragged_many_series(cols, seed=9, min_len=rows, max_len=rows, max_nan_lead=30)
    plan, ins, outs = make_plan(torch, d, None, chunk="sequential")
    plan.run()
    got = host(outs)
    for q, name, params in ((1, "adx", {"period": 14}), (2, "supertrend", {"period": 10, "factor": 3.0})):
        ind = V.CLASSES[name](0)
        r = ind.many_series_one_param_time_major_dev(d["high"], d["low"], d["close"], params=params)
        r = r if isinstance(r, tuple) else (r,)
        for k, arr in enumerate(r):
            assert np.array_equal(got[q][k], arr.to_host(), equal_nan=True), f"{name}[{k}]"
    plan.close()


def test_plan_rejects_bad_jobs():
    import torch

    ctx = V.Context(0)
    x = torch.ones(100, 3, device="cuda")
    o = torch.empty(100, 3, device="cuda")
    with pytest.raises(V.VtaError, match="percentile length above"):
        V.TmPlan(x, x, x, 3, 100, None, [{"kind": "percentile_nearest_rank", "period": 65, "param": 50.0,
                                            "out0": o}], ctx=ctx)
    with pytest.raises(V.VtaError, match="SuperTrend needs d_out1"):
        V.TmPlan(x, x, x, 3, 100, None, [{"kind": "supertrend", "period": 10, "param": 3.0, "out0": o}], ctx=ctx)
    with pytest.raises(V.VtaError, match="exceeds rows"):
        V.TmPlan(x, x, x, 3, 100, [100, 101, 5], [{"kind": "atr", "period": 14, "out0": o}], ctx=ctx)

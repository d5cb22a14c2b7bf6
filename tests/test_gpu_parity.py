"""GPU parity: every indicator's CUDA path, called through the C ABI, against
the FP64 CPU oracle on the same (f32-rounded) inputs.

Comparison rule of the crate's GPU tests (tests/alma_cuda.rs:19-28): NaN
positions must match exactly, values satisfy |a-b| <= tol + tol*max(|a|,|b|)
with the per-indicator tolerance the crate's tests use.
"""
import numpy as np
import pytest

from oracle import oracle as O
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu

# crate GPU-test tolerances (tests/<indicator>_cuda.rs)
TOL = {
    "alma": 5e-6, "ema": 5e-5, "dema": 5e-6, "tema": 1e-5, "wilders": 1e-5, "rsi": 5e-4, "atr": 1e-4,
    "adx": 1e-1, "supertrend": 7e-4, "sma": 1e-5, "stddev": 5e-4, "zscore": 5e-4,
    "bollinger_bands": 1e-3, "donchian": 5e-4, "willr": 5e-5, "percentile_nearest_rank": 1e-4,
    "wma": 1e-5, "swma": 2e-4, "pwma": 5e-4, "sinwma": 1e-5, "trima": 1e-4,
    "cwma": 5e-5, "fwma": 5e-4, "srwma": 2e-5, "sqwma": 1e-5, "epma": 2e-5, "vpwma": 5e-4,
}
TOL_TM = dict(TOL, alma=3e-4, adx=3e-2)


def assert_close(gpu, cpu, tol, what):
    gpu = np.asarray(gpu, dtype=np.float64)
    cpu = np.asarray(cpu, dtype=np.float64)
    assert gpu.shape == cpu.shape, (what, gpu.shape, cpu.shape)
    gn, cn = np.isnan(gpu), np.isnan(cpu)
    bad = np.argwhere(gn != cn)
    assert bad.size == 0, f"{what}: NaN mask differs at {bad[:5].tolist()} (gpu={gpu[tuple(bad[0])]}, cpu={cpu[tuple(bad[0])]})"
    m = ~cn
    diff = np.abs(gpu[m] - cpu[m])
    lim = tol + tol * np.maximum(np.abs(gpu[m]), np.abs(cpu[m]))
    if diff.size and not np.all(diff <= lim):
        i = int(np.argmax(diff - lim))
        idx = np.argwhere(m)[i]
        raise AssertionError(f"{what}: mismatch at {idx.tolist()}: gpu={gpu[m][i]!r} cpu={cpu[m][i]!r} "
                             f"(|d|={diff[i]:.3g}, lim={lim[i]:.3g})")


def f32(a):
    return np.asarray(a, dtype=np.float32)


@pytest.fixture(scope="module")
def data():
    n = 4096
    close = f32(datagen.random_walk(n, seed=11, nan_lead=37))
    hi, lo = datagen.high_low(close.astype(np.float64), seed=12)
    hi, lo = f32(hi), f32(lo)
    hi[:37] = np.nan
    lo[:37] = np.nan
    return {"close": close, "high": hi, "low": lo}


def oracle_batch(name, d, sweep):
    c = d["close"].astype(np.float64)
    h = d["high"].astype(np.float64)
    l = d["low"].astype(np.float64)
    if name == "alma":
        out, _ = O.alma_batch(c, sweep["period"], sweep["offset"], sweep["sigma"])
        return [out]
    ps = O.periods_of(name, sweep.get("period", sweep.get("length")))
    if name == "rsi":
        return [O.rsi_batch(c, ps)]
    if name == "sma":
        return [O.sma_batch(c, ps)]
    if name == "wilders":
        return [O.wilders_batch(c, ps)]
    if name == "pwma":
        return [O.rows_of(O.pwma, c, ps, batch=True)]
    simple = {"ema": O.ema, "dema": O.dema, "tema": O.tema, "wma": O.wma, "swma": O.swma,
              "sinwma": O.sinwma, "trima": O.trima, "cwma": O.cwma, "fwma": O.fwma, "srwma": O.srwma,
              "sqwma": O.sqwma}
    if name == "vpwma":
        pws = O.axis_f64(sweep["power"])
        return [np.stack([O.vpwma(c, p, w) for p in ps for w in pws])]
    if name == "epma":
        offs = O.axis_usize(sweep["offset"], O.AX_SWAP)
        return [np.stack([O.epma(c, p, o) for p in ps for o in offs])]
    if name in simple:
        return [O.rows_of(simple[name], c, ps)]
    if name in ("stddev", "zscore"):
        nb = O.axis_f64(sweep["nbdev"])
        fn = O.stddev if name == "stddev" else O.zscore_batch_row
        return [np.stack([fn(c, p, k) for p in ps for k in nb])]
    if name == "bollinger_bands":
        ups, dns = O.axis_f64(sweep["devup"]), O.axis_f64(sweep["devdn"])
        rows = [O.bollinger(c, p, u, dd) for p in ps for u in ups for dd in dns]
        return [np.stack([r[i] for r in rows]) for i in range(3)]
    if name == "atr":
        return [np.stack([O.atr(h, l, c, p) for p in ps])]
    if name == "adx":
        return [np.stack([O.adx(h, l, c, p) for p in ps])]
    if name == "willr":
        return [np.stack([O.willr(h, l, c, p) for p in ps])]
    if name == "donchian":
        rows = [O.donchian(h, l, p) for p in ps]
        return [np.stack([r[i] for r in rows]) for i in range(3)]
    if name == "supertrend":
        fs = O.axis_f64(sweep["factor"])
        rows = [O.supertrend(h, l, c, p, f) for p in ps for f in fs]
        return [np.stack([r[i] for r in rows]) for i in range(2)]
    if name == "percentile_nearest_rank":
        qs = O.axis_f64(sweep["percentage"])
        return [np.stack([O.percentile_nearest_rank(c, p, q) for p in ps for q in qs])]
    raise KeyError(name)


def inputs_of(name, d):
    kind = V.N.INDICATORS[name][0]
    return {"x": [d["close"]], "hl": [d["high"], d["low"]],
            "hlc": [d["high"], d["low"], d["close"]]}[kind]


SWEEPS = {
    "alma": {"period": (5, 40, 1), "offset": (0.5, 0.95, 0.15), "sigma": (3.0, 9.0, 3.0)},
    "ema": {"period": (2, 200, 3)}, "dema": {"period": (2, 200, 3)}, "tema": {"period": (1, 120, 3)},
    "rsi": {"period": (2, 200, 3)}, "wilders": {"period": (1, 150, 3)}, "sma": {"period": (1, 300, 7)},
    "wma": {"period": (2, 120, 3)}, "swma": {"period": (1, 120, 3)}, "pwma": {"period": (1, 60, 3)},
    "sinwma": {"period": (1, 120, 3)}, "trima": {"period": (4, 120, 3)},
    "stddev": {"period": (2, 300, 7), "nbdev": (1.0, 2.0, 1.0)},
    # z-score is ill-conditioned for p = 2 on near-tied inputs (variance at the
    # f32 ulp level); the workload's windows start at 5
    "zscore": {"period": (5, 300, 7), "nbdev": (1.0, 1.0, 0.0)},
    "bollinger_bands": {"period": (2, 300, 7), "devup": (2.0, 2.0, 0.0), "devdn": (1.5, 2.0, 0.5)},
    "atr": {"period": (1, 120, 3)}, "adx": {"period": (2, 60, 3)},
    "supertrend": {"period": (5, 30, 5), "factor": (2.0, 3.0, 1.0)},
    "donchian": {"period": (1, 500, 13)}, "willr": {"period": (1, 500, 13)},
    "percentile_nearest_rank": {"length": (3, 120, 9), "percentage": (25.0, 75.0, 25.0)},
    "cwma": {"period": (2, 120, 3)}, "fwma": {"period": (1, 60, 3)}, "srwma": {"period": (2, 120, 3)},
    "sqwma": {"period": (2, 120, 3)},
    # offsets even, so no combo has a zero weight sum (p - 1 odd, offset 2 + (p - 2) / 2)
    "epma": {"period": (8, 60, 4), "offset": (0, 6, 2)},
    "vpwma": {"period": (2, 120, 3), "power": (0.2, 0.8, 0.3)},
}


@pytest.mark.parametrize("name", sorted(SWEEPS))
def test_batch_matches_oracle(name, data):
    cls = V.CLASSES[name]
    ind = cls(0)
    sweep = SWEEPS[name]
    got = ind.batch_dev(*inputs_of(name, data), sweep=sweep)
    got = got if isinstance(got, tuple) else (got,)
    exp = oracle_batch(name, data, sweep)
    assert len(got) == len(exp)
    for k, (g, e) in enumerate(zip(got, exp)):
        tol = TOL[name] if not (name == "supertrend" and k == 1) else 1e-6
        assert_close(g.to_host(), e, tol, f"{name}[{k}] ({ind.last_kernel})")


@pytest.mark.parametrize("name", sorted(SWEEPS))
def test_batch_entry_points_agree(name, data):
    """batch_dev, batch_into_host_f32 and batch_device give identical results."""
    import torch

    ind = V.CLASSES[name](0)
    sweep = SWEEPS[name]
    ins = inputs_of(name, data)
    a = ind.batch_dev(*ins, sweep=sweep)
    a = a if isinstance(a, tuple) else (a,)
    h, rows, cols = ind.batch_into_host_f32(*ins, sweep=sweep)
    h = h if isinstance(h, tuple) else (h,)
    assert (rows, cols) == a[0].shape
    d_in = [torch.from_numpy(x).cuda() for x in ins]
    d_out = [torch.empty(rows, cols, device="cuda") for _ in a]
    torch.cuda.synchronize()
    first = V.N.INDICATORS[name][0]
    fv = int(np.argmax(~np.isnan(np.stack(ins)).any(axis=0))) if first != "x" else int(np.argmax(~np.isnan(ins[0])))
    ind.batch_device(d_in, cols, fv, sweep, d_out)
    ind.synchronize()  # device entry points return once queued, like the crate's x_batch_device
    for k in range(len(a)):
        ah = a[k].to_host()
        assert np.array_equal(ah, h[k], equal_nan=True)
        assert np.array_equal(ah, d_out[k].cpu().numpy(), equal_nan=True)


def test_into_host_buffer_policies(data):
    """batch_into_host_f32 with the context-cached device buffer (default,
    grown across calls of different sizes) equals the per-call allocation."""
    x = data["close"]
    for name, sweeps in (("ema", ({"period": (2, 30, 1)}, {"period": (2, 200, 1)}, {"period": (5, 9, 2)})),
                         ("donchian", ({"period": (5, 50, 5)}, {"period": (2, 100, 1)}))):
        ind = V.CLASSES[name](0)
        ins = inputs_of(name, data)
        for sw in sweeps:
            ind.set_policy("host_io", "cached")
            a, r, c = ind.batch_into_host_f32(*ins, sweep=sw)
            ind.set_policy("host_io", "per_call")
            b, r2, c2 = ind.batch_into_host_f32(*ins, sweep=sw)
            a = a if isinstance(a, tuple) else (a,)
            b = b if isinstance(b, tuple) else (b,)
            assert (r, c) == (r2, c2) == (a[0].shape[0], x.size)
            for u, v in zip(a, b):
                assert np.array_equal(u, v, equal_nan=True), (name, sw)
        ind.set_policy("host_io", "cached")


def tm_matrix(seed, cols=7, rows=1500):
    """cols series, series j with a NaN lead of j*3 bars (tests/alma_cuda.rs:107-113)."""
    c = np.full((rows, cols), np.nan)
    h = np.full((rows, cols), np.nan)
    l = np.full((rows, cols), np.nan)
    for j in range(cols):
        x = datagen.random_walk(rows, seed=seed + j)
        hi, lo = datagen.high_low(x, seed=seed + 100 + j)
        lead = 3 * j
        c[lead:, j], h[lead:, j], l[lead:, j] = x[lead:], hi[lead:], lo[lead:]
    return f32(c), f32(h), f32(l)


PARAMS = {
    "alma": {"period": 14, "offset": 0.85, "sigma": 6.0}, "ema": {"period": 21}, "dema": {"period": 21},
    "tema": {"period": 21}, "rsi": {"period": 14}, "wilders": {"period": 14}, "sma": {"period": 20},
    "wma": {"period": 20}, "swma": {"period": 20}, "pwma": {"period": 11}, "sinwma": {"period": 20},
    "trima": {"period": 20}, "stddev": {"period": 20, "nbdev": 2.0}, "zscore": {"period": 20, "nbdev": 1.0},
    "bollinger_bands": {"period": 20, "devup": 2.0, "devdn": 2.0}, "atr": {"period": 14},
    "adx": {"period": 14}, "supertrend": {"period": 10, "factor": 3.0}, "donchian": {"period": 20},
    "willr": {"period": 14}, "percentile_nearest_rank": {"length": 50, "percentage": 50.0},
    "cwma": {"period": 14}, "fwma": {"period": 10}, "srwma": {"period": 14}, "sqwma": {"period": 14},
    "epma": {"period": 11, "offset": 4}, "vpwma": {"period": 14, "power": 0.382},
}


def oracle_series(name, c, h, l, prm):
    p = prm.get("period", prm.get("length"))
    fn = {
        "alma": lambda: [O.alma(c, p, prm["offset"], prm["sigma"])], "ema": lambda: [O.ema(c, p)],
        "dema": lambda: [O.dema(c, p)], "tema": lambda: [O.tema(c, p)], "rsi": lambda: [O.rsi(c, p)],
        "wilders": lambda: [O.wilders(c, p)], "sma": lambda: [O.sma(c, p)], "wma": lambda: [O.wma(c, p)],
        "swma": lambda: [O.swma(c, p)], "pwma": lambda: [O.pwma(c, p)], "sinwma": lambda: [O.sinwma(c, p)],
        "trima": lambda: [O.trima(c, p)], "stddev": lambda: [O.stddev(c, p, prm["nbdev"])],
        "zscore": lambda: [O.zscore(c, p, prm["nbdev"])],
        "bollinger_bands": lambda: list(O.bollinger(c, p, prm["devup"], prm["devdn"])),
        "atr": lambda: [O.atr(h, l, c, p)], "adx": lambda: [O.adx(h, l, c, p)],
        "supertrend": lambda: list(O.supertrend(h, l, c, p, prm["factor"])),
        "donchian": lambda: list(O.donchian(h, l, p)), "willr": lambda: [O.willr(h, l, c, p)],
        "percentile_nearest_rank": lambda: [O.percentile_nearest_rank(c, p, prm["percentage"])],
        "cwma": lambda: [O.cwma(c, p)], "fwma": lambda: [O.fwma(c, p)], "srwma": lambda: [O.srwma(c, p)],
        "sqwma": lambda: [O.sqwma(c, p)], "epma": lambda: [O.epma(c, p, prm["offset"])],
        "vpwma": lambda: [O.vpwma(c, p, prm["power"])],
    }[name]
    return fn()


@pytest.mark.parametrize("name", sorted(PARAMS))
def test_many_series_matches_oracle(name):
    c, h, l = tm_matrix(seed=500)
    kind = V.N.INDICATORS[name][0]
    ins = {"x": [c], "hl": [h, l], "hlc": [h, l, c]}[kind]
    ind = V.CLASSES[name](0)
    got = ind.many_series_one_param_time_major_dev(*ins, params=PARAMS[name])
    got = got if isinstance(got, tuple) else (got,)
    got = [g.to_host() for g in got]
    rows, cols = c.shape
    exp = [np.full((rows, cols), np.nan) for _ in got]
    for j in range(cols):
        res = oracle_series(name, c[:, j].astype(np.float64), h[:, j].astype(np.float64),
                            l[:, j].astype(np.float64), PARAMS[name])
        for k in range(len(got)):
            exp[k][:, j] = res[k]
    for k in range(len(got)):
        tol = TOL_TM[name] if not (name == "supertrend" and k == 1) else 1e-6
        assert_close(got[k], exp[k], tol, f"{name} tm[{k}] ({ind.last_kernel})")


@pytest.mark.parametrize("name", sorted(PARAMS))
def test_many_series_device_entry_agrees(name):
    import torch

    c, h, l = tm_matrix(seed=900, cols=5, rows=700)
    kind = V.N.INDICATORS[name][0]
    ins = {"x": [c], "hl": [h, l], "hlc": [h, l, c]}[kind]
    ind = V.CLASSES[name](0)
    a = ind.many_series_one_param_time_major_dev(*ins, params=PARAMS[name])
    a = a if isinstance(a, tuple) else (a,)
    d_in = [torch.from_numpy(x).cuda() for x in ins]
    d_out = [torch.empty(c.shape, device="cuda") for _ in a]
    torch.cuda.synchronize()
    ind.many_series_one_param_device(d_in, c.shape[1], c.shape[0], PARAMS[name], d_out)
    ind.synchronize()
    for k in range(len(a)):
        assert np.array_equal(a[k].to_host(), d_out[k].cpu().numpy(), equal_nan=True)


# ------------------------------------------------------------- edge cases --
def test_interior_nan_semantics():
    x = f32(datagen.random_walk(600, seed=3, nan_lead=5))
    x[200] = np.nan
    xd = x.astype(np.float64)
    for name, fn, p in (("alma", lambda v, q: O.alma(v, q), 9), ("ema", O.ema, 10), ("sma", O.sma, 10),
                        ("wma", O.wma, 10), ("trima", O.trima, 10), ("pwma", lambda v, q: O.pwma(v, q, True), 7),
                        ("stddev", O.stddev, 10)):
        sweep = {"period": (p, p, 0)}
        if name == "alma":
            sweep = {"period": (p, p, 0), "offset": (0.85, 0.85, 0), "sigma": (6.0, 6.0, 0)}
        if name == "stddev":
            sweep = {"period": (p, p, 0), "nbdev": (1.0, 1.0, 0)}
        g = V.CLASSES[name](0).batch_dev(x, sweep=sweep).to_host()[0]
        assert_close(g, fn(xd, p), TOL[name], f"{name} interior NaN")
    g = V.CudaRsi(0).batch_dev(x, sweep={"period": (14, 14, 0)}).to_host()[0]
    assert_close(g, O.rsi_batch(xd, [14])[0], TOL["rsi"], "rsi batch interior NaN")


def test_weighted_window_family_interior_nan_and_warmup():
    """CWMA / FWMA / SRWMA / SQWMA / EPMA: a NaN inside a window gives NaN
    there and only there, and each row starts at the crate's own warm-up."""
    x = f32(datagen.random_walk(700, seed=5, nan_lead=9))
    x[300] = np.nan
    xd = x.astype(np.float64)
    for name, fn, sweep in (("cwma", O.cwma, {"period": (7, 7, 0)}), ("fwma", O.fwma, {"period": (9, 9, 0)}),
                            ("srwma", O.srwma, {"period": (6, 6, 0)}), ("sqwma", O.sqwma, {"period": (10, 10, 0)})):
        g = V.CLASSES[name](0).batch_dev(x, sweep=sweep).to_host()[0]
        assert_close(g, fn(xd, sweep["period"][0]), TOL[name], f"{name} interior NaN")
    g = V.CudaEpma(0).batch_dev(x, sweep={"period": (11, 11, 0), "offset": (4, 4, 0)}).to_host()[0]
    assert_close(g, O.epma(xd, 11, 4), TOL["epma"], "epma interior NaN")


def test_small_series_and_periods():
    x = f32(datagen.random_walk(40, seed=4, nan_lead=3))
    xd = x.astype(np.float64)
    assert_close(V.CudaEma(0).batch_dev(x, sweep={"period": (1, 37, 1)}).to_host(),
                 O.rows_of(O.ema, xd, range(1, 38)), TOL["ema"], "ema small")
    assert_close(V.CudaSma(0).batch_dev(x, sweep={"period": (1, 37, 1)}).to_host(),
                 O.sma_batch(xd, list(range(1, 38))), TOL["sma"], "sma small")
    assert_close(V.CudaTema(0).batch_dev(x, sweep={"period": (1, 13, 1)}).to_host(),
                 O.rows_of(O.tema, xd, range(1, 14)), TOL["tema"], "tema small")


def test_descending_sweep_order(data):
    g = V.CudaEma(0).batch_dev(data["close"], sweep={"period": (60, 10, 10)})
    assert g.rows == 6
    exp = O.rows_of(O.ema, data["close"].astype(np.float64), [10, 20, 30, 40, 50, 60])
    assert_close(g.to_host(), exp, TOL["ema"], "ema swapped range")


def test_invalid_inputs_raise():
    ind = V.CudaAlma(0)
    with pytest.raises(V.VtaError) as e:
        ind.alma_batch_dev(np.full(100, np.nan, dtype=np.float32), sweep=V.AlmaBatchRange((9, 9, 0)))
    assert e.value.kind == "InvalidInput"
    with pytest.raises(V.VtaError):
        ind.alma_batch_dev(np.arange(10, dtype=np.float32), sweep=V.AlmaBatchRange((20, 20, 0)))
    with pytest.raises(V.VtaError):
        ind.alma_batch_dev(np.arange(100, dtype=np.float32),
                           sweep=V.AlmaBatchRange((9, 9, 0), (0.85, 0.85, 0), (0.0, 0.0, 0)))
    with pytest.raises(V.VtaError):
        V.CudaEma(0).ema_batch_dev(np.zeros(0, dtype=np.float32), sweep={"period": (3, 3, 0)})
    c, h, l = tm_matrix(seed=1, cols=3, rows=50)
    c[:, 1] = np.nan
    with pytest.raises(V.VtaError):
        V.CudaEma(0).ema_many_series_one_param_time_major_dev(c, params={"period": 5})


def test_out_of_memory_carries_its_byte_counts():
    """CudaXError::OutOfMemory{required, free, headroom}: a sweep whose outputs
    exceed the free device memory is refused by the admission check before
    anything that large is allocated, and the error carries the byte counts."""
    import torch

    free, _ = torch.cuda.mem_get_info()
    n = 1 << 24  # 16.8M bars: 64 MB of input
    rows = free // (n * 4) + 64  # outputs larger than all the free memory
    x = datagen.random_walk(n, seed=3).astype(np.float32)
    with pytest.raises(V.VtaError) as e:
        V.CudaEma(0).ema_batch_dev(x, sweep={"period": (2, 1 + int(rows), 1)})
    err = e.value
    assert err.kind == "OutOfMemory"
    assert err.required >= rows * n * 4
    assert 0 < err.free < err.required
    assert err.headroom == 64 << 20
    # a later failure of another kind clears the payload
    with pytest.raises(V.VtaError) as e2:
        V.CudaEma(0).ema_batch_dev(np.zeros(0, dtype=np.float32), sweep={"period": (3, 3, 0)})
    assert e2.value.kind == "InvalidInput" and e2.value.required == 0


def test_golden_fixture_through_gpu(candles, golden):
    """The crate's golden vectors, reproduced by the GPU path on the f32 fixture."""
    c = f32(candles["close"])
    for name, g in golden.items():
        if name not in ("alma", "ema", "dema", "tema", "wma", "sinwma", "sma", "wilders", "rsi"):
            continue
        prm = g["params"]
        sweep = {"period": (prm["period"],) * 2 + (0,)}
        if name == "alma":
            sweep = {"period": (9, 9, 0), "offset": (0.85, 0.85, 0), "sigma": (6.0, 6.0, 0)}
        out = V.CLASSES[name](0).batch_dev(c, sweep=sweep).to_host()[0][-5:].astype(np.float64)
        exp = np.array(g["last5"])
        # f32 input and arithmetic: relative 2e-5 plus the crate's own tolerance
        assert np.all(np.abs(out - exp) <= g["tol"] + 2e-5 * np.abs(exp)), (name, out, exp)


@pytest.mark.parametrize("name,sweep", [
    ("adx", {"period": (5, 60, 5)}),
    ("supertrend", {"period": (7, 21, 7), "factor": (2.0, 3.0, 0.5)}),
])
def test_chunked_hlc_sweeps_equal_sequential(name, sweep):
    """ADX / SuperTrend sweeps cut into time chunks (verified warm restarts,
    also with a warm length too short to converge so the fix-up pass repairs
    chunks) are bit-identical to the sequential per-combo kernel."""
    d = datagen.ohlcv(30000, seed=31, nan_lead=17)
    h, l, c = (f32(d[k]) for k in ("high", "low", "close"))
    seq = V.CLASSES[name](0)
    seq.set_policy("recur_chunk", "sequential")
    ref = seq.batch_dev(h, l, c, sweep=sweep)
    ref = [r.to_host() for r in (ref if isinstance(ref, tuple) else (ref,))]
    for warm in (None, "32"):
        ind = V.CLASSES[name](0)
        if warm:
            ind.set_policy("tm_warm", warm)
        got = ind.batch_dev(h, l, c, sweep=sweep)
        assert ind.last_kernel.endswith("_chunked")
        got = [g.to_host() for g in (got if isinstance(got, tuple) else (got,))]
        for k, (g, r) in enumerate(zip(got, ref)):
            assert np.array_equal(g, r, equal_nan=True), f"{name}[{k}] warm={warm}"

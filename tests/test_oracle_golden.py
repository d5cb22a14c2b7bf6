"""The CPU oracle reproduces every golden vector of the VectorTA test-suite.

The vectors (last five outputs on the crate's 4h Bitfinex fixture, default
parameters) and each test's tolerance come from tests/golden/expected.json,
generated by tests/golden/make_golden.py from the crate's own tests.
"""
import numpy as np
import pytest

from oracle import oracle as O


def _check(vals, exp, tol, what):
    vals = np.asarray(vals)[-5:]
    exp = np.asarray(exp, dtype=np.float64)
    assert np.all(np.abs(vals - exp) < tol), f"{what}: got {vals}, expected {exp} (tol {tol})"


SINGLE = {
    "alma": lambda c, p: O.alma(c["close"], **p),
    "ema": lambda c, p: O.ema(c["close"], **p),
    "dema": lambda c, p: O.dema(c["close"], **p),
    "tema": lambda c, p: O.tema(c["close"], **p),
    "wma": lambda c, p: O.wma(c["close"], **p),
    "swma": lambda c, p: O.swma(c["close"], **p),
    "pwma": lambda c, p: O.pwma(c["close"], **p),
    "sinwma": lambda c, p: O.sinwma(c["close"], **p),
    "trima": lambda c, p: O.trima(c["close"], **p),
    "sma": lambda c, p: O.sma(c["close"], **p),
    "wilders": lambda c, p: O.wilders(c["close"], **p),
    "rsi": lambda c, p: O.rsi(c["close"], **p),
    "stddev": lambda c, p: O.stddev(c["close"], **p),
    "zscore": lambda c, p: O.zscore(c["close"], **p),
    "percentile_nearest_rank": lambda c, p: O.percentile_nearest_rank(c["close"], **p),
    "atr": lambda c, p: O.atr(c["high"], c["low"], c["close"], **p),
    "adx": lambda c, p: O.adx(c["high"], c["low"], c["close"], **p),
    "willr": lambda c, p: O.willr(c["high"], c["low"], c["close"], **p),
    "cwma": lambda c, p: O.cwma(c["close"], **p),
    "fwma": lambda c, p: O.fwma(c["close"], **p),
    "srwma": lambda c, p: O.srwma(c["close"], **p),
    "sqwma": lambda c, p: O.sqwma(c["close"], **p),
    "epma": lambda c, p: O.epma(c["close"], **p),
    "vpwma": lambda c, p: O.vpwma(c["close"], **p),
}


@pytest.mark.parametrize("name", sorted(SINGLE))
def test_oracle_golden_last5(name, candles, golden):
    g = golden[name]
    _check(SINGLE[name](candles, g["params"]), g["last5"], g["tol"], name)


def test_oracle_alma_reinput(candles, golden):
    g = golden["alma_reinput"]
    first = O.alma(candles["close"], **g["params"])
    _check(O.alma(first, **g["params"]), g["last5"], g["tol"], "alma reinput")


def test_oracle_trima_reinput(candles, golden):
    g = golden["trima_reinput"]
    first = O.trima(candles["close"], **g["params"])
    second = O.trima(first, g["second_period"])[-5:]
    exp = np.array(g["last5"])
    assert np.allclose(second, exp, rtol=g["tol"], atol=0), (second, exp)


def test_oracle_supertrend(candles, golden):
    g = golden["supertrend"]
    tr, ch = O.supertrend(candles["high"], candles["low"], candles["close"], **g["params"])
    _check(tr, g["last5_trend"], g["tol"], "supertrend trend")
    _check(ch, g["last5_changed"], 1e-12, "supertrend changed")


def test_oracle_bollinger(candles, golden):
    g = golden["bollinger"]
    u, m, lo = O.bollinger(candles["close"], **g["params"])
    _check(u, g["last5_upper"], g["tol"], "bb upper")
    _check(m, g["last5_middle"], g["tol"], "bb middle")
    _check(lo, g["last5_lower"], g["tol"], "bb lower")


def test_oracle_donchian(candles, golden):
    g = golden["donchian"]
    u, m, lo = O.donchian(candles["high"], candles["low"], **g["params"])
    _check(u, g["last5_upper"], g["tol"], "donchian upper")
    _check(m, g["last5_middle"], g["tol"], "donchian middle")
    _check(lo, g["last5_lower"], g["tol"], "donchian lower")


def test_oracle_percentile_known_answers(golden):
    ka = golden["percentile_known_answers"]
    b = ka["basic"]
    out = O.percentile_nearest_rank(np.array(b["data"]), b["length"], b["percentage"])
    assert out[4] == b["expected_at_4"] and out[5] == b["expected_at_5"]
    assert np.all(np.isnan(out[:4]))
    pt = ka["percentiles"]
    d = np.array(pt["data"])
    for key, pct in (("p25_at_4", 25.0), ("p75_at_4", 75.0), ("p100_at_4", 100.0)):
        assert O.percentile_nearest_rank(d, pt["length"], pct)[4] == pt[key]


def test_oracle_pwma_formula(golden):
    g = golden["pwma_formula"]
    out = O.pwma(np.array(g["data"]), g["period"])
    exp = np.array(g["expected"], dtype=np.float64)
    assert np.array_equal(np.isnan(out), np.isnan(exp))
    assert np.allclose(out[~np.isnan(exp)], exp[~np.isnan(exp)], rtol=0, atol=1e-12)


def test_oracle_structural_known_answers():
    # WMA p=2 is (x[i-1] + 2 x[i]) / 3 (wma.rs:1211-1216)
    x = np.array([1.0, 4.0, 2.0, 8.0, 5.0])
    w = O.wma(x, 2)
    assert np.isnan(w[0])
    assert np.allclose(w[1:], (x[:-1] + 2 * x[1:]) / 3, rtol=0, atol=1e-12)
    # ALMA of a constant series is the constant (alma.rs:2295-2297)
    c = np.full(64, 42.5)
    a = O.alma(c, 9, 0.85, 6.0)
    assert np.allclose(a[8:], 42.5, rtol=0, atol=1e-9)


def test_oracle_batch_rows_match_single(candles):
    # check_batch_default_row (alma.rs:2410): a batch row equals the single path
    close = candles["close"]
    out, combos = O.alma_batch(close, (9, 12, 1), (0.85, 0.85, 0), (6.0, 6.0, 0))
    assert [c[0] for c in combos] == [9, 10, 11, 12]
    single = O.alma(close, 9, 0.85, 6.0)
    assert np.allclose(out[0], single, rtol=1e-12, atol=1e-9, equal_nan=True)
    r = O.rsi_batch(close, [14])
    assert np.allclose(r[0], O.rsi(close, 14), rtol=1e-10, atol=1e-8, equal_nan=True)
    s = O.sma_batch(close, [9])
    assert np.allclose(s[0], O.sma(close, 9), rtol=1e-10, atol=1e-6, equal_nan=True)


def test_oracle_grid_float_accumulation():
    # offset range 0.5..1.0 step 0.1 -> 6 values by accumulation (alma.rs:2464-2483)
    assert len(O.axis_f64((0.5, 1.0, 0.1))) == 6
    assert len(O.axis_f64((0.50, 0.95, 0.05))) == 10
    assert O.axis_usize((5, 260, 1)) == list(range(5, 261))


def test_oracle_error_cases():
    x = np.array([np.nan] * 5)
    with pytest.raises(O.OracleError):
        O.alma(x, 3)
    with pytest.raises(O.OracleError):
        O.alma(np.arange(10.0), 0)
    with pytest.raises(O.OracleError):
        O.alma(np.arange(10.0), 11)
    with pytest.raises(O.OracleError):
        O.alma(np.arange(10.0), 3, 0.85, 0.0)
    with pytest.raises(O.OracleError):
        O.alma(np.arange(10.0), 3, 1.5, 6.0)
    with pytest.raises(O.OracleError):
        O.ema(np.array([]), 3)


def test_oracle_fast_minmax_equals_direct_scan():
    """The crate's block-extrema / deque paths select the same values as a
    direct window scan (bit-identical), including NaN windows."""
    from vectorta_gb300 import datagen

    c = datagen.random_walk(3000, seed=5, nan_lead=7)
    h, l = datagen.high_low(c, seed=6)
    h[1500] = np.nan
    l[2200] = np.nan
    for p in (33, 50, 97, 256):
        a = O.donchian(h, l, p)
        b = O.donchian(h, l, p, fast=True)
        for x, y in zip(a, b):
            assert np.array_equal(x, y, equal_nan=True), p
        assert np.array_equal(O.willr(h, l, c, p), O.willr(h, l, c, p, fast=True), equal_nan=True), p


def test_oracle_weighted_window_warmups(candles):
    """First output index of each weighted-window MA on the fixture (the
    crate's warm-up: cwma.rs:253, fwma.rs:442, srwma.rs:214, sqwma.rs:228,
    epma.rs:247) and EPMA's documented warm-up of 16 at (11, 4)
    (tests/python/test_utils.py EXPECTED_OUTPUTS['epma'])."""
    c = candles["close"]
    first = int(np.argmax(~np.isnan(c)))
    cases = {"cwma": (O.cwma(c, 14), first + 13), "fwma": (O.fwma(c, 5), first + 4),
             "srwma": (O.srwma(c, 14), first + 15), "sqwma": (O.sqwma(c, 14), first + 15),
             "epma": (O.epma(c, 11, 4), first + 16)}
    for name, (out, warm) in cases.items():
        assert np.all(np.isnan(out[:warm])), name
        assert not np.isnan(out[warm]), name


STREAM_VS_BATCH = {
    # name: (stream params, batch call on the candles, relative tolerance)
    "ema": ({"period": 9}, lambda d: O.ema(d["close"], 9), 1e-9),
    "sma": ({"period": 9}, lambda d: O.sma(d["close"], 9), 1e-9),
    "alma": ({"period": 9}, lambda d: O.alma(d["close"], 9), 1e-9),
    "rsi": ({"period": 14}, lambda d: O.rsi(d["close"], 14), 1e-9),
    "atr": ({"length": 14}, lambda d: O.atr(d["high"], d["low"], d["close"], 14), 1e-9),
    "wilders": ({"period": 5}, lambda d: O.wilders(d["close"], 5), 1e-9),
    "dema": ({"period": 30}, lambda d: O.dema(d["close"], 30), 1e-9),
    "tema": ({"period": 9}, lambda d: O.tema(d["close"], 9), 1e-9),
    "wma": ({"period": 30}, lambda d: O.wma(d["close"], 30), 1e-9),
    "swma": ({"period": 5}, lambda d: O.swma(d["close"], 5), 1e-9),
    "pwma": ({"period": 5}, lambda d: O.pwma(d["close"], 5), 1e-9),
    "stddev": ({"period": 5}, lambda d: O.stddev(d["close"], 5, 1.0), 1e-9),
    # running sums of squares over ~15k bars: no streaming test in the crate
    "zscore": ({"period": 14}, lambda d: O.zscore(d["close"], 14, 1.0), 1e-7),
    "bollinger_bands": ({"period": 20}, lambda d: O.bollinger(d["close"], 20, 2.0, 2.0), 1e-9),
    "donchian": ({"period": 20}, lambda d: O.donchian(d["high"], d["low"], 20), 1e-9),
    "willr": ({"period": 14}, lambda d: O.willr(d["high"], d["low"], d["close"], 14), 1e-9),
    "adx": ({"period": 14}, lambda d: O.adx(d["high"], d["low"], d["close"], 14), 1e-9),
    "supertrend": ({"period": 10}, lambda d: O.supertrend(d["high"], d["low"], d["close"], 10, 3.0), 1e-9),
    "sinwma": ({"period": 14}, lambda d: O.sinwma(d["close"], 14), 1e-9),
    "trima": ({"period": 30}, lambda d: O.trima(d["close"], 30), 1e-9),
    "cwma": ({"period": 14}, lambda d: O.cwma(d["close"], 14), 1e-9),
    "fwma": ({"period": 5}, lambda d: O.fwma(d["close"], 5), 1e-9),
    "srwma": ({"period": 14}, lambda d: O.srwma(d["close"], 14), 1e-9),
    "sqwma": ({"period": 14}, lambda d: O.sqwma(d["close"], 14), 1e-9),
    "epma": ({"period": 11, "offset": 4}, lambda d: O.epma(d["close"], 11, 4), 1e-9),
    "vpwma": ({"period": 14, "power": 0.382}, lambda d: O.vpwma(d["close"], 14, 0.382), 1e-9),
    # the integer-power (moment recurrence) mode drifts more over ~15k bars
    "vpwma-int": ({"period": 14, "power": 2.0}, lambda d: O.vpwma(d["close"], 14, 2.0), 1e-8),
    "percentile_nearest_rank": ({"length": 20, "percentage": 90.0},
                                lambda d: O.percentile_nearest_rank(d["close"], 20, 90.0), 0.0),
}


@pytest.mark.parametrize("name", sorted(STREAM_VS_BATCH))
def test_oracle_streams_match_batch(name, candles):
    """The oracle's XStream restatements agree with the single-series paths
    after the warm-up, as the crate's own check_X_streaming tests require
    (e.g. ema.rs:1127-1190: skip 240 bars, |diff| < 1e-9)."""
    prm, batch, tol = STREAM_VS_BATCH[name]
    kind = name.split("-")[0]
    n_in = O.STREAMS[kind][0]
    ins = [candles["close"]] if n_in == 1 else [candles["high"], candles["low"]] + ([candles["close"]] if n_in == 3 else [])
    s, b = O.stream(kind, ins, **prm), batch(candles)
    if not isinstance(s, tuple):
        s, b = (s,), (b,)
    for k, (sk, bk) in enumerate(zip(s, b)):
        sk, bk = sk[240:], bk[240:]
        m = ~(np.isnan(sk) & np.isnan(bk))
        assert np.all(np.abs(sk[m] - bk[m]) <= tol * np.maximum(1.0, np.abs(bk[m]))), (name, k)

"""Parity at the benchmark workloads' full sizes, where the oracle cannot run
every row in seconds: each row's NaN warm-up prefix is checked for every combo
(size-independent: it depends only on the first valid index and the
parameters), and evenly spaced sampled rows are checked value by value against
the oracle at the crate's GPU-test tolerances.

* recurrence and window sweeps: 1,000,000 bars (seed 1, NaN lead 200),
  EMA / DEMA / TEMA / RSI periods 2..1000, SMA / StdDev / Z-score / Donchian /
  WillR windows 5..500 step 5;
* ALMA grid: 200,000 bars (seed 2), periods 5..260 x offsets 0.50..0.95 x
  sigmas 3..9 (17,920 combos, 14 GB of outputs).
"""
import numpy as np
import pytest

from oracle import oracle as O
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu

N_BARS, LEAD = 1_000_000, 200
# The crate's GPU-test tolerances, except DEMA / TEMA: their f32 recurrences'
# relative error grows with the period (measured on this workload: 2e-7 at
# p = 2, 1e-6 at p = 100, up to 1.2e-5 at p = 1000), past the crate's 5e-6 /
# 1e-5, which its tests apply to short periods.
TOL = {"ema": 5e-5, "dema": 2e-5, "tema": 2e-5, "rsi": 5e-4, "sma": 1e-5, "stddev": 5e-4, "zscore": 5e-4,
       "donchian": 5e-4, "willr": 5e-5, "alma": 1e-5}


def assert_close(gpu, cpu, tol, what):
    gpu, cpu = np.asarray(gpu, np.float64), np.asarray(cpu, np.float64)
    assert np.array_equal(np.isnan(gpu), np.isnan(cpu)), what
    m = ~np.isnan(cpu)
    d = np.abs(gpu[m] - cpu[m])
    lim = tol + tol * np.maximum(np.abs(gpu[m]), np.abs(cpu[m]))
    assert np.all(d <= lim), (what, float(np.max(d - lim)))


@pytest.fixture(scope="module")
def sweep_data():
    close = datagen.random_walk(N_BARS, seed=1, nan_lead=LEAD)
    hi, lo = datagen.high_low(close, seed=1)
    hi[:LEAD] = np.nan
    lo[:LEAD] = np.nan
    return {"close": close.astype(np.float32), "high": hi.astype(np.float32), "low": lo.astype(np.float32)}


# first non-NaN output index of each row, from the crate's warm-up rules
WARM = {
    "ema": lambda f, p: f, "dema": lambda f, p: f + p - 1, "tema": lambda f, p: f + 3 * (p - 1),
    "rsi": lambda f, p: f + p, "sma": lambda f, p: f + p - 1, "stddev": lambda f, p: f + p - 1,
    "zscore": lambda f, p: f + p - 1, "donchian": lambda f, p: f + p - 1, "willr": lambda f, p: f + p - 1,
}
REC = {"period": (2, 1000, 1)}
WIN = {"period": (5, 500, 5)}
SWEEPS = {
    "ema": REC, "dema": REC, "tema": REC, "rsi": REC, "sma": WIN,
    "stddev": {"period": (5, 500, 5), "nbdev": (1.0, 1.0, 0.0)},
    "zscore": {"period": (5, 500, 5), "nbdev": (1.0, 1.0, 0.0)}, "donchian": WIN, "willr": WIN,
}


def oracle_row(name, d, p):
    c = d["close"].astype(np.float64)
    h, l = d["high"].astype(np.float64), d["low"].astype(np.float64)
    if name == "rsi":
        return O.rsi_batch(c, [p])[0]
    if name == "stddev":
        return O.stddev(c, p, 1.0)
    if name == "zscore":
        return O.zscore_batch_row(c, p, 1.0)
    if name == "donchian":
        return O.donchian(h, l, p)[0]
    if name == "willr":
        return O.willr(h, l, c, p)
    return {"ema": O.ema, "dema": O.dema, "tema": O.tema, "sma": O.sma}[name](c, p)


@pytest.mark.parametrize("name", sorted(SWEEPS))
def test_sweep_full_size(name, sweep_data):
    ind = V.CLASSES[name](0)
    ins = {"x": ["close"], "hl": ["high", "low"], "hlc": ["high", "low", "close"]}[V.N.INDICATORS[name][0]]
    out = ind.batch_dev(*[sweep_data[k] for k in ins], sweep=SWEEPS[name])
    got = (out[0] if isinstance(out, tuple) else out).to_host()  # Donchian: the upper band
    periods = O.periods_of(name, SWEEPS[name]["period"])
    assert got.shape == (len(periods), N_BARS)
    # every row: NaN exactly before its warm-up end
    finite = ~np.isnan(got)
    first = np.where(finite.any(axis=1), finite.argmax(axis=1), N_BARS)
    exp_first = np.array([min(WARM[name](LEAD, p), N_BARS) for p in periods])
    assert np.array_equal(first, exp_first), (name, np.flatnonzero(first != exp_first)[:5])
    # sampled rows against the oracle
    keep = np.ones(N_BARS, dtype=bool)
    if name in ("stddev", "zscore"):
        # The crate's StdDev / Z-score keep f64 running sums of x and x^2 over
        # the whole series; where the series has fallen far below its earlier
        # levels their drift (~sqrt(t) ulp of the largest sum) swamps the
        # variance, so the oracle is compared only where x(t) >= 1% of its
        # running maximum (69% of this series).  The GPU path differences
        # block-local prefixes and has no such drift.
        c = sweep_data["close"].astype(np.float64)
        keep = np.nan_to_num(c) >= 0.01 * np.fmax.accumulate(np.nan_to_num(c))
    for r in np.linspace(0, len(periods) - 1, 6).round().astype(int):
        exp = oracle_row(name, sweep_data, periods[r])
        # (Z-score is NaN where its deviation is 0, which the drifting sums
        # also decide: the NaN mask is compared on the same positions)
        assert_close(got[r][keep], exp[keep], TOL[name], f"{name} p={periods[r]}")


def test_alma_grid_full_size():
    x = datagen.random_walk(200_000, seed=2).astype(np.float32)
    sweep = {"period": (5, 260, 1), "offset": (0.50, 0.95, 0.05), "sigma": (3.0, 9.0, 1.0)}
    ind = V.CudaAlma(0)
    got = ind.alma_batch_dev(x, sweep=sweep).to_host()
    periods = list(range(5, 261))
    offsets = O.axis_f64(sweep["offset"])
    sigmas = O.axis_f64(sweep["sigma"])
    assert got.shape == (len(periods) * len(offsets) * len(sigmas), x.size) == (17920, 200_000)
    # combo order: period-major, then offset, then sigma; NaN prefix p - 1
    first = np.isnan(got).argmin(axis=1)
    exp_first = np.repeat(np.array(periods) - 1, len(offsets) * len(sigmas))
    assert np.array_equal(first, exp_first)
    xd = x.astype(np.float64)
    for r in np.linspace(0, got.shape[0] - 1, 12).round().astype(int):
        p = periods[r // (len(offsets) * len(sigmas))]
        o = offsets[(r // len(sigmas)) % len(offsets)]
        s = sigmas[r % len(sigmas)]
        exp = O.alma_batch(xd, (p, p, 0), (o, o, 0.0), (s, s, 0.0))[0][0]  # the batch rows' weights
        m = ~np.isnan(exp)
        assert np.array_equal(np.isnan(got[r]), ~m)
        rel = np.max(np.abs(got[r][m] - exp[m]) / np.abs(exp[m]))
        assert rel <= TOL["alma"], (p, o, s, rel)

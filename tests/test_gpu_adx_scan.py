"""Batch ADX sweeps with long periods: the 32-combo groups whose warm-restart
run would exceed 4,096 steps take the exact chunked scan (two Wilder levels
composed across chunks), the others the verified warm restart.  Both against
the sequential per-combo kernel and the oracle, also with NaN bars (the
crate's NaN-skipping max makes them change values, not poison rows: every
path must agree)."""
import numpy as np
import pytest

from oracle import oracle as O
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu


def hlc(n, seed, gap=None):
    d = datagen.ohlcv(n, seed=seed, nan_lead=17)
    h, l, c = (np.asarray(d[k], np.float32) for k in ("high", "low", "close"))
    if gap is not None:
        c[gap] = np.nan
        h[gap + 7] = np.nan
        l[gap + 300] = np.nan
    return h, l, c


def run(h, l, c, sweep, policy=None):
    ind = V.CLASSES["adx"](0)
    if policy:
        ind.set_policy(*policy)
    out = ind.batch_dev(h, l, c, sweep=sweep).to_host()
    return out, ind.last_kernel


def close(g, e, rtol, atol, what):
    g, e = np.asarray(g, np.float64), np.asarray(e, np.float64)
    assert np.array_equal(np.isnan(g), np.isnan(e)), what
    m = ~np.isnan(e)
    d = np.abs(g[m] - e[m])
    assert np.all(d <= atol + rtol * np.abs(e[m])), (what, float(d.max()))


@pytest.mark.parametrize("sweep", [{"period": (150, 400, 10)}, {"period": (2, 400, 3)}])
def test_scan_equals_sequential_and_oracle(sweep):
    h, l, c = hlc(60_000, 81)
    got, kern = run(h, l, c, sweep)
    assert "exact scan" in kern, kern
    seq, _ = run(h, l, c, sweep, ("recur_chunk", "sequential"))
    # ADX lies in [0, 100]: the composed carries round differently from one
    # f32 pass, by a few 1e-7 of the Wilder sums
    close(got, seq, 1e-5, 1e-4, "scan vs sequential")
    periods = list(range(sweep["period"][0], sweep["period"][1] + 1, sweep["period"][2]))
    h64, l64, c64 = (a.astype(np.float64) for a in (h, l, c))
    for i in (0, len(periods) // 2, len(periods) - 1):
        exp = O.adx(h64, l64, c64, periods[i])
        close(got[i], exp, 0.0, 1e-1, f"scan vs oracle p={periods[i]}")  # the crate's GPU tolerance


def test_scan_with_nan_gap():
    h, l, c = hlc(50_000, 83, gap=31_000)
    sweep = {"period": (200, 420, 20)}
    got, kern = run(h, l, c, sweep)
    assert "exact scan" in kern, kern
    seq, _ = run(h, l, c, sweep, ("recur_chunk", "sequential"))
    close(got, seq, 1e-5, 1e-4, "scan vs sequential with NaN bars")


@pytest.mark.parametrize("chunk", ["1024", "3008"])
def test_scan_chunk_lengths(chunk):
    # the chunk length changes only how the carries compose
    h, l, c = hlc(70_000, 87)
    sweep = {"period": (180, 300, 4)}
    got, kern = run(h, l, c, sweep, ("scan_chunk", chunk))
    assert f"L={chunk}" in kern, kern
    seq, _ = run(h, l, c, sweep, ("recur_chunk", "sequential"))
    close(got, seq, 1e-5, 1e-4, f"scan L={chunk} vs sequential")


def test_scan_chunk_policy_rejects_bad_lengths():
    ind = V.CLASSES["adx"](0)
    for bad in ("1000", "512", "x"):
        with pytest.raises(Exception):
            ind.set_policy("scan_chunk", bad)


def test_short_periods_stay_bit_identical():
    # every group below the threshold: the warm-restart path alone
    h, l, c = hlc(40_000, 85)
    sweep = {"period": (5, 100, 5)}
    got, kern = run(h, l, c, sweep)
    assert kern == "adx_chunked", kern
    seq, _ = run(h, l, c, sweep, ("recur_chunk", "sequential"))
    assert np.array_equal(got, seq, equal_nan=True)

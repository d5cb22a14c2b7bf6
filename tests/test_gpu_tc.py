"""The tcgen05 split-precision contraction of the weighted-window MAs.

North-star accuracy bar: on the ALMA grid the result is within 1e-5 relative
error of the FP64 oracle with the NaN warm-up positions exact.  Runs a
reduced ALMA grid (same period / offset / sigma axes as the 17,920-combo
workload, fewer bars) plus the other weighted-window indicators, through the
C ABI with the tensor-core policy forced.
"""
import numpy as np
import pytest

from oracle import oracle as O
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu

GRID = {"period": (5, 260, 1), "offset": (0.50, 0.95, 0.05), "sigma": (3.0, 9.0, 1.0)}


def max_rel(g, e):
    m = ~np.isnan(e)
    return float(np.max(np.abs(g[m].astype(np.float64) - e[m]) / np.abs(e[m])))


@pytest.fixture(scope="module")
def series():
    return datagen.random_walk(3000, seed=2).astype(np.float32)


@pytest.mark.parametrize("variant,bound", [("tc_fp16x3", 1e-5), ("tc_bf16x3", 1e-4)])
def test_alma_grid_relative_error(series, variant, bound):
    ind = V.CudaAlma(0)
    ind.set_policy("wma_batch", variant)
    sweep = {"period": (5, 260, 9), "offset": GRID["offset"], "sigma": GRID["sigma"]}
    got = ind.alma_batch_dev(series, sweep=sweep).to_host()
    assert ind.last_kernel == f"wwma_{variant}"
    exp, combos = O.alma_batch(series.astype(np.float64), sweep["period"], sweep["offset"], sweep["sigma"])
    assert got.shape == exp.shape == (len(combos), series.size)
    assert np.array_equal(np.isnan(got), np.isnan(exp))
    err = max_rel(got, exp)
    assert err <= bound, f"{variant}: max relative error {err:.3g}"


def test_tc_matches_plain_kernel(series):
    sweep = {"period": (5, 260, 17), "offset": (0.85, 0.85, 0.0), "sigma": (6.0, 6.0, 0.0)}
    a = V.CudaAlma(0)
    a.set_policy("wma_batch", "tc_fp16x3")
    b = V.CudaAlma(0)
    b.set_policy("wma_batch", "plain")
    ga = a.alma_batch_dev(series, sweep=sweep).to_host()
    gb = b.alma_batch_dev(series, sweep=sweep).to_host()
    assert np.array_equal(np.isnan(ga), np.isnan(gb))
    m = ~np.isnan(ga)
    assert np.max(np.abs(ga[m] - gb[m]) / np.abs(gb[m])) < 2e-6


@pytest.mark.parametrize("name,fn,rng", [
    ("wma", O.wma, (2, 200, 7)), ("swma", O.swma, (1, 200, 7)), ("sinwma", O.sinwma, (1, 200, 7)),
    ("trima", O.trima, (4, 200, 7)), ("pwma", lambda x, p: O.pwma(x, p, True), (1, 60, 3)),
])
def test_other_weighted_mas_on_tensor_cores(series, name, fn, rng):
    ind = V.CLASSES[name](0)
    ind.set_policy("wma_batch", "tc_fp16x3")
    got = ind.batch_dev(series, sweep={"period": rng}).to_host()
    ps = O.periods_of(name, rng)
    exp = np.stack([fn(series.astype(np.float64), p) for p in ps])
    assert np.array_equal(np.isnan(got), np.isnan(exp))
    assert max_rel(got, exp) <= 1e-5


def test_tc_ragged_tail_and_nan(series):
    """Length not a multiple of the tile, a NaN lead and an interior NaN."""
    x = series[:2999].copy()
    x[:11] = np.nan
    x[1500] = np.nan
    sweep = {"period": (5, 150, 13), "offset": (0.85, 0.85, 0.0), "sigma": (6.0, 6.0, 0.0)}
    ind = V.CudaAlma(0)
    ind.set_policy("wma_batch", "tc_fp16x3")
    got = ind.alma_batch_dev(x, sweep=sweep).to_host()
    exp, _ = O.alma_batch(x.astype(np.float64), sweep["period"], sweep["offset"], sweep["sigma"])
    assert np.array_equal(np.isnan(got), np.isnan(exp))
    assert max_rel(got, exp) <= 1e-5


@pytest.fixture(scope="module")
def long_series():
    return datagen.random_walk(100_000, seed=9, nan_lead=37).astype(np.float32)


@pytest.mark.parametrize("variant,bound", [("auto", 1e-5), ("tc_bf16x3", 1e-4)])
def test_long_windows_stay_on_tensor_cores(long_series, variant, bound):
    """Windows longer than one shared-memory A tile (K > 272) run as K slices
    accumulating in the same TMEM accumulator; the sweep mixes whole-tile and
    sliced combo tiles.  WMA periods 2..1000 on 100,000 bars against the
    oracle on every 7th row, every bar."""
    ind = V.CudaWma(0)
    ind.set_policy("wma_batch", variant)
    rng = (2, 1000, 1)
    got = ind.batch_dev(long_series, sweep={"period": rng}).to_host()
    assert ind.last_kernel == ("wwma_tc_fp16x3" if variant == "auto" else f"wwma_{variant}")
    ps = O.periods_of("wma", rng)
    xd = long_series.astype(np.float64)
    for r in range(0, len(ps), 7):
        exp = O.wma(xd, ps[r])
        assert np.array_equal(np.isnan(got[r]), np.isnan(exp)), ps[r]
        assert max_rel(got[r], exp) <= bound, (ps[r], max_rel(got[r], exp))


def test_long_alma_windows_every_row_sampled(long_series):
    """ALMA periods 200..600 (401 combos, tiles of K up to 608) on 100,000
    bars: every row against the oracle on a time sample (every 499th bar and
    the first 2p bars after the warm-up)."""
    ind = V.CudaAlma(0)
    sweep = {"period": (200, 600, 1), "offset": (0.85, 0.85, 0.0), "sigma": (6.0, 6.0, 0.0)}
    got = ind.alma_batch_dev(long_series, sweep=sweep).to_host()
    assert ind.last_kernel == "wwma_tc_fp16x3"
    xd = long_series.astype(np.float64)
    first = int(np.argmax(~np.isnan(xd)))
    for r, p in enumerate(range(200, 601)):
        warm = first + p - 1
        assert np.isnan(got[r][:warm]).all() and not np.isnan(got[r][warm:]).any(), p
        idx = np.union1d(np.arange(warm, xd.size, 499), np.arange(warm, min(xd.size, warm + 2 * p)))
        exp = O.alma_batch_row_at(xd, p, 0.85, 6.0, idx)
        assert max_rel(got[r][idx], exp) <= 1e-5, (p, max_rel(got[r][idx], exp))


def test_sliced_tiles_with_nan_and_ragged_tail(series):
    x = series[:2999].copy()
    x[:11] = np.nan
    x[1500] = np.nan
    sweep = {"period": (300, 420, 40), "offset": (0.85, 0.85, 0.0), "sigma": (6.0, 6.0, 0.0)}
    ind = V.CudaAlma(0)
    got = ind.alma_batch_dev(x, sweep=sweep).to_host()
    assert ind.last_kernel == "wwma_tc_fp16x3"
    exp, _ = O.alma_batch(x.astype(np.float64), sweep["period"], sweep["offset"], sweep["sigma"])
    assert np.array_equal(np.isnan(got), np.isnan(exp))
    assert max_rel(got, exp) <= 1e-5

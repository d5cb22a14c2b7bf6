"""Chunk aggregates of the EMA / DEMA / TEMA / RSI batch sweeps on the tensor
cores (split-precision tcgen05 contraction) against the oracle and against
the CUDA-core aggregate pass: chunk lengths of one and several K slices, lane
counts that are not multiples of the 128-row tile, interior NaN gaps (those
chunks stay on the CUDA-core pass), a series far from zero (the per-chunk
centring) and a long sweep at the bench's shape."""
import numpy as np
import pytest

from oracle import oracle as O
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu

# same bands as the chunked-scan tests: the aggregates feed f64 carries and
# the emit pass starts every chunk from its exact carry-in state
TOL = {"ema": 5e-5, "dema": 5e-6, "tema": 1e-5, "rsi": 5e-4}


def assert_close(gpu, cpu, tol, what):
    gpu, cpu = np.asarray(gpu, np.float64), np.asarray(cpu, np.float64)
    assert np.array_equal(np.isnan(gpu), np.isnan(cpu)), what
    m = ~np.isnan(cpu)
    lim = tol + tol * np.maximum(np.abs(gpu[m]), np.abs(cpu[m]))
    d = np.abs(gpu[m] - cpu[m])
    assert np.all(d <= lim), (what, float(np.max(d - lim)))


def oracle_rows(name, c, periods):
    if name == "rsi":
        return O.rsi_batch(c, periods)
    fn = {"ema": O.ema, "dema": O.dema, "tema": O.tema}[name]
    return np.stack([fn(c, p) for p in periods])


def close_series(n, seed, gaps, offset=0.0):
    c = datagen.random_walk(n, seed=seed, nan_lead=23).astype(np.float64) + offset
    if gaps:
        for g in (5000, 17003, 29999):
            c[g:g + 3] = np.nan
    return c.astype(np.float32)


def run(name, c, sweep, agg, chunk=None):
    ind = V.CLASSES[name](0)
    ind.set_policy("recur_agg", agg)
    if chunk:
        ind.set_policy("recur_chunk", chunk)
    out = ind.batch_dev(c, sweep=sweep).to_host()
    return out, ind.last_kernel


@pytest.mark.parametrize("name", ["ema", "dema", "tema", "rsi"])
@pytest.mark.parametrize("gaps,chunk", [(False, None), (True, None), (False, "64"), (False, "416")])
def test_tc_aggregates_match_oracle_and_cuda_cores(name, gaps, chunk):
    c = close_series(40000, 43, gaps)
    sweep = {"period": (2, 520, 3)}  # 173 combos: two 128-row tiles, ragged
    tc, kern = run(name, c, sweep, "tc", chunk)
    assert "tc aggregates" in kern, kern
    cu, kern_cu = run(name, c, sweep, "cuda", chunk)
    assert "tc aggregates" not in kern_cu, kern_cu
    periods = list(range(2, 521, 3))
    exp = oracle_rows(name, c.astype(np.float64), periods)
    assert_close(tc, exp, TOL[name], f"{name} tc vs oracle")
    assert_close(tc, cu, TOL[name], f"{name} tc vs cuda cores")


@pytest.mark.parametrize("name", ["ema", "tema", "rsi"])
def test_tc_aggregates_far_from_zero(name):
    # prices near 1e4 with small moves: each chunk is centred on its first
    # value before the split, so the contraction sees only the moves
    c = close_series(30000, 47, False, offset=1.0e4)
    sweep = {"period": (5, 300, 5)}
    tc, kern = run(name, c, sweep, "tc", "256")
    assert "tc aggregates" in kern, kern
    periods = list(range(5, 301, 5))
    exp = oracle_rows(name, c.astype(np.float64), periods)
    assert_close(tc, exp, TOL[name], f"{name} tc vs oracle (offset series)")


def test_tc_aggregates_constant_stretch():
    # a flat stretch gives chunks whose centred inputs are all zero
    c = close_series(20000, 53, False)
    c[6000:12000] = c[6000]
    sweep = {"period": (2, 200, 9)}
    periods = list(range(2, 201, 9))
    for name in ("ema", "dema"):
        tc, kern = run(name, c, sweep, "tc", "128")
        assert "tc aggregates" in kern, kern
        exp = oracle_rows(name, c.astype(np.float64), periods)
        assert_close(tc, exp, TOL[name], f"{name} tc vs oracle (flat stretch)")
    # RSI: over a flat stretch the Wilder averages of gains and losses decay
    # by (1 - 1/p) per bar and reach the f32 subnormal range within a few
    # thousand bars, where their ratio is ill-conditioned for any f32
    # implementation (the oracle runs in f64).  Both aggregate routes give a
    # flat chunk the exact zero record, so they must agree.
    tc, kern = run("rsi", c, sweep, "tc", "128")
    assert "tc aggregates" in kern, kern
    cu, _ = run("rsi", c, sweep, "cuda", "128")
    assert_close(tc, cu, TOL["rsi"], "rsi tc vs cuda cores (flat stretch)")


@pytest.mark.parametrize("name", ["ema", "dema", "tema", "rsi"])
def test_tc_aggregates_long_sweep(name):
    # the bench's shape, thinned: 1M bars, periods 2..1000 step 37 (28 combos),
    # automatic chunking; every row against the CUDA-core pass, three rows
    # against the oracle
    c = close_series(1_000_000, 59, False)
    sweep = {"period": (2, 1000, 37)}
    tc, kern = run(name, c, sweep, "auto")
    assert "tc aggregates" in kern, kern
    cu, _ = run(name, c, sweep, "cuda")
    assert_close(tc, cu, TOL[name], f"{name} tc vs cuda cores (1M)")
    periods = list(range(2, 1001, 37))
    for i in (0, len(periods) // 2, len(periods) - 1):
        exp = oracle_rows(name, c.astype(np.float64), [periods[i]])[0]
        assert_close(tc[i], exp, TOL[name], f"{name} tc vs oracle row {periods[i]}")


def test_tc_required_on_an_ineligible_sweep_is_an_error():
    c = close_series(5000, 61, False)
    ind = V.CLASSES["wilders"](0)
    ind.set_policy("recur_agg", "tc")
    with pytest.raises(V.VtaError):
        ind.batch_dev(c, sweep={"period": (2, 50, 1)})

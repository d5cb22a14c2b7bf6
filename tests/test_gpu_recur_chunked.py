"""Chunked batch recurrences (aggregate, carry scan, emit) and the
sequential per-combo kernel against the oracle, across many time chunks and
several lane blocks, with interior NaN gaps (chunks whose aggregate skips
steps) and with chunks short enough for long carry chains."""
import numpy as np
import pytest

from oracle import oracle as O
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu

TOL = {"ema": 5e-5, "dema": 5e-6, "tema": 1e-5, "rsi": 5e-4, "wilders": 1e-5, "atr": 1e-4}


def assert_close(gpu, cpu, tol, what):
    gpu, cpu = np.asarray(gpu, np.float64), np.asarray(cpu, np.float64)
    assert np.array_equal(np.isnan(gpu), np.isnan(cpu)), what
    m = ~np.isnan(cpu)
    lim = tol + tol * np.maximum(np.abs(gpu[m]), np.abs(cpu[m]))
    d = np.abs(gpu[m] - cpu[m])
    assert np.all(d <= lim), (what, float(np.max(d - lim)))


def series(n, seed, gaps):
    close = datagen.random_walk(n, seed=seed, nan_lead=23)
    if gaps:
        for g in (5000, 17003, 29999):
            close[g:g + 3] = np.nan
    hi, lo = datagen.high_low(close, seed=seed + 1)
    hi[:23] = np.nan
    lo[:23] = np.nan
    return [a.astype(np.float32) for a in (hi, lo, close)]


def oracle_rows(name, h, l, c, periods):
    if name == "atr":
        return np.stack([O.atr(h, l, c, p) for p in periods])
    if name == "rsi":
        return O.rsi_batch(c, periods)  # batch-row NaN semantics
    if name == "wilders":
        return O.wilders_batch(c, periods)
    fn = {"ema": O.ema, "dema": O.dema, "tema": O.tema}[name]
    return np.stack([fn(c, p) for p in periods])


@pytest.mark.parametrize("name,gaps,chunk", [
    ("ema", False, None), ("ema", True, None), ("ema", False, "64"),
    ("dema", False, None), ("tema", False, None), ("tema", False, "64"),
    ("rsi", False, None), ("wilders", True, None), ("wilders", False, "64"), ("atr", False, None),
])
def test_chunked_equals_sequential_and_oracle(name, gaps, chunk):
    h, l, c = series(40000, 41, gaps)
    sweep = {"period": (2, 520, 3)}  # 173 combos: two lane blocks
    ins = [h, l, c] if name == "atr" else [c]
    out = {}
    for mode in ("chunked", "sequential"):
        ind = V.CLASSES[name](0)
        ind.set_policy("recur_chunk", chunk if mode == "chunked" and chunk else
                       ("sequential" if mode == "sequential" else "auto"))
        out[mode] = ind.batch_dev(*ins, sweep=sweep).to_host()
        assert ind.last_kernel.startswith(f"recurrence_{mode}")
    periods = list(range(2, 521, 3))
    exp = oracle_rows(name, h.astype(np.float64), l.astype(np.float64), c.astype(np.float64), periods)
    assert_close(out["chunked"], exp, TOL[name], f"{name} chunked vs oracle")
    # one f32 recurrence over the whole 40k-bar series drifts a little more
    # than the chunked scan, whose carries are composed in f64
    assert_close(out["sequential"], exp, max(TOL[name], 2e-5), f"{name} sequential vs oracle")

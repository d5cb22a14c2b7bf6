"""Error statistics of device outputs against the oracle.

TEST INFRASTRUCTURE ONLY: used by tests/ and by the CPU-baseline leg of
bench.py as the checker, never by the product package.

The figures follow one convention everywhere:
  * ``abs``  = max |gpu - ref| over the compared cells;
  * ``rel``  = max |gpu - ref| / max(|ref|, floor), where ``floor`` is 0 for
    indicators on the price scale (moving averages, bands, channels, StdDev)
    and 1 for the oscillators whose values cross or touch zero (RSI in
    0..100, Williams %R in -100..0, Z-score around 0); a cell whose reference
    is exactly 0 under floor 0 counts in ``abs`` only;
  * NaN cells must coincide exactly and are not part of either figure.
The reference ``ref`` is the oracle's restatement of the crate's scalar f64
path.  StdDev and Z-score additionally report against the exact window
statistics (``oracle.window_exact``), because the crate's running f64 sums
drift on long series whose level falls far below its earlier maximum.
"""
from __future__ import annotations

import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import oracle as O

REL_FLOOR = {"rsi": 1.0, "willr": 1.0, "zscore": 1.0}


def rel_floor(name: str) -> float:
    return REL_FLOOR.get(name, 0.0)


def oracle_row(name: str, s: dict, combo) -> np.ndarray:
    """The crate's scalar f64 row of one combo.  `s` maps close/high/low to
    f64 arrays; `combo` is (period, a, b) as the library's expand_grid gives
    (a = nbdev for StdDev / Z-score, offset for ALMA; b = sigma)."""
    p = int(combo[0])
    c, h, l = s.get("close"), s.get("high"), s.get("low")
    if name == "ema":
        return O.ema(c, p)
    if name == "dema":
        return O.dema(c, p)
    if name == "tema":
        return O.tema(c, p)
    if name == "rsi":
        return O.rsi_batch(c, [p])[0]
    if name == "sma":
        return O.sma(c, p)
    if name == "stddev":
        return O.stddev(c, p, float(combo[1]))
    if name == "zscore":
        return O.zscore_batch_row(c, p, float(combo[1]))
    if name == "donchian":  # upper, middle and lower bands, one after another
        return np.concatenate(O.donchian(h, l, p, fast=True))
    if name == "willr":
        return O.willr(h, l, c, p, fast=True)
    if name == "alma":
        return O.alma_batch(c, (p, p, 0), (combo[1], combo[1], 0.0), (combo[2], combo[2], 0.0))[0][0]
    if name == "wma":
        return O.wma(c, p)
    raise KeyError(name)


def cell_err(got, ref, floor: float):
    """(abs, rel, cells, nan_mismatch) of two equally shaped arrays."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    gn, rn = np.isnan(got), np.isnan(ref)
    mism = int(np.count_nonzero(gn != rn))
    m = ~(gn | rn)
    if not m.any():
        return 0.0, 0.0, 0, mism
    d = np.abs(got[m] - ref[m])
    den = np.maximum(np.abs(ref[m]), floor)
    ok = den > 0
    rel = float(np.max(d[ok] / den[ok])) if ok.any() else 0.0
    return float(d.max()), rel, int(m.sum()), mism


def exact_window(name: str, c: np.ndarray, combo, idx: np.ndarray) -> np.ndarray:
    """Exact StdDev / Z-score at the end indices `idx` (windows all finite)."""
    p, k = int(combo[0]), float(combo[1])
    mean, sd = O.window_exact(c, p, idx)
    if name == "stddev":
        return sd * k
    with np.errstate(divide="ignore", invalid="ignore"):
        z = (c[idx] - mean) / (sd * k)
    z[sd * k == 0.0] = np.nan
    return z


class Acc:
    """Running maxima of the error figures over many rows."""

    def __init__(self, floor: float):
        self.floor = floor
        self.abs = 0.0
        self.rel = 0.0
        self.cells = 0
        self.rows = 0
        self.nan_mismatch = 0

    def add(self, got, ref):
        a, r, n, mm = cell_err(got, ref, self.floor)
        self.abs = max(self.abs, a)
        self.rel = max(self.rel, r)
        self.cells += n
        self.rows += 1
        self.nan_mismatch += mm
        return a, r

    def as_dict(self):
        return {"abs": self.abs, "rel": self.rel, "rel_floor": self.floor, "rows": self.rows,
                "cells": self.cells, "nan_mismatch": self.nan_mismatch}


def sweep_err(name: str, series32: dict, combos, fetch_row, rows, threads: int | None = None) -> dict:
    """Error of the device rows `rows` (each fetched by fetch_row(r) as a host
    f32 array over every bar; Donchian: its three bands concatenated in the
    order upper, middle, lower) against the oracle rows of the same combos.
    StdDev / Z-score also report the device and the crate against the exact
    window statistics on every 97th bar."""
    s = {k: v.astype(np.float64) for k, v in series32.items()}
    floor = rel_floor(name)
    acc = Acc(floor)
    ex_dev, ex_crate = Acc(floor), Acc(floor)
    drift = name in ("stddev", "zscore")

    def one(r):
        got = fetch_row(r)
        ref = oracle_row(name, s, combos[r])
        out = [(got, ref)]
        if drift:
            first = int(np.argmax(~np.isnan(s["close"])))
            idx = np.arange(first + int(combos[r][0]) - 1, got.size, 97)
            ex = exact_window(name, s["close"], combos[r], idx)
            out.append((got[idx], ex, ref[idx]))
        return out

    with ThreadPoolExecutor(threads or os.cpu_count() or 1) as ex:
        for res in ex.map(one, rows):
            acc.add(*res[0])
            if drift:
                g, e, c = res[1]
                ex_dev.add(g, e)
                ex_crate.add(c, e)
    d = acc.as_dict()
    d["vs"] = "crate scalar f64 path (oracle), every bar of the sampled rows"
    if drift:
        d["vs_exact"] = dict(ex_dev.as_dict(), vs="exact window statistics, every 97th bar")
        d["crate_vs_exact"] = dict(ex_crate.as_dict(), vs="the crate's own f64 running sums against the exact "
                                                          "window statistics (their drift)")
    return d

"""The error bookkeeping of oracle/parity.py (used by the full-size tests and
by bench.py's error report), checked on the CPU with planted differences."""
import numpy as np

from oracle import oracle as O
from oracle import parity as P
from vectorta_gb300 import datagen


def test_cell_err_definitions():
    got = np.array([np.nan, 1.0, 2.5, 0.0, -3.0])
    ref = np.array([np.nan, 1.0, 2.0, 0.0, -2.0])
    a, r, n, mm = P.cell_err(got, ref, 0.0)
    assert (a, n, mm) == (1.0, 4, 0)
    assert r == 0.5  # |-3 - -2| / 2; the reference 0 cell counts in abs only
    a, r, n, mm = P.cell_err(np.array([0.5, np.nan]), np.array([0.25, 1.0]), 1.0)
    assert (a, r, mm) == (0.25, 0.25, 1)  # floor 1: |d| / max(|ref|, 1)


def test_sweep_err_on_oracle_rows():
    c = datagen.random_walk(5000, seed=3, nan_lead=7).astype(np.float32)
    s = {"close": c}
    combos = [(p, 1.0) for p in (5, 20, 60)]
    rows_f64 = [P.oracle_row("stddev", {"close": c.astype(np.float64)}, cb) for cb in combos]

    def fetch(r):
        g = rows_f64[r].astype(np.float32)
        if r == 1:
            g[500] *= 1.001  # planted: a 1e-3 relative error in row 1
        return g

    d = P.sweep_err("stddev", s, combos, fetch, [0, 1, 2])
    assert d["rows"] == 3 and d["nan_mismatch"] == 0
    assert 9e-4 < d["rel"] < 1.1e-3
    assert d["vs_exact"]["rows"] == 3 and d["crate_vs_exact"]["rel"] < 1e-9


def test_window_exact_and_batch_prefix_on_a_plain_series():
    x = datagen.random_walk(3000, seed=4).astype(np.float64)
    idx = np.arange(49, 3000, 13)
    mean, sd = O.window_exact(x, 50, idx)
    exp = np.array([x[i - 49:i + 1].std() for i in idx])
    assert np.allclose(sd, exp, rtol=1e-12, atol=0)
    assert np.allclose(mean, [x[i - 49:i + 1].mean() for i in idx], rtol=1e-14)
    # the crate's batch prefix row and its scalar running-sum row agree on a
    # series that stays near its level
    assert np.allclose(O.stddev_batch_prefix(x, 50), O.stddev(x, 50), rtol=1e-8, equal_nan=True)


def test_alma_row_at_matches_the_batch_row():
    x = datagen.random_walk(2000, seed=5, nan_lead=3)
    full = O.alma_batch(x, (33, 33, 0), (0.6, 0.6, 0.0), (4.0, 4.0, 0.0))[0][0]
    idx = np.array([0, 34, 35, 36, 1999])
    assert np.array_equal(O.alma_batch_row_at(x, 33, 0.6, 4.0, idx), full[idx], equal_nan=True)

"""Sliding min/max sweeps (Donchian, WillR) whose periods form an ascending
arithmetic progression: the progression kernel (clean tiles) together with
the sparse-table kernel (tiles holding a NaN or infinite bar) against the
oracle, for steps of 1 and more, first periods that are and are not multiples
of the step, and series with interior NaN gaps; plus the tuner's sparse-table
choices on the same sweep."""
import numpy as np
import pytest

from oracle import oracle as O
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu


def hlc(n, seed, gaps):
    c = datagen.random_walk(n, seed=seed, nan_lead=17)
    h, l = datagen.high_low(c, seed=seed + 1)
    h[:17] = np.nan
    l[:17] = np.nan
    if gaps:
        for g in (9000, 23011):
            h[g] = np.nan
            l[g + 5] = np.nan
            c[g + 40] = np.nan
    return [a.astype(np.float32) for a in (h, l, c)]


def expect(name, h, l, c, periods):
    h64, l64, c64 = (a.astype(np.float64) for a in (h, l, c))
    if name == "willr":
        return [np.stack([O.willr(h64, l64, c64, p, fast=True) for p in periods])]
    rows = [O.donchian(h64, l64, p, fast=True) for p in periods]
    return [np.stack([r[k] for r in rows]) for k in range(3)]


def close(g, e, tol, what):
    g, e = np.asarray(g, np.float64), np.asarray(e, np.float64)
    assert np.array_equal(np.isnan(g), np.isnan(e)), what
    m = ~np.isnan(e)
    assert np.all(np.abs(g[m] - e[m]) <= tol * (1.0 + np.abs(e[m]))), (what, float(np.max(np.abs(g[m] - e[m]))))


@pytest.mark.parametrize("name", ["willr", "donchian"])
@pytest.mark.parametrize("rng,gaps", [((5, 300, 5), False), ((7, 307, 5), True), ((2, 90, 1), True),
                                      ((16, 400, 32), False)])
def test_progression_sweep_matches_oracle(name, rng, gaps):
    h, l, c = hlc(60_000, 71, gaps)
    ins = [h, l, c] if name == "willr" else [h, l]
    ind = V.CLASSES[name](0)
    ind.set_policy("tune", "off")  # the launcher's default: the progression kernel
    out = ind.batch_dev(*ins, sweep={"period": rng})
    assert "progression" in ind.last_kernel, ind.last_kernel
    out = out if isinstance(out, tuple) else (out,)
    periods = list(range(rng[0], rng[1] + 1, rng[2]))
    exp = expect(name, h, l, c, periods)
    tol = 5e-5 if name == "willr" else 1e-6
    for k in range(len(exp)):
        close(out[k].to_host(), exp[k], tol, f"{name} {rng} output {k}")


@pytest.mark.parametrize("name", ["willr", "donchian"])
def test_progression_equals_sparse_table(name):
    # the tuner times both kernels; whichever it keeps, the values agree
    # with the progression kernel's to the last bit (min / max are exact)
    h, l, c = hlc(700_001, 73, False)
    ins = [h, l, c] if name == "willr" else [h, l]
    sweep = {"period": (5, 500, 5)}
    a = V.CLASSES[name](0)
    a.set_policy("tune", "off")
    ref = a.batch_dev(*ins, sweep=sweep)
    ref = ref if isinstance(ref, tuple) else (ref,)
    b = V.CLASSES[name](0)
    b.set_policy("tune", "on")
    got = b.batch_dev(*ins, sweep=sweep)
    got = got if isinstance(got, tuple) else (got,)
    for k in range(len(ref)):
        assert np.array_equal(ref[k].to_host(), got[k].to_host(), equal_nan=True), (name, k, b.last_kernel)

"""Request server (vta_server_*) through the C ABI.

* Alone vs in the mix: a mix of requests (ALMA on tensor cores, EMA, RSI,
  ADX, Bollinger and more) submitted together runs concurrently on several
  slots; every result equals the same sweep run alone through the
  indicator's own entry point (the server runs the same kernels, so the
  results are expected to be bit-identical; the comparison allows 1e-6
  relative with NaN positions exact).
* A memory budget smaller than the mix's outputs defers requests until
  earlier ones are released, and they still complete correctly.
* Invalid requests are refused at submit.
"""
import time

import numpy as np
import pytest

from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu

RTOL = 1e-6

MIX = [
    ("alma", 0, {"period": (5, 60, 5), "offset": (0.5, 0.95, 0.15), "sigma": (3.0, 9.0, 3.0)}),
    ("ema", 1, {"period": (2, 200, 3)}),
    ("rsi", 2, {"period": (2, 100, 1)}),
    ("adx", 0, {"period": (5, 40, 5)}),
    ("bollinger_bands", 1, {"period": (5, 100, 5), "devup": (2.0, 2.0, 0.0), "devdn": (2.0, 2.0, 0.0)}),
    ("sma", 2, {"period": (5, 300, 5)}),
    ("willr", 1, {"period": (5, 60, 5)}),
    ("supertrend", 2, {"period": (7, 14, 7), "factor": (2.0, 3.0, 1.0)}),
    ("alma", 1, {"period": (9, 9, 0), "offset": (0.85, 0.85, 0.0), "sigma": (6.0, 6.0, 0.0)}),
    ("ema", 0, {"period": (10, 10, 0)}),
]


@pytest.fixture(scope="module")
def store():
    out = []
    for i, (n, lead) in enumerate(((20000, 0), (7001, 13), (3000, 40))):
        d = datagen.ohlcv(n, seed=70 + i, nan_lead=lead)
        out.append({k: d[k].astype(np.float32) for k in ("high", "low", "close")})
    return out


def alone(name, s, sweep):
    kind = V.N.INDICATORS[name][0]
    ins = {"x": [s["close"]], "hl": [s["high"], s["low"]], "hlc": [s["high"], s["low"], s["close"]]}[kind]
    ind = V.CLASSES[name](0)
    r = ind.batch_dev(*ins, sweep=sweep)
    r = r if isinstance(r, tuple) else (r,)
    return [a.to_host() for a in r]


def same(got, exp, what):
    assert got.shape == exp.shape, what
    assert np.array_equal(np.isnan(got), np.isnan(exp)), f"{what}: NaN positions differ"
    m = ~np.isnan(exp)
    np.testing.assert_allclose(got[m], exp[m], rtol=RTOL, atol=0, err_msg=what)


def drain(srv, n, timeout=120.0):
    done, t0 = {}, time.time()
    while len(done) < n:
        for c in srv.poll(64, wait_ms=100):
            done[c["ticket"]] = c
        assert time.time() - t0 < timeout, "server did not finish"
    return done


def test_results_alone_equal_results_in_the_mix(store):
    srv = V.Server(0, slots=4)
    ids = [srv.add_series(s["close"], s["high"], s["low"]) for s in store]
    tickets = [srv.submit(name, ids[si], sw) for name, si, sw in MIX]
    done = drain(srv, len(tickets))
    st = srv.stats()
    assert st["completed"] == st["submitted"] == len(MIX) and st["failed"] == 0
    for t, (name, si, sw) in zip(tickets, MIX):
        c = done[t]
        assert c["status"] == 0, name
        assert c["t_submit"] <= c["t_start"] <= c["t_done"]
        exp = alone(name, store[si], sw)
        for k, e in enumerate(exp):
            same(srv.copy_out(t, k, c["rows"], c["cols"]), e, f"{name}[{k}] on series {si}")
        srv.release(t)
    assert srv.stats()["bytes_in_use"] == 0
    srv.close()


def test_memory_budget_defers_and_completes(store):
    s = store[0]
    one = 20 * s["close"].size * 4  # bytes of a 20-combo request on series 0
    srv = V.Server(0, slots=4, memory_budget=int(one * 1.5))
    sid = srv.add_series(s["close"], s["high"], s["low"])
    sweeps = [{"period": (p, p + 19, 1)} for p in (2, 30, 60, 90)]
    tickets = [srv.submit("ema", sid, sw) for sw in sweeps]
    got = {}
    t0 = time.time()
    while len(got) < len(tickets):
        for c in srv.poll(8, wait_ms=100):
            assert c["status"] == 0
            got[c["ticket"]] = srv.copy_out(c["ticket"], 0, c["rows"], c["cols"])
            srv.release(c["ticket"])  # frees budget for the next one
        assert time.time() - t0 < 60
    st = srv.stats()
    assert st["deferred"] > 0 and st["completed"] == len(tickets)
    for t, sw in zip(tickets, sweeps):
        same(got[t], alone("ema", s, sw)[0], f"ema {sw}")
    srv.close()


def test_invalid_requests_are_refused(store):
    srv = V.Server(0, slots=2)
    s = store[2]
    sid = srv.add_series(s["close"], s["high"], s["low"])
    cid = srv.add_series(s["close"])  # close only
    with pytest.raises(V.VtaError, match="unknown indicator"):
        srv.submit("nope", sid, {"period": (5, 5, 0)})
    with pytest.raises(V.VtaError, match="unknown series"):
        srv.submit("ema", 99, {"period": (5, 5, 0)})
    with pytest.raises(V.VtaError, match="no high/low"):
        srv.submit("adx", cid, {"period": (14, 14, 0)})
    with pytest.raises(V.VtaError):
        srv.submit("ema", sid, {"period": (5000, 5000, 0)})  # period longer than the series
    with pytest.raises(V.VtaError):
        srv.release(12345)
    assert srv.stats()["submitted"] == 0
    srv.close()

"""Stream banks (the crate's XStream structs on the device): S streams fed
bar by bar agree bit for bit with the oracle's restatement of each
XStream::update, NaN gaps included, through the host and the device entry."""
import numpy as np
import pytest

from oracle import oracle as O
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu

S, T = 37, 700


def series(seed):
    xs = []
    for j in range(S):
        x = datagen.random_walk(T, seed=seed + j, nan_lead=j % 5)
        if j % 7 == 3:
            x[200 + j] = np.nan  # an interior gap in some streams
        xs.append(x.astype(np.float32))
    return np.stack(xs, axis=1)  # [T][S]


def bars(x, finite=False):
    """(high, low, close) around x; finite=True replaces the NaN bars (for
    streams the crate feeds finite candles only)."""
    rng = np.random.default_rng(7)
    xc = np.nan_to_num(x, nan=100.0) if finite else x
    hi = (xc * (1 + np.abs(rng.normal(0, 0.005, x.shape)))).astype(np.float32)
    lo = (xc * (1 - np.abs(rng.normal(0, 0.005, x.shape)))).astype(np.float32)
    return hi, lo, xc.astype(np.float32)


CASES = [
    ("ema", {"period": 12}), ("sma", {"period": 9}),
    ("alma", {"period": 21, "offset": 0.8, "sigma": 5.0}),
    ("rsi", {"period": 14}), ("wilders", {"period": 7}), ("atr", {"length": 10}),
    ("dema", {"period": 20}), ("tema", {"period": 9}), ("tema", {"period": 1}),
    ("wma", {"period": 15}), ("swma", {"period": 6}), ("swma", {"period": 7}), ("pwma", {"period": 9}),
    ("stddev", {"period": 10, "nbdev": 1.5}), ("zscore", {"period": 14, "nbdev": 1.0}),
    ("bollinger_bands", {"period": 20, "devup": 2.0, "devdn": 1.5, "matype": "sma"}),
    ("bollinger_bands", {"period": 12, "matype": "ema"}),
    ("donchian", {"period": 20}), ("willr", {"period": 14}), ("adx", {"period": 14}),
    ("supertrend", {"period": 10, "factor": 3.0}),
    ("sinwma", {"period": 14}), ("trima", {"period": 30}), ("trima", {"period": 9}),
    ("cwma", {"period": 14}), ("fwma", {"period": 5}), ("srwma", {"period": 14}), ("srwma", {"period": 1}),
    ("sqwma", {"period": 14}), ("epma", {"period": 11, "offset": 4}), ("epma", {"period": 20, "offset": 0}),
    ("vpwma", {"period": 14, "power": 0.382}), ("vpwma", {"period": 10, "power": 2.0}),
    ("vpwma", {"period": 9, "power": 0.0}), ("vpwma", {"period": 30, "power": 5.0}),
    ("percentile_nearest_rank", {"length": 15, "percentage": 50.0}),
    ("percentile_nearest_rank", {"length": 20, "percentage": 90.0}),
]


def inputs_for(name, x):
    n_in = O.STREAMS[name][0]
    if n_in == 1:
        return [x]
    # ATR / ADX / SuperTrend: finite candles, as the crate's own streams
    # assume; Donchian / WillR keep the NaN bars (their windows handle them)
    hi, lo, cl = bars(x, finite=name in ("atr", "adx", "supertrend"))
    return [hi, lo] if n_in == 2 else [hi, lo, cl]


@pytest.mark.parametrize("name,params", CASES, ids=[f"{n}-{i}" for i, (n, _) in enumerate(CASES)])
def test_stream_bank_matches_oracle(name, params):
    x = series(100)
    ins = inputs_for(name, x)
    bank = V.StreamBank(name, S, params)
    n_out = O.STREAMS[name][1]
    assert (bank.n_inputs, bank.n_outputs) == (len(ins), n_out)
    got = np.stack([bank.update(*[a[t] for a in ins]) for t in range(T)])  # [T]([n_out])[S]
    if n_out == 1:
        got = got[:, None, :]
    for j in range(S):
        exp = O.stream(name, [a[:, j].astype(np.float64) for a in ins], **params)
        exp = exp if isinstance(exp, tuple) else (exp,)
        for k in range(n_out):
            e = exp[k].astype(np.float32)
            assert np.array_equal(got[:, k, j], e, equal_nan=True), (name, j, k, np.flatnonzero(
                ~((got[:, k, j] == e) | (np.isnan(got[:, k, j]) & np.isnan(e))))[:5])
    # reset: the same bars give the same values again, now through device buffers
    import torch

    bank.reset()
    d_out = torch.empty(n_out, S, device="cuda")
    for t in range(60):
        d_in = [torch.from_numpy(np.ascontiguousarray(a[t])).cuda() for a in ins]
        bank.update_device(*d_in, d_out=d_out)
        assert np.array_equal(d_out.cpu().numpy(), got[t], equal_nan=True), (name, t)
    bank.close()


def test_stream_bank_rejects_unknown_and_bad_params():
    with pytest.raises(RuntimeError):
        V.StreamBank("hma", 4)
    with pytest.raises(RuntimeError):
        V.StreamBank("ema", 4, {"period": 0})
    with pytest.raises(RuntimeError):
        V.StreamBank("alma", 4, {"period": 9, "offset": 1.5})
    with pytest.raises(RuntimeError):
        V.StreamBank("wma", 4, {"period": 1})
    with pytest.raises(RuntimeError):
        V.StreamBank("stddev", 4, {"nbdev": -1.0})
    with pytest.raises(RuntimeError):
        V.StreamBank("bollinger_bands", 4, {"matype": "wma"})
    with pytest.raises(RuntimeError):
        V.StreamBank("zscore", 4, {"devtype": 1})
    with pytest.raises(RuntimeError):
        V.StreamBank("trima", 4, {"period": 3})
    with pytest.raises(RuntimeError):
        V.StreamBank("epma", 4, {"period": 5, "offset": 5})
    with pytest.raises(RuntimeError):
        V.StreamBank("percentile_nearest_rank", 4, {"percentage": 101.0})

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


@pytest.mark.parametrize("name,params", [("ema", {"period": 12}), ("sma", {"period": 9}),
                                         ("alma", {"period": 21, "offset": 0.8, "sigma": 5.0}),
                                         ("rsi", {"period": 14}), ("wilders", {"period": 7}),
                                         ("atr", {"length": 10})])
def test_stream_bank_matches_oracle(name, params):
    x = series(100)
    ins = [x]
    if name == "atr":
        rng = np.random.default_rng(7)
        xf = np.nan_to_num(x, nan=100.0)  # AtrStream assumes finite inputs
        hi = (xf * (1 + np.abs(rng.normal(0, 0.005, x.shape)))).astype(np.float32)
        lo = (xf * (1 - np.abs(rng.normal(0, 0.005, x.shape)))).astype(np.float32)
        ins = [hi, lo, xf]
    bank = V.StreamBank(name, S, params)
    got = np.stack([bank.update(*[a[t] for a in ins]) for t in range(T)])
    for j in range(S):
        exp = O.stream(name, [a[:, j].astype(np.float64) for a in ins], **params).astype(np.float32)
        assert np.array_equal(got[:, j], exp, equal_nan=True), (name, j)
    # reset: the same bars give the same values again, now through device buffers
    import torch

    bank.reset()
    d_out = torch.empty(S, device="cuda")
    for t in range(50):
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

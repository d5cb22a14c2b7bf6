"""Seeded synthetic market data with the shapes of the benchmark workloads.

Counter-based RNG: splitmix64 over (seed, stream, index) -> 53-bit uniform ->
Box-Muller normal.  Prices are a geometric random walk x_0 = 100,
x_{t+1} = x_t * exp(eps_t), eps ~ N(0, sigma^2).  The same function of
(seed, length) always yields the same float64 series, on any machine.
"""
from __future__ import annotations

import numpy as np

_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
_G = np.uint64(0x9E3779B97F4A7C15)


def splitmix64(x: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = x + _G
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, n: int, offset: int = 0) -> np.ndarray:
    """(0, 1) uniforms: 53 high bits of splitmix64(seed<<40 | stream<<32 | i)."""
    base = (np.uint64(seed & 0xFFFFFF) << np.uint64(40)) | (np.uint64(stream & 0xFF) << np.uint64(32))
    k = np.arange(offset, offset + n, dtype=np.uint64) + base
    return ((splitmix64(k) >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def normal(seed: int, stream: int, n: int) -> np.ndarray:
    u1 = uniform(seed, 2 * stream, n)
    u2 = uniform(seed, 2 * stream + 1, n)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def random_walk(n: int, seed: int, sigma: float = 0.01, start: float = 100.0, nan_lead: int = 0) -> np.ndarray:
    eps = sigma * normal(seed, 0, max(n - 1, 0))
    x = np.empty(n, dtype=np.float64)
    if n:
        x[0] = 0.0
        np.cumsum(eps, out=x[1:])
        x = start * np.exp(x)
    x[:nan_lead] = np.nan
    return x


def high_low(close: np.ndarray, seed: int, sigma: float = 0.005):
    """high/low = close * (1 +- |N(0, sigma^2)|) (the recurrence/window sweep workload)."""
    n = close.size
    hi = close * (1.0 + np.abs(sigma * normal(seed, 1, n)))
    lo = close * (1.0 - np.abs(sigma * normal(seed, 2, n)))
    return hi, lo


def ohlcv(n: int, seed: int, nan_lead: int = 0, sigma: float = 0.01, hl_sigma: float = 0.004):
    """open = previous close; high/low = max/min(open, close) * (1 +- |N(0, hl_sigma^2)|);
    volume lognormal(10, 1)."""
    close = random_walk(n, seed, sigma)
    opn = np.empty_like(close)
    opn[0] = close[0]
    opn[1:] = close[:-1]
    hi = np.maximum(opn, close) * (1.0 + np.abs(hl_sigma * normal(seed, 1, n)))
    lo = np.minimum(opn, close) * (1.0 - np.abs(hl_sigma * normal(seed, 2, n)))
    vol = np.exp(10.0 + normal(seed, 3, n))
    for a in (opn, hi, lo, close, vol):
        a[:nan_lead] = np.nan
    return {"open": opn, "high": hi, "low": lo, "close": close, "volume": vol}


def ragged_many_series(n_series: int, seed: int, min_len: int = 1000, max_len: int = 50000,
                       max_nan_lead: int = 500, fields=("open", "high", "low", "close", "volume"),
                       threads: int | None = None):
    """Many OHLCV series of uneven length and NaN lead, stacked time-major
    [max_len][n_series] as float32 with a NaN tail past each series' end.
    Series s is ohlcv(len_s, seed * 100003 + s, lead_s); series are generated
    on `threads` threads (numpy releases the GIL), each writing its column."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    u_len = uniform(seed, 10, n_series)
    u_lead = uniform(seed, 11, n_series)
    lens = (min_len + np.floor(u_len * (max_len - min_len + 1))).astype(np.int64)
    leads = np.floor(u_lead * (max_nan_lead + 1)).astype(np.int64)
    rows = int(lens.max())
    out = {k: np.full((rows, n_series), np.nan, dtype=np.float32) for k in fields}

    def one(s):
        d = ohlcv(int(lens[s]), seed * 100003 + s, nan_lead=int(leads[s]))
        for k in fields:
            out[k][: lens[s], s] = d[k]

    # many small numpy calls hold the GIL often: scaling stops at ~4 threads
    workers = threads or min(4, os.cpu_count() or 1)
    if workers <= 1:
        for s in range(n_series):
            one(s)
    else:
        with ThreadPoolExecutor(workers) as ex:
            list(ex.map(one, range(n_series)))
    return out, lens, leads


# ------------------------------------------------------------ GPU version ----
# The same generator evaluated with torch on a device, for many series at once
# (int64 arithmetic wraps like the uint64 one; shifts are made logical).  The
# float64 results equal the numpy ones up to the last bits of exp/log/cos, so
# the float32 series agree with ohlcv() to rounding.
def _i64(u: int) -> int:
    u &= (1 << 64) - 1
    return u - (1 << 64) if u >= (1 << 63) else u


def _lsr(z, k: int):
    return (z >> k) & ((1 << (64 - k)) - 1)


def _splitmix64_t(x):
    z = x + _i64(0x9E3779B97F4A7C15)
    z = (z ^ _lsr(z, 30)) * _i64(0xBF58476D1CE4E5B9)
    z = (z ^ _lsr(z, 27)) * _i64(0x94D049BB133111EB)
    return z ^ _lsr(z, 31)


def _base_t(torch, seeds, stream: int, device):
    return torch.tensor([_i64(((s & 0xFFFFFF) << 40) | ((stream & 0xFF) << 32)) for s in seeds], dtype=torch.int64,
                        device=device)


def _uniform_t(torch, base_e, idx):
    z = _splitmix64_t(base_e + idx)
    return (_lsr(z, 11).to(torch.float64) + 0.5) * (1.0 / 9007199254740992.0)


def _normal_t(torch, seeds, rep, stream: int, idx, device):
    b1 = torch.repeat_interleave(_base_t(torch, seeds, 2 * stream, device), rep)
    b2 = torch.repeat_interleave(_base_t(torch, seeds, 2 * stream + 1, device), rep)
    u1 = _uniform_t(torch, b1, idx)
    u2 = _uniform_t(torch, b2, idx)
    return torch.sqrt(-2.0 * torch.log(u1)) * torch.cos(2.0 * np.pi * u2)


def ohlc_many_torch(lens, seeds, leads, device="cuda", sigma: float = 0.01, hl_sigma: float = 0.004):
    """high, low, close of series s = ohlcv(lens[s], seeds[s], leads[s]),
    concatenated as float32 device tensors, plus the int64 segment offsets."""
    import torch

    lens = [int(v) for v in lens]
    rep = torch.tensor(lens, dtype=torch.int64, device=device)
    offs = torch.zeros(len(lens), dtype=torch.int64, device=device)
    offs[1:] = torch.cumsum(rep, 0)[:-1]
    total = int(sum(lens))
    j = torch.arange(total, dtype=torch.int64, device=device) - torch.repeat_interleave(offs, rep)
    # random walk: x[0] = 0, x[j] = sum of eps[0..j-1], eps = sigma * normal(seed, 0, .)
    eps = sigma * _normal_t(torch, seeds, rep, 0, j - 1, device)
    eps[j == 0] = 0.0
    cs = torch.cumsum(eps, 0)
    del eps
    close = 100.0 * torch.exp(cs - torch.repeat_interleave(cs[offs], rep))
    del cs
    opn = torch.empty_like(close)
    opn[1:] = close[:-1]
    first = j == 0
    opn[first] = close[first]
    hi = torch.maximum(opn, close) * (1.0 + torch.abs(hl_sigma * _normal_t(torch, seeds, rep, 1, j, device)))
    lo = torch.minimum(opn, close) * (1.0 - torch.abs(hl_sigma * _normal_t(torch, seeds, rep, 2, j, device)))
    del opn
    lead = torch.repeat_interleave(torch.tensor([int(v) for v in leads], dtype=torch.int64, device=device), rep)
    nan = j < lead
    out = []
    for a in (hi, lo, close):
        a = a.to(torch.float32)
        a[nan] = float("nan")
        out.append(a)
    return out[0], out[1], out[2], offs

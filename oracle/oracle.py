"""ctypes front-end for the C oracle (oracle/vta_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, always as the checker.  The product package
(vectorta_gb300) never imports this module.

Every function takes float64 numpy arrays and returns float64 outputs with the
reference crate's NaN warm-up prefix.  Batch helpers expand parameter grids
with the oracle's own restatement of each indicator's ``expand_grid``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libvta_oracle.so")
_lib = None

# descending-range modes of vto_axis_usize (see vta_oracle.c)
AX_DESC, AX_SWAP, AX_REV_FROM_END, AX_DESC_PLUS_END = 0, 1, 2, 3

# per-indicator descending-axis behaviour of the crate's expand_grid
AXIS_MODE = {
    "alma": AX_DESC, "ema": AX_SWAP, "dema": AX_DESC, "tema": AX_DESC,
    "rsi": AX_SWAP, "wilders": AX_DESC, "atr": AX_REV_FROM_END, "adx": AX_DESC,
    "supertrend": AX_DESC, "sma": AX_DESC, "stddev": AX_DESC, "zscore": AX_DESC,
    "bollinger": AX_DESC, "bollinger_bands": AX_DESC, "donchian": AX_DESC, "willr": AX_DESC,
    "percentile_nearest_rank": AX_DESC, "wma": AX_DESC_PLUS_END, "swma": AX_DESC,
    "pwma": AX_DESC, "sinwma": AX_DESC, "trima": AX_SWAP,
    "cwma": AX_SWAP, "fwma": AX_SWAP, "srwma": AX_DESC, "sqwma": AX_DESC, "epma": AX_SWAP,
    "vpwma": AX_DESC,
}


class OracleError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"oracle {what}: status {code}")
        self.code = code


def build() -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or (
            os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "vta_oracle.c"))
        ):
            build()
        L = C.CDLL(_LIB_PATH)
        dp, sz, db, ip = C.POINTER(C.c_double), C.c_size_t, C.c_double, C.c_int
        szp = C.POINTER(C.c_size_t)
        sig = {
            "vto_axis_usize": ([sz, sz, sz, C.c_int, szp, sz], sz),
            "vto_axis_f64": ([db, db, db, dp, sz], sz),
            "vto_alma": ([dp, sz, sz, db, db, dp], ip),
            "vto_alma_batch": ([dp, sz, sz, szp, dp, dp, dp], ip),
            "vto_alma_weights_batch": ([sz, db, db, dp, dp], None),
            "vto_ema": ([dp, sz, sz, dp], ip),
            "vto_dema": ([dp, sz, sz, dp], ip),
            "vto_tema": ([dp, sz, sz, dp], ip),
            "vto_rsi": ([dp, sz, sz, dp], ip),
            "vto_rsi_batch": ([dp, sz, sz, szp, dp], ip),
            "vto_wilders": ([dp, sz, sz, dp], ip),
            "vto_wilders_batch": ([dp, sz, sz, szp, dp], ip),
            "vto_atr": ([dp, dp, dp, sz, sz, dp], ip),
            "vto_adx": ([dp, dp, dp, sz, sz, dp], ip),
            "vto_supertrend": ([dp, dp, dp, sz, sz, db, dp, dp], ip),
            "vto_sma": ([dp, sz, sz, dp], ip),
            "vto_sma_batch": ([dp, sz, sz, szp, dp], ip),
            "vto_stddev": ([dp, sz, sz, db, dp], ip),
            "vto_zscore": ([dp, sz, sz, db, dp], ip),
            "vto_zscore_batch_row": ([dp, sz, sz, db, dp], ip),
            "vto_stddev_batch_prefix": ([dp, sz, sz, db, dp], ip),
            "vto_window_exact": ([dp, sz, sz, szp, sz, dp, dp], ip),
            "vto_alma_batch_row_at": ([dp, sz, sz, db, db, szp, sz, dp], ip),
            "vto_bollinger": ([dp, sz, sz, db, db, dp, dp, dp], ip),
            "vto_donchian": ([dp, dp, sz, sz, dp, dp, dp], ip),
            "vto_willr": ([dp, dp, dp, sz, sz, dp], ip),
            "vto_percentile_nearest_rank": ([dp, sz, sz, db, dp], ip),
            "vto_wma": ([dp, sz, sz, dp], ip),
            "vto_swma": ([dp, sz, sz, dp], ip),
            "vto_pwma": ([dp, sz, sz, C.c_int, dp], ip),
            "vto_pwma_weights": ([sz, dp], None),
            "vto_sinwma": ([dp, sz, sz, dp], ip),
            "vto_sinwma_weights": ([sz, dp], None),
            "vto_trima": ([dp, sz, sz, dp], ip),
            "vto_donchian_fast": ([dp, dp, sz, sz, dp, dp, dp], ip),
            "vto_willr_fast": ([dp, dp, dp, sz, sz, dp], ip),
            "vto_cwma": ([dp, sz, sz, dp], ip),
            "vto_fwma": ([dp, sz, sz, dp], ip),
            "vto_srwma": ([dp, sz, sz, dp], ip),
            "vto_sqwma": ([dp, sz, sz, dp], ip),
            "vto_epma": ([dp, sz, sz, sz, dp], ip),
            "vto_vpwma": ([dp, sz, sz, db, dp], ip),
            "vto_ema_stream": ([dp, sz, sz, dp], ip),
            "vto_sma_stream": ([dp, sz, sz, dp], ip),
            "vto_alma_stream": ([dp, sz, sz, db, db, dp], ip),
            "vto_rsi_stream": ([dp, sz, sz, dp], ip),
            "vto_atr_stream": ([dp, dp, dp, sz, sz, dp], ip),
            "vto_wilders_stream": ([dp, sz, sz, dp], ip),
            "vto_dema_stream": ([dp, sz, sz, dp], ip),
            "vto_tema_stream": ([dp, sz, sz, dp], ip),
            "vto_wma_stream": ([dp, sz, sz, dp], ip),
            "vto_swma_stream": ([dp, sz, sz, dp], ip),
            "vto_pwma_stream": ([dp, sz, sz, dp], ip),
            "vto_stddev_stream": ([dp, sz, sz, db, dp], ip),
            "vto_zscore_stream": ([dp, sz, sz, db, dp], ip),
            "vto_bollinger_stream": ([dp, sz, sz, db, db, ip, dp, dp, dp], ip),
            "vto_donchian_stream": ([dp, dp, sz, sz, dp, dp, dp], ip),
            "vto_willr_stream": ([dp, dp, dp, sz, sz, dp], ip),
            "vto_adx_stream": ([dp, dp, dp, sz, sz, dp], ip),
            "vto_supertrend_stream": ([dp, dp, dp, sz, sz, db, dp, dp], ip),
            "vto_sinwma_stream": ([dp, sz, sz, dp], ip),
            "vto_trima_stream": ([dp, sz, sz, dp], ip),
            "vto_cwma_stream": ([dp, sz, sz, dp], ip),
            "vto_fwma_stream": ([dp, sz, sz, dp], ip),
            "vto_srwma_stream": ([dp, sz, sz, dp], ip),
            "vto_sqwma_stream": ([dp, sz, sz, dp], ip),
            "vto_epma_stream": ([dp, sz, sz, sz, dp], ip),
            "vto_vpwma_stream": ([dp, sz, sz, db, dp], ip),
            "vto_percentile_nearest_rank_stream": ([dp, sz, sz, db, dp], ip),
        }
        for name, (args, res) in sig.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _lib = L
    return _lib


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _check(code: int, what: str):
    if code != 0:
        raise OracleError(code, what)


# ---------------------------------------------------------------- grids ----
def axis_usize(rng, mode=AX_DESC) -> list[int]:
    start, end, step = (int(v) for v in rng)
    n = lib().vto_axis_usize(start, end, step, mode, None, 0)
    buf = (C.c_size_t * max(n, 1))()
    lib().vto_axis_usize(start, end, step, mode, buf, n)
    return [int(buf[i]) for i in range(n)]


def axis_f64(rng) -> list[float]:
    start, end, step = (float(v) for v in rng)
    n = lib().vto_axis_f64(start, end, step, None, 0)
    buf = np.zeros(max(n, 1))
    lib().vto_axis_f64(start, end, step, _p(buf), n)
    return [float(v) for v in buf[:n]]


def periods_of(name: str, rng) -> list[int]:
    return axis_usize(rng, AXIS_MODE[name])


# ------------------------------------------------------- single series ----
def _single(fname, x, *params):
    x = _f64(x)
    out = np.empty_like(x)
    _check(getattr(lib(), fname)(_p(x), x.size, *params, _p(out)), fname)
    return out


def alma(x, period=9, offset=0.85, sigma=6.0):
    return _single("vto_alma", x, period, offset, sigma)


def ema(x, period=9):
    return _single("vto_ema", x, period)


def dema(x, period=30):
    return _single("vto_dema", x, period)


def tema(x, period=9):
    return _single("vto_tema", x, period)


def rsi(x, period=14):
    return _single("vto_rsi", x, period)


def wilders(x, period=5):
    return _single("vto_wilders", x, period)


def sma(x, period=9):
    return _single("vto_sma", x, period)


def stddev(x, period=5, nbdev=1.0):
    return _single("vto_stddev", x, period, nbdev)


def zscore(x, period=14, nbdev=1.0):
    return _single("vto_zscore", x, period, nbdev)


def zscore_batch_row(x, period=14, nbdev=1.0):
    return _single("vto_zscore_batch_row", x, period, nbdev)


def stddev_batch_prefix(x, period=5, nbdev=1.0):
    """The crate's batch StdDev row: differences of whole-series f64 prefixes."""
    return _single("vto_stddev_batch_prefix", x, period, nbdev)


def window_exact(x, period, idx):
    """Exact (corrected two-pass f64) mean and population standard deviation of
    the windows [i-period+1, i] ending at each index in `idx`.  Not a crate
    path: the yardstick that measures the crate's running-sum drift."""
    x = _f64(x)
    idx = np.ascontiguousarray(idx, dtype=np.uintp)
    mean = np.empty(idx.size)
    sd = np.empty(idx.size)
    _check(lib().vto_window_exact(_p(x), x.size, period, idx.ctypes.data_as(C.POINTER(C.c_size_t)), idx.size,
                                  _p(mean), _p(sd)), "window_exact")
    return mean, sd


def percentile_nearest_rank(x, length=15, percentage=50.0):
    return _single("vto_percentile_nearest_rank", x, length, percentage)


def wma(x, period=30):
    return _single("vto_wma", x, period)


def swma(x, period=5):
    return _single("vto_swma", x, period)


def pwma(x, period=5, batch=False):
    return _single("vto_pwma", x, period, int(batch))


def sinwma(x, period=14):
    return _single("vto_sinwma", x, period)


def cwma(x, period=14):
    return _single("vto_cwma", x, period)


def fwma(x, period=5):
    return _single("vto_fwma", x, period)


def srwma(x, period=14):
    return _single("vto_srwma", x, period)


def sqwma(x, period=14):
    return _single("vto_sqwma", x, period)


def vpwma(x, period=14, power=0.382):
    return _single("vto_vpwma", x, period, power)


def epma(x, period=11, offset=4):
    return _single("vto_epma", x, period, offset)


# The crate's XStream parameter defaults (XParams::default / try_new) and
# each stream's inputs and outputs.
STREAMS = {
    "ema": (1, 1, {"period": 9}),
    "sma": (1, 1, {"period": 9}),
    "alma": (1, 1, {"period": 9, "offset": 0.85, "sigma": 6.0}),
    "rsi": (1, 1, {"period": 14}),
    "atr": (3, 1, {"length": 14}),
    "wilders": (1, 1, {"period": 5}),
    "dema": (1, 1, {"period": 30}),
    "tema": (1, 1, {"period": 9}),
    "wma": (1, 1, {"period": 30}),
    "swma": (1, 1, {"period": 5}),
    "pwma": (1, 1, {"period": 5}),
    "stddev": (1, 1, {"period": 5, "nbdev": 1.0}),
    "zscore": (1, 1, {"period": 14, "nbdev": 1.0}),
    "bollinger_bands": (1, 3, {"period": 20, "devup": 2.0, "devdn": 2.0, "matype": "sma"}),
    "donchian": (2, 3, {"period": 20}),
    "willr": (3, 1, {"period": 14}),
    "adx": (3, 1, {"period": 14}),
    "supertrend": (3, 2, {"period": 10, "factor": 3.0}),
    "sinwma": (1, 1, {"period": 14}),
    "trima": (1, 1, {"period": 30}),
    "cwma": (1, 1, {"period": 14}),
    "fwma": (1, 1, {"period": 5}),
    "srwma": (1, 1, {"period": 14}),
    "sqwma": (1, 1, {"period": 14}),
    "epma": (1, 1, {"period": 11, "offset": 4}),
    "vpwma": (1, 1, {"period": 14, "power": 0.382}),
    "percentile_nearest_rank": (1, 1, {"length": 15, "percentage": 50.0}),
}


def stream(name, inputs, **prm):
    """The crate's XStream for `name` fed the inputs bar by bar (NaN where
    update() returns None).  One output: an array; several (Bollinger,
    Donchian: upper / middle / lower; SuperTrend: trend / changed): a tuple."""
    xs = [_f64(a) for a in inputs]
    n_in, n_out, dflt = STREAMS[name]
    assert len(xs) == n_in, (name, len(xs))
    q = dict(dflt)
    q.update(prm)
    outs = [np.empty_like(xs[0]) for _ in range(n_out)]
    n = xs[0].size
    L = lib()
    P = [_p(a) for a in xs]
    O_ = [_p(o) for o in outs]
    if name == "alma":
        code = L.vto_alma_stream(P[0], n, int(q["period"]), float(q["offset"]), float(q["sigma"]), O_[0])
    elif name == "atr":
        code = L.vto_atr_stream(*P, n, int(q["length"]), O_[0])
    elif name in ("stddev", "zscore"):
        code = getattr(L, f"vto_{name}_stream")(P[0], n, int(q["period"]), float(q["nbdev"]), O_[0])
    elif name == "bollinger_bands":
        mt = {"sma": 0, "ema": 1}[str(q["matype"]).lower()]
        code = L.vto_bollinger_stream(P[0], n, int(q["period"]), float(q["devup"]), float(q["devdn"]), mt, *O_)
    elif name == "donchian":
        code = L.vto_donchian_stream(*P, n, int(q["period"]), *O_)
    elif name == "epma":
        code = L.vto_epma_stream(P[0], n, int(q["period"]), int(q["offset"]), O_[0])
    elif name == "vpwma":
        code = L.vto_vpwma_stream(P[0], n, int(q["period"]), float(q["power"]), O_[0])
    elif name == "percentile_nearest_rank":
        code = L.vto_percentile_nearest_rank_stream(P[0], n, int(q["length"]), float(q["percentage"]), O_[0])
    elif name == "supertrend":
        code = L.vto_supertrend_stream(*P, n, int(q["period"]), float(q["factor"]), *O_)
    elif n_in == 3:
        code = getattr(L, f"vto_{name}_stream")(*P, n, int(q["period"]), O_[0])
    else:
        code = getattr(L, f"vto_{name}_stream")(P[0], n, int(q["period"]), O_[0])
    _check(code, f"{name} stream")
    return outs[0] if n_out == 1 else tuple(outs)


def trima(x, period=30):
    return _single("vto_trima", x, period)


def bollinger(x, period=20, devup=2.0, devdn=2.0):
    x = _f64(x)
    u, m, lo = np.empty_like(x), np.empty_like(x), np.empty_like(x)
    _check(lib().vto_bollinger(_p(x), x.size, period, devup, devdn, _p(u), _p(m), _p(lo)), "bb")
    return u, m, lo


def _hlc(h, l, c):
    h, l, c = _f64(h), _f64(l), _f64(c)
    assert h.size == l.size == c.size
    return h, l, c


def atr(h, l, c, length=14):
    h, l, c = _hlc(h, l, c)
    out = np.empty_like(c)
    _check(lib().vto_atr(_p(h), _p(l), _p(c), c.size, length, _p(out)), "atr")
    return out


def adx(h, l, c, period=14):
    h, l, c = _hlc(h, l, c)
    out = np.empty_like(c)
    _check(lib().vto_adx(_p(h), _p(l), _p(c), c.size, period, _p(out)), "adx")
    return out


def supertrend(h, l, c, period=10, factor=3.0):
    h, l, c = _hlc(h, l, c)
    tr, ch = np.empty_like(c), np.empty_like(c)
    _check(lib().vto_supertrend(_p(h), _p(l), _p(c), c.size, period, factor, _p(tr), _p(ch)), "st")
    return tr, ch


def willr(h, l, c, period=14, fast=False):
    h, l, c = _hlc(h, l, c)
    out = np.empty_like(c)
    fn = lib().vto_willr_fast if fast else lib().vto_willr
    _check(fn(_p(h), _p(l), _p(c), c.size, period, _p(out)), "willr")
    return out


def donchian(h, l, period=20, fast=False):
    h, l = _f64(h), _f64(l)
    u, m, lo = np.empty_like(h), np.empty_like(h), np.empty_like(h)
    fn = lib().vto_donchian_fast if fast else lib().vto_donchian
    _check(fn(_p(h), _p(l), h.size, period, _p(u), _p(m), _p(lo)), "donchian")
    return u, m, lo


# ---------------------------------------------------------------- batch ----
def alma_batch(x, period_rng, offset_rng, sigma_rng):
    """alma_batch_with_kernel(ScalarBatch): rows in expand_grid order."""
    x = _f64(x)
    ps = axis_usize(period_rng, AX_DESC)
    os_ = axis_f64(offset_rng)
    ss = axis_f64(sigma_rng)
    combos = [(p, o, s) for p in ps for o in os_ for s in ss]
    rows = len(combos)
    P = np.array([c[0] for c in combos], dtype=np.uintp)
    O = np.array([c[1] for c in combos], dtype=np.float64)
    S = np.array([c[2] for c in combos], dtype=np.float64)
    out = np.empty((rows, x.size))
    _check(lib().vto_alma_batch(_p(x), x.size, rows, P.ctypes.data_as(C.POINTER(C.c_size_t)),
                                _p(O), _p(S), _p(out)), "alma_batch")
    return out, combos


def alma_batch_row_at(x, period, offset, sigma, idx):
    """One alma_batch row (batch weights) evaluated at the end indices idx."""
    x = _f64(x)
    idx = np.ascontiguousarray(idx, dtype=np.uintp)
    out = np.empty(idx.size)
    _check(lib().vto_alma_batch_row_at(_p(x), x.size, period, offset, sigma,
                                       idx.ctypes.data_as(C.POINTER(C.c_size_t)), idx.size, _p(out)),
           "alma_batch_row_at")
    return out


def _period_batch(fname, x, periods):
    x = _f64(x)
    P = np.array(periods, dtype=np.uintp)
    out = np.empty((len(periods), x.size))
    _check(getattr(lib(), fname)(_p(x), x.size, len(periods),
                                 P.ctypes.data_as(C.POINTER(C.c_size_t)), _p(out)), fname)
    return out


def rsi_batch(x, periods):
    return _period_batch("vto_rsi_batch", x, periods)


def sma_batch(x, periods):
    return _period_batch("vto_sma_batch", x, periods)


def wilders_batch(x, periods):
    return _period_batch("vto_wilders_batch", x, periods)


def rows_of(fn, x, periods, **kw):
    """Batch of a single-series oracle: one row per period (the crate's batch
    rows call the same scalar row function)."""
    return np.stack([fn(x, p, **kw) for p in periods])

"""Python mirror of the crate's per-indicator CUDA wrappers (src/cuda/*).

For every indicator X there is a class ``CudaX`` (``CudaAlma``, ``CudaEma`` ...)
whose constructor takes a device id like ``CudaAlma::new(device_id)``
(alma_wrapper.rs:133) and whose methods keep the wrapper names:

    x_batch_dev(data_f32, sweep)                          -> DeviceArrayF32
    x_batch_into_host_f32(data_f32, sweep)                -> (ndarray, rows, cols)
    x_batch_device(d_data, len, first_valid, sweep, d_out)
    x_many_series_one_param_time_major_dev(data_tm, params) -> DeviceArrayF32
    x_many_series_one_param_device(d_data_tm, cols, rows, params, d_out)
    expand_grid(sweep)                                    -> list of params

High/low/close indicators take ``high, low, close`` (Donchian: ``high, low``)
where the crate does; multi-output indicators return tuples.  Sweeps are the
crate's ``XBatchRange`` as plain tuples ``(start, end, step)``; errors raise
``VtaError`` whose ``kind`` is the crate's error variant.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field, fields
from typing import Any

import numpy as np

from . import _native as N

__all__ = ["DeviceArrayF32", "Context", "VtaError", "TmPlan", "Server"]
VtaError = N.VtaError


# ------------------------------------------------------------------ sweeps --
@dataclass
class AlmaBatchRange:
    period: tuple = (9, 258, 1)       # alma.rs:1074-1082
    offset: tuple = (0.85, 0.85, 0.0)
    sigma: tuple = (6.0, 6.0, 0.0)


@dataclass
class PeriodBatchRange:
    period: tuple = (9, 258, 1)


@dataclass
class StdDevBatchRange:
    period: tuple = (5, 254, 1)       # stddev.rs:578-585
    nbdev: tuple = (1.0, 1.0, 0.0)


@dataclass
class ZscoreBatchRange:
    period: tuple = (14, 263, 1)      # zscore.rs:793-802 (ma_type "sma", devtype 0)
    nbdev: tuple = (1.0, 1.0, 0.0)


@dataclass
class BollingerBandsBatchRange:
    period: tuple = (20, 269, 1)      # bollinger_bands.rs:1095-1104
    devup: tuple = (2.0, 2.0, 0.0)
    devdn: tuple = (2.0, 2.0, 0.0)


@dataclass
class SuperTrendBatchRange:
    period: tuple = (10, 10, 0)
    factor: tuple = (3.0, 3.0, 0.0)


@dataclass
class PercentileNearestRankBatchRange:
    length: tuple = (15, 264, 1)      # percentile_nearest_rank.rs:820-827
    percentage: tuple = (50.0, 50.0, 0.0)


@dataclass
class EpmaBatchRange:
    period: tuple = (11, 260, 1)      # epma.rs:754-760
    offset: tuple = (4, 4, 0)


@dataclass
class AlmaParams:
    period: int = 9
    offset: float = 0.85
    sigma: float = 6.0


@dataclass
class PeriodParams:
    period: int = 9


@dataclass
class StdDevParams:
    period: int = 5
    nbdev: float = 1.0


@dataclass
class ZscoreParams:
    period: int = 14
    nbdev: float = 1.0


@dataclass
class BollingerBandsParams:
    period: int = 20
    devup: float = 2.0
    devdn: float = 2.0


@dataclass
class SuperTrendParams:
    period: int = 10
    factor: float = 3.0


@dataclass
class PercentileNearestRankParams:
    length: int = 15
    percentage: float = 50.0


@dataclass
class VpwmaBatchRange:
    period: tuple = (14, 263, 1)      # vpwma.rs:892-899
    power: tuple = (0.382, 0.382, 0.0)


@dataclass
class VpwmaParams:
    period: int = 14
    power: float = 0.382


@dataclass
class EpmaParams:
    period: int = 11
    offset: int = 4


_RANGE_CLS = {"alma": AlmaBatchRange, "period": PeriodBatchRange, "stddev": StdDevBatchRange,
              "zscore": ZscoreBatchRange, "bollinger": BollingerBandsBatchRange,
              "supertrend": SuperTrendBatchRange, "percentile": PercentileNearestRankBatchRange,
              "epma": EpmaBatchRange, "vpwma": VpwmaBatchRange}
_PARAM_CLS = {"alma": AlmaParams, "period": PeriodParams, "stddev": StdDevParams,
              "zscore": ZscoreParams, "bollinger": BollingerBandsParams,
              "supertrend": SuperTrendParams, "percentile": PercentileNearestRankParams,
              "epma": EpmaParams, "vpwma": VpwmaParams}


def _to_sweep(fam: str, sweep) -> Any:
    S = N.SWEEPS[fam]
    if sweep is None:
        sweep = _RANGE_CLS[fam]()
    s = S()
    for fname, ftype in S._fields_:
        v = getattr(sweep, fname) if not isinstance(sweep, dict) else sweep[fname]
        if ftype is N.RangeUsize:
            setattr(s, fname, N.RangeUsize(int(v[0]), int(v[1]), int(v[2])))
        else:
            setattr(s, fname, N.RangeF64(float(v[0]), float(v[1]), float(v[2])))
    return s


def _to_params(fam: str, params) -> Any:
    P = N.PARAMS[fam]
    if params is None:
        params = _PARAM_CLS[fam]()
    p = P()
    for fname, ftype in P._fields_:
        v = getattr(params, fname) if not isinstance(params, dict) else params[fname]
        setattr(p, fname, int(v) if ftype is C.c_size_t else float(v))
    return p


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


def _dptr(obj) -> int:
    """Device pointer of a torch tensor, a __cuda_array_interface__ object or an int."""
    if isinstance(obj, int):
        return obj
    if hasattr(obj, "data_ptr"):
        return int(obj.data_ptr())
    if hasattr(obj, "__cuda_array_interface__"):
        return int(obj.__cuda_array_interface__["data"][0])
    if isinstance(obj, DeviceArrayF32):
        return obj.ptr
    raise TypeError(f"not a device buffer: {type(obj)!r}")


# ------------------------------------------------------------------ context --
def pinned_empty(shape, dtype=np.float32) -> np.ndarray:
    """A numpy array in page-locked host memory from vta_pinned_alloc (the
    crate's LockedBuffer); freed when the array is collected.  As the output
    of batch_into_host_f32 it takes the kernels' stores directly."""
    import weakref

    dt = np.dtype(dtype)
    shape = (shape,) if isinstance(shape, int) else tuple(shape)
    nbytes = int(np.prod(shape, dtype=np.int64)) * dt.itemsize
    p = C.c_void_p()
    N.check(N.lib().vta_pinned_alloc(max(nbytes, 1), C.byref(p)))
    raw = (C.c_char * max(nbytes, 1)).from_address(p.value)
    weakref.finalize(raw, N.lib().vta_pinned_free, C.c_void_p(p.value))
    return np.frombuffer(raw, dtype=dt, count=int(np.prod(shape, dtype=np.int64))).reshape(shape)


class Context:
    """Owns a vta_ctx (one stream and a scratch workspace on one device)."""

    def __init__(self, device_id: int = 0):
        L = N.lib()
        h = C.c_void_p()
        N.check(L.vta_ctx_create(int(device_id), C.byref(h)))
        self.handle = h
        self.device_id = int(device_id)

    def synchronize(self):
        N.check(N.lib().vta_ctx_synchronize(self.handle))

    def set_policy(self, key: str, value: str):
        N.check(N.lib().vta_ctx_set_policy(self.handle, key.encode(), str(value).encode()))

    def set_stream(self, cuda_stream: int | None):
        N.check(N.lib().vta_ctx_set_stream(self.handle, C.c_void_p(cuda_stream or 0)))

    @property
    def stream(self) -> int:
        return int(N.lib().vta_ctx_get_stream(self.handle) or 0)

    @property
    def last_kernel(self) -> str:
        return N.lib().vta_ctx_last_kernel(self.handle).decode()

    @property
    def scratch_bytes(self) -> int:
        return int(N.lib().vta_ctx_scratch_bytes(self.handle))

    @property
    def kernel_ms(self) -> float:
        """Duration of the last call's main kernel (policy timing=on), else -1."""
        return float(N.lib().vta_ctx_kernel_ms(self.handle))

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            N.lib().vta_ctx_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# DLPack capsules (the Python side of vta_device_array_to_dlpack).  A
# consumer renames the capsule to "used_dltensor[_versioned]" and takes over
# the managed tensor; a capsule that is dropped unconsumed still carries its
# original name, and its destructor then frees the tensor.
# private prototypes: the shared C.pythonapi function objects can have their
# argtypes changed by other code in the process
_capsule_new = C.PYFUNCTYPE(C.py_object, C.c_void_p, C.c_char_p, C.c_void_p)(("PyCapsule_New", C.pythonapi))
_capsule_valid = C.PYFUNCTYPE(C.c_int, C.c_void_p, C.c_char_p)(("PyCapsule_IsValid", C.pythonapi))
_capsule_ptr = C.PYFUNCTYPE(C.c_void_p, C.c_void_p, C.c_char_p)(("PyCapsule_GetPointer", C.pythonapi))
_DL_NAMES = {0: b"dltensor", 1: b"dltensor_versioned"}


def _make_capsule_dtor(versioned: int):
    name = _DL_NAMES[versioned]

    @C.CFUNCTYPE(None, C.c_void_p)
    def dtor(cap):
        if _capsule_valid(cap, name):
            N.lib().vta_dlpack_delete(_capsule_ptr(cap, name), versioned)

    return dtor


_CAPSULE_DTORS = {v: _make_capsule_dtor(v) for v in (0, 1)}  # kept alive for the process


class DeviceArrayF32:
    """Owned device array (alma_wrapper.rs:103-117) with zero-copy export via
    ``__cuda_array_interface__`` (torch.as_tensor / cupy.asarray work on it)
    and ``__dlpack__`` / ``__dlpack_device__`` (torch.from_dlpack), as the
    crate's DeviceArrayF32Py does (dlpack_cuda.rs:267-374).  ``__dlpack__``
    hands the buffer over to the capsule, as the crate does: the array is
    empty afterwards."""

    def __init__(self, c: N.DeviceArrayC, ctx: Context):
        self._c = c
        self._ctx = ctx  # keeps the context (and its device) alive

    @property
    def ptr(self) -> int:
        return int(self._c.ptr or 0)

    @property
    def rows(self) -> int:
        return int(self._c.rows)

    @property
    def cols(self) -> int:
        return int(self._c.cols)

    @property
    def shape(self):
        return (self.rows, self.cols)

    def __len__(self):
        return self.rows * self.cols

    @property
    def __cuda_array_interface__(self):
        return {"shape": (self.rows, self.cols), "typestr": "<f4", "data": (self.ptr, False),
                "version": 3, "strides": None}

    def __dlpack_device__(self):
        return (2, int(self._c.device))  # kDLCUDA

    def __dlpack__(self, stream=None, max_version=None, dl_device=None, copy=None):
        if dl_device is not None and tuple(dl_device) != self.__dlpack_device__():
            raise ValueError("dl_device mismatch for __dlpack__" if not copy else
                             "device copy not implemented for __dlpack__")
        # every entry point returns after its work has finished, so the data
        # is complete on any consumer stream
        versioned = 1 if (max_version is not None and tuple(max_version)[0] >= 1) else 0
        out = C.c_void_p()
        N.check(N.lib().vta_device_array_to_dlpack(C.byref(self._c), versioned, C.byref(out)))
        dtor = _CAPSULE_DTORS[versioned]
        return _capsule_new(out.value, _DL_NAMES[versioned], C.cast(dtor, C.c_void_p).value)

    def to_host(self) -> np.ndarray:
        out = np.empty((self.rows, self.cols), dtype=np.float32)
        N.check(N.lib().vta_device_array_copy_to_host(
            self._ctx.handle, C.byref(self._c), out.ctypes.data_as(C.POINTER(C.c_float)), out.size))
        return out

    def free(self):
        if self._c.ptr:
            N.lib().vta_device_array_free(C.byref(self._c))

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


# ------------------------------------------------------------- indicators --
class _CudaIndicator:
    NAME = ""

    def __init__(self, device_id: int = 0, ctx: "Context | None" = None):
        self.ctx = ctx if ctx is not None else Context(device_id)
        kind, outs, fam = N.INDICATORS[self.NAME]
        self._kind, self._outs, self._fam = kind, outs, fam
        self._nin = N.N_IN[kind]

    # crate: CudaX::synchronize / set_policy / selected kernel
    def synchronize(self):
        self.ctx.synchronize()

    def set_policy(self, key: str, value: str):
        self.ctx.set_policy(key, value)

    @property
    def last_kernel(self) -> str:
        return self.ctx.last_kernel

    def _fn(self, suffix):
        return getattr(N.lib(), f"vta_{self.NAME}_{suffix}")

    def _wrap(self, arrs):
        res = [DeviceArrayF32(a, self.ctx) for a in arrs]
        return res[0] if len(res) == 1 else tuple(res)

    def expand_grid(self, sweep=None) -> list:
        s = _to_sweep(self._fam, sweep)
        n = C.c_size_t()
        self._fn("expand_grid")(C.byref(s), None, 0, C.byref(n))
        P = N.PARAMS[self._fam]
        buf = (P * max(n.value, 1))()
        N.check(self._fn("expand_grid")(C.byref(s), buf, n.value, C.byref(n)))
        return [{f: getattr(buf[i], f) for f, _ in P._fields_} for i in range(n.value)]

    def batch_dev(self, *inputs, sweep=None):
        ins = [_f32(a) for a in inputs]
        assert len(ins) == self._nin, f"{self.NAME} takes {self._nin} input series"
        n = ins[0].size
        assert all(a.size == n for a in ins), "inconsistent input lengths"
        outs = [N.DeviceArrayC() for _ in self._outs]
        N.check(self._fn("batch_dev")(self.ctx.handle, *[a.ctypes.data for a in ins], n,
                                      C.byref(_to_sweep(self._fam, sweep)), *[C.byref(o) for o in outs]))
        return self._wrap(outs)

    def batch_into_host_f32(self, *inputs, sweep=None, out=None):
        ins = [_f32(a) for a in inputs]
        n = ins[0].size
        s = _to_sweep(self._fam, sweep)
        rows = len(self.expand_grid(sweep))
        hs = out if out is not None else [np.empty((rows, n), dtype=np.float32) for _ in self._outs]
        r, c = C.c_size_t(), C.c_size_t()
        N.check(self._fn("batch_into_host_f32")(self.ctx.handle, *[a.ctypes.data for a in ins], n, C.byref(s),
                                                *[h.ctypes.data for h in hs], rows * n, C.byref(r), C.byref(c)))
        res = hs[0] if len(hs) == 1 else tuple(hs)
        return res, r.value, c.value

    def batch_device(self, d_inputs, length: int, first_valid: int, sweep, d_outs):
        d_inputs = d_inputs if isinstance(d_inputs, (list, tuple)) else [d_inputs]
        d_outs = d_outs if isinstance(d_outs, (list, tuple)) else [d_outs]
        N.check(self._fn("batch_device")(self.ctx.handle, *[_dptr(x) for x in d_inputs], int(length),
                                         int(first_valid), C.byref(_to_sweep(self._fam, sweep)),
                                         *[_dptr(o) for o in d_outs]))

    def many_series_one_param_time_major_dev(self, *inputs_tm, params=None):
        ins = [_f32(a) for a in inputs_tm]
        assert len(ins) == self._nin
        rows, cols = ins[0].shape
        outs = [N.DeviceArrayC() for _ in self._outs]
        N.check(self._fn("many_series_one_param_time_major_dev")(
            self.ctx.handle, *[a.ctypes.data for a in ins], cols, rows,
            C.byref(_to_params(self._fam, params)), *[C.byref(o) for o in outs]))
        return self._wrap(outs)

    def many_series_one_param_device(self, d_inputs_tm, cols: int, rows: int, params, d_outs):
        d_inputs_tm = d_inputs_tm if isinstance(d_inputs_tm, (list, tuple)) else [d_inputs_tm]
        d_outs = d_outs if isinstance(d_outs, (list, tuple)) else [d_outs]
        N.check(self._fn("many_series_one_param_device")(
            self.ctx.handle, *[_dptr(x) for x in d_inputs_tm], int(cols), int(rows),
            C.byref(_to_params(self._fam, params)), *[_dptr(o) for o in d_outs]))


class VramMaComputer:
    """One MA by name over a device-resident series for an arbitrary period
    list, like the crate's VramMaComputer (vram_ma.rs:87-160, 574, 2153);
    outputs go to a caller-provided device buffer, [period][t] or, with
    time_major=True, [t][period]."""

    def __init__(self, device_id: int = 0, ctx: "Context | None" = None):
        self.ctx = ctx if ctx is not None else Context(device_id)

    @staticmethod
    def supports(ma_type: str) -> bool:
        """supports_vram_kernel_ma (vram_ma.rs:68-76) for this library's kernels."""
        return bool(N.lib().vta_ma_supported(ma_type.encode()))

    def compute_period_ma_into(self, ma_type: str, params, d_prices, series_len: int, first_valid: int,
                               periods, d_out, time_major: bool = False):
        keys, vals, n = _kv(params)
        per = (C.c_int * len(periods))(*[int(p) for p in periods])
        N.check(N.lib().vta_ma_periods_device(self.ctx.handle, ma_type.encode(), keys, vals, n,
                                              _dptr(d_prices), int(series_len), int(first_valid), per,
                                              len(periods), 1 if time_major else 0, _dptr(d_out)))


def _kv(params):
    params = params or {}
    keys = (C.c_char_p * max(len(params), 1))(*[k.encode() for k in params])
    vals = (C.c_double * max(len(params), 1))(*[float(v) for v in params.values()])
    return keys, vals, len(params)


class CudaMaSelector:
    """MA by name from host prices (the crate's CudaMaSelector,
    ma_selector.rs:194-1820): one period or a period sweep, to a device array
    or to host f32."""

    def __init__(self, device_id: int = 0, ctx: "Context | None" = None):
        self.ctx = ctx if ctx is not None else Context(device_id)

    def ma_sweep_to_device(self, ma_type: str, data, start: int, end: int, step: int, params=None):
        x = _f32(data)
        keys, vals, n = _kv(params)
        out = N.DeviceArrayC()
        N.check(N.lib().vta_ma_select_dev(self.ctx.handle, ma_type.encode(), keys, vals, n, x.ctypes.data, x.size,
                                          int(start), int(end), int(step), C.byref(out)))
        return DeviceArrayF32(out, self.ctx)

    def ma_to_device(self, ma_type: str, data, period: int, params=None):
        return self.ma_sweep_to_device(ma_type, data, period, period, 0, params)

    def ma_sweep_to_host_f32(self, ma_type: str, data, start: int, end: int, step: int, params=None):
        x = _f32(data)
        keys, vals, n = _kv(params)
        r, c = C.c_size_t(), C.c_size_t()
        rows = len(_selector_periods(int(start), int(end), int(step)))
        out = np.empty((rows, x.size), dtype=np.float32)
        N.check(N.lib().vta_ma_select_into_host_f32(self.ctx.handle, ma_type.encode(), keys, vals, n, x.ctypes.data,
                                                    x.size, int(start), int(end), int(step), out.ctypes.data,
                                                    out.size, C.byref(r), C.byref(c)))
        return out, r.value, c.value

    def ma_to_host_f32(self, ma_type: str, data, period: int, params=None):
        out, _, _ = self.ma_sweep_to_host_f32(ma_type, data, period, period, 0, params)
        return out[0]


class StreamBank:
    """n_streams streams of one indicator on the device, advanced together one
    bar per update, each as the crate's XStream (EmaStream, SmaStream,
    AlmaStream, RsiStream, AtrStream, WildersStream, DemaStream, TemaStream,
    WmaStream, SwmaStream, PwmaStream, StdDevStream, ZscoreStream,
    BollingerBandsStream, DonchianStream, WillrStream, AdxStream,
    SuperTrendStream).  update() takes one array of n_streams values per input
    (value; Donchian high, low; ATR / WillR / ADX / SuperTrend high, low,
    close) and returns the n_streams new values, NaN where the crate's
    update() returns None; several outputs (Bollinger and Donchian upper /
    middle / lower, SuperTrend trend / changed) come as an
    [n_outputs][n_streams] array.  String parameters take the crate's names:
    Bollinger matype "sma" / "ema", Z-score ma_type "sma"."""

    _CODES = {"matype": {"sma": 0.0, "ema": 1.0}, "ma_type": {"sma": 0.0}}

    def __init__(self, indicator: str, n_streams: int, params=None, device_id: int = 0,
                 ctx: "Context | None" = None):
        self.ctx = ctx if ctx is not None else Context(device_id)
        self.indicator, self.n = indicator, int(n_streams)
        prm = {}
        for k, v in dict(params or {}).items():
            if isinstance(v, str):
                codes = self._CODES.get(k, {})
                if v.lower() not in codes:
                    raise RuntimeError(f"streams: {k}={v!r} has no streaming kernel")
                v = codes[v.lower()]
            prm[k] = v
        keys, vals, n = _kv(prm)
        h = C.c_void_p()
        N.check(N.lib().vta_streams_create(self.ctx.handle, indicator.encode(), keys, vals, n, self.n, C.byref(h)))
        self._h = h
        ni, no = C.c_int(), C.c_int()
        N.check(N.lib().vta_streams_shape(self._h, C.byref(ni), C.byref(no)))
        self.n_inputs, self.n_outputs = ni.value, no.value

    def update(self, *bars) -> np.ndarray:
        assert len(bars) == self.n_inputs, (self.indicator, len(bars))
        xs = [_f32(b) for b in bars]
        assert all(x.size == self.n for x in xs)
        out = np.empty((self.n_outputs, self.n), dtype=np.float32)
        ptrs = [x.ctypes.data for x in xs] + [None] * (3 - len(xs))
        N.check(N.lib().vta_streams_update_host(self._h, *ptrs, out.ctypes.data))
        return out[0] if self.n_outputs == 1 else out

    def update_device(self, *d_bars, d_out):
        """d_out: n_outputs x n_streams f32 on the device."""
        assert len(d_bars) == self.n_inputs, (self.indicator, len(d_bars))
        ptrs = [_dptr(b) for b in d_bars] + [None] * (3 - len(d_bars))
        N.check(N.lib().vta_streams_update_device(self._h, *ptrs, _dptr(d_out)))

    def reset(self):
        N.check(N.lib().vta_streams_reset(self._h))

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            N.lib().vta_streams_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _selector_periods(start: int, end: int, step: int) -> list:
    """The selector's period range rule (ma_selector.rs:1037-1061)."""
    if step == 0 or start == end:
        return [start]
    if start < end:
        return list(range(start, end + 1, step))
    v, cur = [], start
    while cur >= end:
        v.append(cur)
        if cur == 0:
            break
        nxt = max(cur - step, 0)
        if nxt == cur:
            break
        cur = nxt
        if cur < end:
            break
    return v


def _make(name: str, cls_name: str):
    def method(suffix):
        def f(self, *a, **k):
            return getattr(_CudaIndicator, suffix)(self, *a, **k)
        f.__name__ = f"{name}_{suffix}"
        return f

    ns = {"NAME": name}
    for suffix in ("batch_dev", "batch_into_host_f32", "batch_device",
                   "many_series_one_param_time_major_dev", "many_series_one_param_device"):
        ns[f"{name}_{suffix}"] = method(suffix)
    cls = type(cls_name, (_CudaIndicator,), ns)
    globals()[cls_name] = cls
    __all__.append(cls_name)
    return cls


_CLASS_NAMES = {
    "alma": "CudaAlma", "ema": "CudaEma", "dema": "CudaDema", "tema": "CudaTema", "rsi": "CudaRsi",
    "wilders": "CudaWilders", "sma": "CudaSma", "wma": "CudaWma", "swma": "CudaSwma", "pwma": "CudaPwma",
    "sinwma": "CudaSinwma", "trima": "CudaTrima", "stddev": "CudaStddev", "zscore": "CudaZscore",
    "bollinger_bands": "CudaBollingerBands", "atr": "CudaAtr", "adx": "CudaAdx",
    "supertrend": "CudaSupertrend", "donchian": "CudaDonchian", "willr": "CudaWillr",
    "percentile_nearest_rank": "CudaPercentileNearestRank",
    "cwma": "CudaCwma", "fwma": "CudaFwma", "srwma": "CudaSrwma", "sqwma": "CudaSqwma", "epma": "CudaEpma",
    "vpwma": "CudaVpwma",
}
CLASSES = {name: _make(name, cls) for name, cls in _CLASS_NAMES.items()}
__all__ += ["AlmaBatchRange", "PeriodBatchRange", "StdDevBatchRange", "ZscoreBatchRange",
            "BollingerBandsBatchRange", "SuperTrendBatchRange", "PercentileNearestRankBatchRange",
            "AlmaParams", "PeriodParams", "StdDevParams", "ZscoreParams", "BollingerBandsParams",
            "SuperTrendParams", "PercentileNearestRankParams", "EpmaBatchRange", "EpmaParams", "VpwmaBatchRange",
            "VpwmaParams", "VramMaComputer",
            "CudaMaSelector", "StreamBank",
            "CLASSES", "pinned_empty",
            "device_count", "launch_count"]


class TmPlan:
    """Several indicators over ragged time-major OHLC series in one persistent,
    graph-captured launch (vta_tm_plan_*).

    high/low/close: device [rows][cols] float32 (torch tensors or pointers);
    lengths: per-series valid rows (None = all rows); jobs: dicts with
    kind in {"atr", "adx", "supertrend", "percentile_nearest_rank"}, period,
    param (SuperTrend factor / percentile percentage) and device outputs out0
    (and out1 for SuperTrend).  The buffers stay bound to the plan.
    """

    def __init__(self, high, low, close, cols: int, rows: int, lengths, jobs, ctx: "Context | None" = None,
                 device_id: int = 0):
        self.ctx = ctx or Context(device_id)
        self._keep = (high, low, close, jobs)
        arr = (N.TmJobC * len(jobs))()
        for i, j in enumerate(jobs):
            arr[i].kind = N.TM_KINDS[j["kind"]]
            arr[i].period = int(j["period"])
            arr[i].param = float(j.get("param", 0.0))
            arr[i].d_out0 = _dptr(j["out0"])
            arr[i].d_out1 = _dptr(j["out1"]) if j.get("out1") is not None else None
        lens = None
        if lengths is not None:
            self._lens = (C.c_size_t * cols)(*[int(v) for v in lengths])
            lens = self._lens
        h = C.c_void_p()
        N.check(N.lib().vta_tm_plan_create(self.ctx.handle, _dptr(high), _dptr(low), _dptr(close), int(cols),
                                           int(rows), lens, arr, len(jobs), C.byref(h)))
        self.handle = h

    def run(self):
        N.check(N.lib().vta_tm_plan_run(self.handle))

    def info(self) -> dict:
        i = N.TmPlanInfoC()
        N.check(N.lib().vta_tm_plan_info_get(self.handle, C.byref(i)))
        return {"n_items": i.n_items, "chunk": list(i.chunk), "fixups": i.fixups, "tuned": bool(i.tuned)}

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            N.lib().vta_tm_plan_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _sweep_c(sweep: dict) -> "N.SweepC":
    """dict with "period" (start, end, step) and optionally p1 / p2 (start, end, step);
    the indicator's own names (offset/sigma, nbdev, devup/devdn, factor, percentage) map to p1/p2."""
    alias = {"offset": "p1", "sigma": "p2", "nbdev": "p1", "devup": "p1", "devdn": "p2", "factor": "p1",
             "percentage": "p1", "length": "period"}
    d = {alias.get(k, k): v for k, v in sweep.items()}
    s = N.SweepC()
    p = d["period"]
    s.period = N.RangeUsize(int(p[0]), int(p[1]), int(p[2]))
    for f in ("p1", "p2"):
        v = d.get(f, (0.0, 0.0, 0.0))
        setattr(s, f, N.RangeF64(float(v[0]), float(v[1]), float(v[2])))
    return s


class Server:
    """Request server (vta_server_*): a device-resident series store and
    continuously batched single-series sweeps of any batch indicator."""

    def __init__(self, device_id: int = 0, slots: int = 0, memory_budget: int = 0):
        cfg = N.ServerConfigC(int(slots), int(memory_budget))
        h = C.c_void_p()
        N.check(N.lib().vta_server_create(int(device_id), C.byref(cfg), C.byref(h)))
        self.handle = h

    def add_series(self, close, high=None, low=None) -> int:
        c = _f32(close)
        hi = None if high is None else _f32(high)
        lo = None if low is None else _f32(low)
        i = C.c_uint32()
        N.check(N.lib().vta_server_add_series(self.handle, None if hi is None else hi.ctypes.data,
                                              None if lo is None else lo.ctypes.data, c.ctypes.data, c.size,
                                              C.byref(i)))
        return i.value

    def add_series_device(self, close, length: int, high=None, low=None) -> int:
        i = C.c_uint32()
        N.check(N.lib().vta_server_add_series_device(self.handle, None if high is None else _dptr(high),
                                                     None if low is None else _dptr(low), _dptr(close),
                                                     int(length), C.byref(i)))
        return i.value

    def submit(self, indicator: str, series: int, sweep: dict) -> int:
        r = N.RequestC(indicator.encode(), int(series), _sweep_c(sweep))
        t = C.c_uint64()
        N.check(N.lib().vta_server_submit(self.handle, C.byref(r), C.byref(t)))
        return t.value

    def poll(self, cap: int = 64, wait_ms: int = 0) -> list:
        arr = (N.CompletionC * cap)()
        n = C.c_size_t()
        N.check(N.lib().vta_server_poll(self.handle, arr, cap, C.byref(n), int(wait_ms)))
        out = []
        for c in arr[: n.value]:
            out.append({"ticket": c.ticket, "status": c.status, "rows": c.rows, "cols": c.cols, "n_out": c.n_out,
                        "d_out": [c.d_out[k] for k in range(c.n_out)], "t_submit": c.t_submit,
                        "t_start": c.t_start, "t_done": c.t_done})
        return out

    def copy_out(self, ticket: int, k: int, rows: int, cols: int) -> np.ndarray:
        h = np.empty((rows, cols), dtype=np.float32)
        N.check(N.lib().vta_server_copy_out(self.handle, int(ticket), int(k), h.ctypes.data, h.size))
        return h

    def release(self, ticket: int):
        N.check(N.lib().vta_server_release(self.handle, int(ticket)))

    def stats(self) -> dict:
        st = N.ServerStatsC()
        N.check(N.lib().vta_server_get_stats(self.handle, C.byref(st)))
        return {f: getattr(st, f) for f, _ in N.ServerStatsC._fields_}

    def close(self):
        if getattr(self, "handle", None) is not None and self.handle.value:
            N.lib().vta_server_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def launch_count() -> int:
    """Kernels launched by the library so far in this process."""
    return int(N.lib().vta_launch_count())


def device_count() -> int:
    """cuda_device_count() (src/cuda/mod.rs:560-575)."""
    return int(N.lib().vta_device_count())

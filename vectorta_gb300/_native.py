"""Loads libvta_gb300.so (built in-tree by vectorta_gb300/build.py) and
declares the ctypes signatures of its C ABI (include/vta_gb300.h).

There is no CPU fallback: if the library is missing this module raises, and
every GPU entry point returns an error status when no sm_103a device exists.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_lib", "libvta_gb300.so")
HEADER = os.path.join(ROOT, "include", "vta_gb300.h")

STATUS = {
    0: "OK", 1: "Cuda", 2: "OutOfMemory", 3: "MissingKernelSymbol", 4: "InvalidInput",
    5: "InvalidPolicy", 6: "LaunchConfigTooLarge", 7: "DeviceMismatch", 8: "NotImplemented",
}


class VtaError(RuntimeError):
    """Mirrors the crate's CudaXError enums: `kind` is the variant name.
    OutOfMemory also carries the variant's fields `required`, `free` and
    `headroom` (bytes)."""

    def __init__(self, status: int, message: str, oom=None):
        self.status = status
        self.kind = STATUS.get(status, f"status{status}")
        self.required, self.free, self.headroom = oom if oom else (0, 0, 0)
        super().__init__(f"{self.kind}: {message}")


class RangeUsize(C.Structure):
    _fields_ = [("start", C.c_size_t), ("end", C.c_size_t), ("step", C.c_size_t)]


class RangeF64(C.Structure):
    _fields_ = [("start", C.c_double), ("end", C.c_double), ("step", C.c_double)]


class DeviceArrayC(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("rows", C.c_size_t), ("cols", C.c_size_t), ("device", C.c_int)]


# sweep / params structs (field order as in the header)
def _struct(name, fields):
    return type(name, (C.Structure,), {"_fields_": fields})


SWEEPS = {
    "alma": _struct("vta_alma_batch_range", [("period", RangeUsize), ("offset", RangeF64), ("sigma", RangeF64)]),
    "period": _struct("vta_period_batch_range", [("period", RangeUsize)]),
    "stddev": _struct("vta_stddev_batch_range", [("period", RangeUsize), ("nbdev", RangeF64)]),
    "zscore": _struct("vta_zscore_batch_range", [("period", RangeUsize), ("nbdev", RangeF64)]),
    "bollinger": _struct("vta_bollinger_batch_range",
                         [("period", RangeUsize), ("devup", RangeF64), ("devdn", RangeF64)]),
    "supertrend": _struct("vta_supertrend_batch_range", [("period", RangeUsize), ("factor", RangeF64)]),
    "percentile": _struct("vta_percentile_batch_range", [("length", RangeUsize), ("percentage", RangeF64)]),
    "epma": _struct("vta_epma_batch_range", [("period", RangeUsize), ("offset", RangeUsize)]),
    "vpwma": _struct("vta_vpwma_batch_range", [("period", RangeUsize), ("power", RangeF64)]),
}
PARAMS = {
    "alma": _struct("vta_alma_params", [("period", C.c_size_t), ("offset", C.c_double), ("sigma", C.c_double)]),
    "period": _struct("vta_period_params", [("period", C.c_size_t)]),
    "stddev": _struct("vta_stddev_params", [("period", C.c_size_t), ("nbdev", C.c_double)]),
    "zscore": _struct("vta_zscore_params", [("period", C.c_size_t), ("nbdev", C.c_double)]),
    "bollinger": _struct("vta_bollinger_params",
                         [("period", C.c_size_t), ("devup", C.c_double), ("devdn", C.c_double)]),
    "supertrend": _struct("vta_supertrend_params", [("period", C.c_size_t), ("factor", C.c_double)]),
    "percentile": _struct("vta_percentile_params", [("length", C.c_size_t), ("percentage", C.c_double)]),
    "epma": _struct("vta_epma_params", [("period", C.c_size_t), ("offset", C.c_size_t)]),
    "vpwma": _struct("vta_vpwma_params", [("period", C.c_size_t), ("power", C.c_double)]),
}

# name -> (input kind, outputs, sweep/params family)
INDICATORS = {
    "alma": ("x", ["out"], "alma"),
    "ema": ("x", ["out"], "period"),
    "dema": ("x", ["out"], "period"),
    "tema": ("x", ["out"], "period"),
    "rsi": ("x", ["out"], "period"),
    "wilders": ("x", ["out"], "period"),
    "sma": ("x", ["out"], "period"),
    "wma": ("x", ["out"], "period"),
    "swma": ("x", ["out"], "period"),
    "pwma": ("x", ["out"], "period"),
    "sinwma": ("x", ["out"], "period"),
    "trima": ("x", ["out"], "period"),
    "stddev": ("x", ["out"], "stddev"),
    "zscore": ("x", ["out"], "zscore"),
    "bollinger_bands": ("x", ["upper", "middle", "lower"], "bollinger"),
    "atr": ("hlc", ["out"], "period"),
    "adx": ("hlc", ["out"], "period"),
    "supertrend": ("hlc", ["trend", "changed"], "supertrend"),
    "donchian": ("hl", ["upper", "middle", "lower"], "period"),
    "willr": ("hlc", ["out"], "period"),
    "percentile_nearest_rank": ("x", ["out"], "percentile"),
    "cwma": ("x", ["out"], "period"),
    "fwma": ("x", ["out"], "period"),
    "srwma": ("x", ["out"], "period"),
    "sqwma": ("x", ["out"], "period"),
    "epma": ("x", ["out"], "epma"),
    "vpwma": ("x", ["out"], "vpwma"),
}
N_IN = {"x": 1, "hl": 2, "hlc": 3}


# many-series plans (vta_tm_job / vta_tm_plan_info)
class TmJobC(C.Structure):
    _fields_ = [("kind", C.c_int), ("period", C.c_size_t), ("param", C.c_double),
                ("d_out0", C.c_void_p), ("d_out1", C.c_void_p)]


class TmPlanInfoC(C.Structure):
    _fields_ = [("n_items", C.c_size_t), ("chunk", C.c_size_t * 8), ("fixups", C.c_size_t), ("tuned", C.c_int)]


TM_KINDS = {"atr": 0, "adx": 1, "supertrend": 2, "percentile_nearest_rank": 3}


# request server (vta_sweep / vta_request / vta_completion / ...)
class SweepC(C.Structure):
    _fields_ = [("period", RangeUsize), ("p1", RangeF64), ("p2", RangeF64)]


class ServerConfigC(C.Structure):
    _fields_ = [("slots", C.c_int), ("memory_budget", C.c_size_t)]


class RequestC(C.Structure):
    _fields_ = [("indicator", C.c_char_p), ("series", C.c_uint32), ("sweep", SweepC)]


class CompletionC(C.Structure):
    _fields_ = [("ticket", C.c_uint64), ("status", C.c_int), ("rows", C.c_size_t), ("cols", C.c_size_t),
                ("n_out", C.c_int), ("d_out", C.c_void_p * 3), ("t_submit", C.c_double), ("t_start", C.c_double),
                ("t_done", C.c_double)]


class ServerStatsC(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("admitted", C.c_uint64), ("deferred", C.c_uint64),
                ("completed", C.c_uint64), ("failed", C.c_uint64), ("queued", C.c_size_t), ("running", C.c_size_t),
                ("bytes_in_use", C.c_size_t), ("memory_budget", C.c_size_t)]

_lib = None


def header_symbols() -> list[str]:
    """Every function the public header declares."""
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const char\*|vta_status|int|void\*|size_t|float|uint64_t)\s+(vta_\w+)\s*\(",
                                 text, re.M)))


def lib() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libvta_gb300.so not built ({LIB_PATH}); run vectorta_gb300.build.build()")
    L = C.CDLL(LIB_PATH)
    vp, sz, st = C.c_void_p, C.c_size_t, C.c_int
    fp = C.POINTER(C.c_float)
    L.vta_last_error.restype = C.c_char_p
    L.vta_last_error_oom.argtypes = [C.POINTER(sz)] * 3
    L.vta_last_error_oom.restype = st
    L.vta_version.restype = C.c_char_p
    L.vta_device_count.restype = C.c_int
    L.vta_ctx_create.argtypes = [C.c_int, C.POINTER(vp)]
    L.vta_ctx_destroy.argtypes = [vp]
    L.vta_ctx_synchronize.argtypes = [vp]
    L.vta_ctx_set_stream.argtypes = [vp, vp]
    L.vta_ctx_get_stream.argtypes = [vp]
    L.vta_ctx_get_stream.restype = vp
    L.vta_ctx_set_policy.argtypes = [vp, C.c_char_p, C.c_char_p]
    L.vta_ctx_last_kernel.argtypes = [vp]
    L.vta_ctx_last_kernel.restype = C.c_char_p
    L.vta_ctx_scratch_bytes.argtypes = [vp]
    L.vta_ctx_scratch_bytes.restype = sz
    L.vta_ctx_kernel_ms.argtypes = [vp]
    L.vta_ctx_kernel_ms.restype = C.c_float
    L.vta_launch_count.restype = C.c_uint64
    L.vta_device_array_free.argtypes = [C.POINTER(DeviceArrayC)]
    L.vta_device_array_copy_to_host.argtypes = [vp, C.POINTER(DeviceArrayC), fp, sz]
    L.vta_device_array_to_dlpack.argtypes = [C.POINTER(DeviceArrayC), C.c_int, C.POINTER(vp)]
    L.vta_dlpack_delete.argtypes = [vp, C.c_int]
    L.vta_ma_supported.argtypes = [C.c_char_p]
    L.vta_ma_supported.restype = C.c_int
    L.vta_ma_periods_device.argtypes = [vp, C.c_char_p, C.POINTER(C.c_char_p), C.POINTER(C.c_double), sz, vp, sz,
                                        sz, C.POINTER(C.c_int), sz, C.c_int, vp]
    L.vta_ma_select_dev.argtypes = [vp, C.c_char_p, C.POINTER(C.c_char_p), C.POINTER(C.c_double), sz, vp, sz, sz,
                                    sz, sz, C.POINTER(DeviceArrayC)]
    L.vta_streams_create.argtypes = [vp, C.c_char_p, C.POINTER(C.c_char_p), C.POINTER(C.c_double), sz, sz,
                                     C.POINTER(vp)]
    L.vta_streams_shape.argtypes = [vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]
    L.vta_streams_update_device.argtypes = [vp, vp, vp, vp, vp]
    L.vta_streams_update_host.argtypes = [vp, vp, vp, vp, vp]
    L.vta_streams_reset.argtypes = [vp]
    L.vta_streams_destroy.argtypes = [vp]
    L.vta_ma_select_into_host_f32.argtypes = [vp, C.c_char_p, C.POINTER(C.c_char_p), C.POINTER(C.c_double), sz,
                                              vp, sz, sz, sz, sz, vp, sz, C.POINTER(sz), C.POINTER(sz)]
    L.vta_pinned_alloc.argtypes = [sz, C.POINTER(vp)]
    L.vta_pinned_free.argtypes = [vp]
    L.vta_device_alloc.argtypes = [vp, sz, C.POINTER(vp)]
    L.vta_device_free.argtypes = [vp, vp]
    L.vta_memcpy_h2d.argtypes = [vp, vp, vp, sz]
    L.vta_memcpy_d2h.argtypes = [vp, vp, vp, sz]
    for name, (kind, outs, fam) in INDICATORS.items():
        R, P = C.POINTER(SWEEPS[fam]), C.POINTER(PARAMS[fam])
        nin, nout = N_IN[kind], len(outs)
        da = C.POINTER(DeviceArrayC)
        f = getattr(L, f"vta_{name}_expand_grid")
        f.argtypes = [R, P, sz, C.POINTER(sz)]
        getattr(L, f"vta_{name}_batch_dev").argtypes = [vp] + [vp] * nin + [sz, R] + [da] * nout
        getattr(L, f"vta_{name}_batch_device").argtypes = [vp] + [vp] * nin + [sz, sz, R] + [vp] * nout
        getattr(L, f"vta_{name}_batch_into_host_f32").argtypes = (
            [vp] + [vp] * nin + [sz, R] + [vp] * nout + [sz, C.POINTER(sz), C.POINTER(sz)])
        getattr(L, f"vta_{name}_many_series_one_param_time_major_dev").argtypes = (
            [vp] + [vp] * nin + [sz, sz, P] + [da] * nout)
        getattr(L, f"vta_{name}_many_series_one_param_device").argtypes = (
            [vp] + [vp] * nin + [sz, sz, P] + [vp] * nout)
        for suffix in ("expand_grid", "batch_dev", "batch_device", "batch_into_host_f32",
                       "many_series_one_param_time_major_dev", "many_series_one_param_device"):
            getattr(L, f"vta_{name}_{suffix}").restype = st
    L.vta_tm_plan_create.argtypes = [vp, vp, vp, vp, sz, sz, C.POINTER(sz), C.POINTER(TmJobC), sz, C.POINTER(vp)]
    L.vta_tm_plan_run.argtypes = [vp]
    L.vta_tm_plan_info_get.argtypes = [vp, C.POINTER(TmPlanInfoC)]
    L.vta_tm_plan_destroy.argtypes = [vp]
    for fn in ("vta_tm_plan_create", "vta_tm_plan_run", "vta_tm_plan_info_get", "vta_tm_plan_destroy"):
        getattr(L, fn).restype = st
    L.vta_server_create.argtypes = [C.c_int, C.POINTER(ServerConfigC), C.POINTER(vp)]
    L.vta_server_add_series.argtypes = [vp, vp, vp, vp, sz, C.POINTER(C.c_uint32)]
    L.vta_server_add_series_device.argtypes = [vp, vp, vp, vp, sz, C.POINTER(C.c_uint32)]
    L.vta_server_submit.argtypes = [vp, C.POINTER(RequestC), C.POINTER(C.c_uint64)]
    L.vta_server_poll.argtypes = [vp, C.POINTER(CompletionC), sz, C.POINTER(sz), C.c_int]
    L.vta_server_copy_out.argtypes = [vp, C.c_uint64, C.c_int, vp, sz]
    L.vta_server_release.argtypes = [vp, C.c_uint64]
    L.vta_server_get_stats.argtypes = [vp, C.POINTER(ServerStatsC)]
    L.vta_server_destroy.argtypes = [vp]
    for fn in ("vta_server_create", "vta_server_add_series", "vta_server_add_series_device", "vta_server_submit",
               "vta_server_poll", "vta_server_copy_out", "vta_server_release", "vta_server_get_stats",
               "vta_server_destroy"):
        getattr(L, fn).restype = st
    L.vta_sma_batch_device_noalloc.argtypes = [vp, vp, sz, sz, C.POINTER(SWEEPS["period"]), vp]
    L.vta_sma_batch_device_noalloc.restype = st
    for fn in ("vta_ctx_create", "vta_ctx_destroy", "vta_ctx_synchronize", "vta_ctx_set_stream",
               "vta_ctx_set_policy", "vta_device_array_free", "vta_device_array_copy_to_host",
               "vta_pinned_alloc", "vta_pinned_free", "vta_device_alloc", "vta_device_free",
               "vta_memcpy_h2d", "vta_memcpy_d2h"):
        getattr(L, fn).restype = st
    _lib = L
    return L


def check(status: int):
    if status != 0:
        L = lib()
        msg = L.vta_last_error()
        oom = None
        if status == 2:  # VTA_ERR_OUT_OF_MEMORY
            r, f, h = C.c_size_t(), C.c_size_t(), C.c_size_t()
            if L.vta_last_error_oom(C.byref(r), C.byref(f), C.byref(h)) == 0:
                oom = (r.value, f.value, h.value)
        raise VtaError(status, msg.decode() if msg else "", oom)

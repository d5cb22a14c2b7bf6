"""Benchmark of the GB300 indicator hot path.

Default workload (the recurrence and window sweeps): one close series of
1,000,000 bars (geometric random walk, seed 1, first 200 NaN) and
high/low = close * (1 +- |N(0, 0.005^2)|); one step computes
  EMA, DEMA, TEMA, RSI           periods 2..1000 step 1 (999 combos each)
  SMA, StdDev, Z-score           windows 5..500 step 5 (100 combos each)
  Donchian (3 bands), Williams %R windows 5..500 step 5
= 4.696e9 f32 outputs (18.8 GB written per step, which also flushes L2).
`--workload alma_grid` runs the ALMA grid instead (200,000 bars, seed 2,
periods 5..260 x offsets 0.50..0.95/0.05 x sigmas 3..9 = 17,920 combos).

Metric: indicator outputs per second (higher is better).
  value: inputs resident in HBM, outputs into preallocated device buffers,
         through the crate-facing *_batch_device C-ABI calls; CUDA events on
         the calls' stream around exactly K steps.
  e2e:   the *_batch_into_host_f32 C-ABI calls from pinned host inputs to
         pinned host outputs (H2D + kernels + D2H of every output).
  calls: each indicator's whole call (every kernel and the gaps between
         them) timed with CUDA events; roofline.call_frac is the dominant
         indicator's algorithmic bytes over its whole call.
  err:   outside every timed region, in the CPU-baseline leg: max abs / rel
         error of the device outputs against the oracle over every bar of
         sampled rows (every row of the 100-combo windows, every 10th of the
         999-combo recurrences); StdDev / Z-score also against the exact
         window statistics.
The default run adds two more figures, each with its own clock record:
`alma_grid` (the 17,920-combo ALMA grid, roofline and error) and
`served_stream` (Poisson 2,000 req/s for --duration = 60 s over the
10,000-series store: p50/p99 latency, capacity, plain per-request ratio).
`--impl reference` times the CPU reference restatement (oracle, all host
threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# measured peaks of this GPU pool (HBM copy GB/s); fallback 6800 if absent
_FALLBACK_HBM = 6800.0


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return _FALLBACK_HBM, "fallback"


# ------------------------------------------------------------- workloads ----
def _dist():
    """torch.distributed when a process group is up (torchrun, N > 1), else None."""
    try:
        import torch.distributed as dist
    except Exception:
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def barrier():
    """All ranks meet here (no-op on one rank)."""
    d = _dist()
    if d is not None:
        d.barrier()


def rank_max(x: float) -> float:
    """Maximum of x over the ranks (x itself on one rank)."""
    d = _dist()
    if d is None:
        return float(x)
    import torch

    dev = "cuda" if d.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def combine_ranks(res: dict, world: int) -> dict:
    """Whole-job figures of N replicas: the slowest rank's step time, and the
    outputs of all ranks over it."""
    res["ms_per_step"] = rank_max(res["ms_per_step"])
    res["value"] = res["outputs_per_step"] * world / (res["ms_per_step"] / 1e3)
    return res


def workload_sweeps():
    from vectorta_gb300 import datagen

    n = 1_000_000
    close = datagen.random_walk(n, seed=1, nan_lead=200)
    hi, lo = datagen.high_low(close, seed=1)
    hi[:200] = np.nan
    lo[:200] = np.nan
    series = {"close": close.astype(np.float32), "high": hi.astype(np.float32), "low": lo.astype(np.float32)}
    rec = {"period": (2, 1000, 1)}
    win = {"period": (5, 500, 5)}
    jobs = [
        ("ema", ["close"], rec), ("dema", ["close"], rec), ("tema", ["close"], rec), ("rsi", ["close"], rec),
        ("sma", ["close"], win), ("stddev", ["close"], {"period": (5, 500, 5), "nbdev": (1.0, 1.0, 0.0)}),
        ("zscore", ["close"], {"period": (5, 500, 5), "nbdev": (1.0, 1.0, 0.0)}),
        ("donchian", ["high", "low"], win), ("willr", ["high", "low", "close"], win),
    ]
    return {"name": "recurrence_window_sweeps", "n": n, "series": series, "jobs": jobs, "dominant": "ema",
            "config": {"workload": "recurrence_window_sweeps", "bars": n, "nan_lead": 200, "seed": 1,
                       "recurrences": "EMA/DEMA/TEMA/RSI periods 2..1000 (999 each)",
                       "windows": "SMA/StdDev/Zscore/Donchian/WillR 5..500 step 5 (100 each)"}}


def workload_alma_grid():
    from vectorta_gb300 import datagen

    n = 200_000
    close = datagen.random_walk(n, seed=2)
    sweep = {"period": (5, 260, 1), "offset": (0.50, 0.95, 0.05), "sigma": (3.0, 9.0, 1.0)}
    return {"name": "alma_grid", "n": n, "series": {"close": close.astype(np.float32)},
            "jobs": [("alma", ["close"], sweep)], "dominant": "alma",
            "config": {"workload": "alma_grid", "bars": n, "seed": 2, "combos": 17920,
                       "sweep": "periods 5..260 x offsets 0.50..0.95/0.05 x sigmas 3..9"}}


def workload_wwma_family():
    """The remaining weighted-window moving averages on the tensor-core
    contraction: CWMA, FWMA, SRWMA, SQWMA, VPWMA (power 0.382) periods 5..260
    (256 combos each) and EPMA periods 16..260 x offset 4 (245 combos) on
    1,000,000 bars (seed 6, 100 leading NaN): 1.525e9 outputs = 6.1 GB per
    step."""
    from vectorta_gb300 import datagen

    n = 1_000_000
    close = datagen.random_walk(n, seed=6, nan_lead=100)
    per = {"period": (5, 260, 1)}
    jobs = [("cwma", ["close"], per), ("fwma", ["close"], per), ("srwma", ["close"], per),
            ("sqwma", ["close"], per), ("vpwma", ["close"], {"period": (5, 260, 1), "power": (0.382, 0.382, 0.0)}),
            ("epma", ["close"], {"period": (16, 260, 1), "offset": (4, 4, 0)})]
    return {"name": "wwma_family", "n": n, "series": {"close": close.astype(np.float32)}, "jobs": jobs,
            "dominant": "cwma",
            "config": {"workload": "wwma_family", "bars": n, "seed": 6, "nan_lead": 100,
                       "sweeps": "CWMA/FWMA/SRWMA/SQWMA/VPWMA periods 5..260; EPMA periods 16..260 x offset 4"}}


def workload_wma_long():
    """Long weighted windows on the tensor cores: WMA periods 2..1000 (999
    combos, tiles of K up to 1008, run as 256-wide K slices) on 1,000,000 bars
    (seed 7): 4.0 GB of outputs per step."""
    from vectorta_gb300 import datagen

    n = 1_000_000
    close = datagen.random_walk(n, seed=7, nan_lead=10)
    return {"name": "wma_long", "n": n, "series": {"close": close.astype(np.float32)},
            "jobs": [("wma", ["close"], {"period": (2, 1000, 1)})], "dominant": "wma",
            "config": {"workload": "wma_long", "bars": n, "seed": 7, "nan_lead": 10, "combos": 999,
                       "sweep": "WMA periods 2..1000"}}


def workload_ema_small():
    """Profiling case: one EMA sweep (periods 2..1000) on 200,000 bars
    (0.8 GB of outputs: larger than L2, a few GB on the device at most)."""
    from vectorta_gb300 import datagen

    n = 200_000
    close = datagen.random_walk(n, seed=1, nan_lead=200)
    return {"name": "ema_small", "n": n, "series": {"close": close.astype(np.float32)},
            "jobs": [("ema", ["close"], {"period": (2, 1000, 1)})], "dominant": "ema",
            "config": {"workload": "ema_small", "bars": n, "seed": 1, "combos": 999}}


def workload_recur_small():
    """Profiling case of the chunked recurrences: EMA, DEMA and RSI sweeps
    (periods 2..1000, 999 combos) on 400,000 bars (1.6 GB of outputs per
    call)."""
    from vectorta_gb300 import datagen

    n = 400_000
    close = datagen.random_walk(n, seed=1, nan_lead=200)
    rec = {"period": (2, 1000, 1)}
    return {"name": "recur_small", "n": n, "series": {"close": close.astype(np.float32)},
            "jobs": [("ema", ["close"], rec), ("dema", ["close"], rec), ("rsi", ["close"], rec)], "dominant": "ema",
            "config": {"workload": "recur_small", "bars": n, "seed": 1, "combos": 999}}


def workload_tema_small():
    """Profiling case of the tensor-core chunk aggregates and the carry scan
    with a three-component state: one TEMA sweep (periods 2..1000, 999
    combos) on 200,000 bars (0.8 GB of outputs per call)."""
    from vectorta_gb300 import datagen

    n = 200_000
    close = datagen.random_walk(n, seed=1, nan_lead=200)
    return {"name": "tema_small", "n": n, "series": {"close": close.astype(np.float32)},
            "jobs": [("tema", ["close"], {"period": (2, 1000, 1)})], "dominant": "tema",
            "config": {"workload": "tema_small", "bars": n, "seed": 1, "combos": 999}}


def workload_percentile_small():
    """Profiling case of the batch percentile: window lengths 10..64 step 2 x
    percentages 25/50/75 (84 combos) on 200,000 bars."""
    from vectorta_gb300 import datagen

    n = 200_000
    close = datagen.random_walk(n, seed=1, nan_lead=50)
    return {"name": "percentile_small", "n": n, "series": {"close": close.astype(np.float32)},
            "jobs": [("percentile_nearest_rank", ["close"], {"length": (10, 64, 2), "percentage": (25.0, 75.0, 25.0)})],
            "dominant": "percentile_nearest_rank",
            "config": {"workload": "percentile_small", "bars": n, "seed": 1, "combos": 84}}


def workload_windows_small():
    """Profiling case of the window kernels: StdDev and WillR sweeps (windows
    5..500 step 5, 100 combos) on 400,000 bars (160 MB of outputs per call:
    larger than L2)."""
    from vectorta_gb300 import datagen

    n = 400_000
    close = datagen.random_walk(n, seed=1, nan_lead=200)
    hi, lo = datagen.high_low(close, seed=1)
    series = {"close": close.astype(np.float32), "high": hi.astype(np.float32), "low": lo.astype(np.float32)}
    jobs = [("stddev", ["close"], {"period": (5, 500, 5), "nbdev": (1.0, 1.0, 0.0)}),
            ("willr", ["high", "low", "close"], {"period": (5, 500, 5)})]
    return {"name": "windows_small", "n": n, "series": series, "jobs": jobs, "dominant": "stddev",
            "config": {"workload": "windows_small", "bars": n, "seed": 1, "combos": 100}}


def workload_adx_sweep():
    """ADX sweep, periods 2..400 (399 combos) on 1,000,000 OHLC bars (seed 3,
    NaN lead 100): the single-series ADX path (time-chunked, verified warm
    restarts)."""
    from vectorta_gb300 import datagen

    n = 1_000_000
    d = datagen.ohlcv(n, seed=3, nan_lead=100)
    series = {k: d[k].astype(np.float32) for k in ("high", "low", "close")}
    return {"name": "adx_sweep", "n": n, "series": series,
            "jobs": [("adx", ["high", "low", "close"], {"period": (2, 400, 1)})], "dominant": "adx",
            "config": {"workload": "adx_sweep", "bars": n, "seed": 3, "nan_lead": 100, "combos": 399}}


def workload_ragged_small():
    """Profiling case of the many-series plan: 1,024 series of length
    U[1000, 20000] (seed 4), the four jobs of ragged_tm."""
    wl = workload_ragged_tm(n_series=1024, max_len=20000)
    wl["name"] = "ragged_small"
    wl["config"] = dict(wl["config"], workload="ragged_small_plan", series=1024, lengths="U[1000, 20000]")
    return wl


def workload_alma_small():
    """Profiling case: the 17,920-combo ALMA grid on 20,000 bars (1.4 GB of
    outputs: larger than L2, a few GB on the device at most)."""
    w = workload_alma_grid()
    from vectorta_gb300 import datagen

    n = 20_000
    w.update(name="alma_small", n=n, series={"close": datagen.random_walk(n, seed=2).astype(np.float32)})
    w["config"] = dict(w["config"], workload="alma_small", bars=n)
    return w


def workload_ragged_tm(n_series=4096, max_len=50000):
    """4,096 OHLCV series of uneven length (U[1000, 50000]) and NaN lead
    (U[0, 500]), time-major and padded with NaN, through one many-series plan
    running ATR(14), ADX(14), SuperTrend(10, 3.0) and percentile(50, 50%)."""
    from vectorta_gb300 import datagen

    d, lens, leads = datagen.ragged_many_series(n_series, seed=4, max_len=max_len, fields=("high", "low", "close"))
    jobs = [("atr", 14, 0.0, 1), ("adx", 14, 0.0, 1), ("supertrend", 10, 3.0, 2),
            ("percentile_nearest_rank", 50, 50.0, 1)]
    return {"name": "ragged_tm", "kind": "plan", "tm": d, "lens": lens, "plan_jobs": jobs,
            "config": {"workload": "ragged_many_series_plan", "series": 4096, "rows": int(d["close"].shape[0]),
                       "lengths": "U[1000, 50000]", "nan_lead": "U[0, 500]", "sum_lengths": int(lens.sum()),
                       "seed": 4, "indicators": "ATR(14), ADX(14), SuperTrend(10, 3.0), percentile(50, 50%)",
                       "layout": "time-major f32, NaN tail past each series (not read, not written)"}}


def workload_served_stream():
    """10,000 OHLC series (lengths log-uniform 1e3..1e6, NaN lead U[0, 500])
    resident on the device; requests arrive as a Poisson stream (2,000/s), each
    an indicator from {ALMA, EMA, RSI, ADX, Bollinger(20-style grid, 2.0)} over
    a random stored series with a sweep of log-uniform 1..4,096 combos drawn
    from the grids of the other workloads (capped at each grid's size)."""
    return {"name": "served_stream", "kind": "server",
            "config": {"workload": "served_mixed_stream", "series": 10000, "lengths": "log-uniform 1e3..1e6",
                       "nan_lead": "U[0, 500]", "arrivals": "Poisson 2000 req/s", "seed": 5,
                       "indicators": "alma, ema, rsi, adx, bollinger_bands (uniform)",
                       "sweep_size": "log-uniform 1..4096 combos, capped at the grid"}}


WORKLOADS = {"sweeps": workload_sweeps, "ragged_tm": workload_ragged_tm, "served_stream": workload_served_stream,
             "adx_sweep": workload_adx_sweep, "wwma_family": workload_wwma_family, "ragged_small": workload_ragged_small, "alma_grid": workload_alma_grid, "ema_small": workload_ema_small,
             "alma_small": workload_alma_small, "windows_small": workload_windows_small,
             "recur_small": workload_recur_small, "wma_long": workload_wma_long, "tema_small": workload_tema_small,
             "percentile_small": workload_percentile_small}


# ------------------------------------------------------------- clocks -------
class ClockSampler:
    """SM clocks and clock-event (throttle) reasons sampled while the timed
    region runs: NVML read-only queries every 10 ms through ctypes, or
    `nvidia-smi -lms 200` when NVML cannot be loaded."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    # NVML clock-event reason bits
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8, "sw_thermal_slowdown": 0x20, "hw_thermal_slowdown": 0x40}

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.lines = []
        self.samples = []  # (sm_mhz, max_mhz, reason bits)
        self._nvml = None
        self._stop = threading.Event()

    def _nvml_open(self):
        import ctypes as C
        lib = C.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            return None
        h = C.c_void_p()
        ok = False
        try:
            import torch
            pr = torch.cuda.get_device_properties(self.device)
            bus = f"{pr.pci_domain_id:08X}:{pr.pci_bus_id:02X}:{pr.pci_device_id:02X}.0".encode()
            ok = lib.nvmlDeviceGetHandleByPciBusId_v2(C.c_char_p(bus), C.byref(h)) == 0
        except Exception:
            ok = False
        if not ok and lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.device), C.byref(h)) != 0:
            return None
        reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            getattr(lib, "nvmlDeviceGetCurrentClocksThrottleReasons")
        return lib, h, reasons

    def _nvml_loop(self):
        import ctypes as C
        lib, h, reasons = self._nvml
        sm, mx, rb = C.c_uint(), C.c_uint(), C.c_ulonglong()
        while not self._stop.is_set():
            if (lib.nvmlDeviceGetClockInfo(h, 1, C.byref(sm)) == 0 and
                    lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx)) == 0 and reasons(h, C.byref(rb)) == 0):
                self.samples.append((float(sm.value), float(mx.value), int(rb.value)))
            self._stop.wait(0.01)

    def __enter__(self):
        try:
            self._nvml = self._nvml_open()
        except Exception:
            self._nvml = None
        if self._nvml:
            self._t = threading.Thread(target=self._nvml_loop, daemon=True)
            self._t.start()
            return self
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        self._stop.set()
        if self._nvml:
            self._t.join(timeout=2)
            try:
                self._nvml[0].nvmlShutdown()
            except Exception:
                pass
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        for s_mhz, m_mhz, bits in self.samples:
            sm.append(s_mhz)
            mx.append(m_mhz)
            reasons.update(nm for nm, b in self.BITS.items() if bits & b)
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm), "source": "nvml" if self.samples else "nvidia-smi"}


# ------------------------------------------------------------- CPU side -----
def cpu_sample(wl, budget_rows=None):
    """Bounded sample of the workload for the CPU reference: every k-th combo
    of each sweep over the full series.  Returns a list of (callable, outputs)."""
    from oracle import oracle as O

    s = {k: v.astype(np.float64) for k, v in wl["series"].items()}
    tasks = []
    for name, ins, sweep in wl["jobs"]:
        if name == "alma":
            ps = O.axis_usize(sweep["period"])[::16]
            for p in ps:
                tasks.append((lambda p=p: O.alma_batch(s["close"], (p, p, 0), sweep["offset"], sweep["sigma"]),
                              wl["n"] * len(O.axis_f64(sweep["offset"])) * len(O.axis_f64(sweep["sigma"]))))
            continue
        if name in ("cwma", "fwma", "srwma", "sqwma", "epma", "vpwma", "wma"):
            fn = getattr(O, name)
            offs = (O.axis_usize(sweep["offset"], O.AX_SWAP) if name == "epma" else
                    O.axis_f64(sweep["power"]) if name == "vpwma" else [None])
            for p in O.periods_of(name, sweep["period"])[::16]:
                for o in offs:
                    args_ = (p,) if o is None else (p, o)
                    tasks.append((lambda fn=fn, a=args_: fn(s["close"], *a), wl["n"]))
            continue
        ps = O.periods_of(name, sweep["period"])
        stride = 4 if len(ps) > 500 else 1
        for p in ps[::stride]:
            if name in ("ema", "dema", "tema"):
                fn = {"ema": O.ema, "dema": O.dema, "tema": O.tema}[name]
                tasks.append((lambda fn=fn, p=p: fn(s["close"], p), wl["n"]))
            elif name == "rsi":
                tasks.append((lambda p=p: O.rsi_batch(s["close"], [p]), wl["n"]))
            elif name == "sma":
                tasks.append((lambda p=p: O.sma_batch(s["close"], [p]), wl["n"]))
            elif name == "stddev":
                tasks.append((lambda p=p: O.stddev(s["close"], p, 1.0), wl["n"]))
            elif name == "zscore":
                tasks.append((lambda p=p: O.zscore_batch_row(s["close"], p, 1.0), wl["n"]))
            elif name == "donchian":
                tasks.append((lambda p=p: O.donchian(s["high"], s["low"], p, fast=True), 3 * wl["n"]))
            elif name == "willr":
                tasks.append((lambda p=p: O.willr(s["high"], s["low"], s["close"], p, fast=True), wl["n"]))
            elif name == "adx":
                tasks.append((lambda p=p: O.adx(s["high"], s["low"], s["close"], p), wl["n"]))
    return tasks


def sample_desc(wl, tasks, outs, dt, threads):
    kind = wl.get("kind")
    what = (f"{len(tasks) // 4} of the workload's series (every 64th) x its 4 indicators" if kind == "plan" else
            f"the first {len(tasks)} requests of the stream, first combo of each sweep" if kind == "server" else
            f"{len(tasks)} rows of the workload's sweeps over the full series")
    took = f", {dt:.1f} s" if dt is not None else " per step"
    return f"{what} ({outs:.3g} outputs{took}), C oracle, {threads} threads"


def run_cpu(tasks, threads):
    from concurrent.futures import ThreadPoolExecutor

    t0 = time.perf_counter()
    if threads <= 1:
        for fn, _ in tasks:
            fn()
    else:
        with ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda t: t[0](), tasks))
    dt = time.perf_counter() - t0
    outs = sum(o for _, o in tasks)
    return outs / dt, dt, outs


# ------------------------------------------------------------- GPU side -----
def gpu_bench(args, wl):
    import torch

    from vectorta_gb300 import cuda as V

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ctx = V.Context(0)
    # one dedicated stream for torch's work, the library's calls and the
    # events (torch's default stream is the legacy NULL stream, which a
    # context given handle 0 would replace with a stream of its own)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_policy("timing", "on")
    ctx.set_policy("tune", args.tune)
    ctx.set_policy("recur_agg", args.recur_agg)
    inds = {name: V.CLASSES[name](0, ctx=ctx) for name, _, _ in wl["jobs"]}
    d_series = {k: torch.from_numpy(v).to(dev) for k, v in wl["series"].items()}
    firsts = {}
    for name, ins, _ in wl["jobs"]:
        arr = np.stack([wl["series"][k] for k in ins])
        firsts[name] = int(np.argmax(~np.isnan(arr).any(axis=0)))
    n = wl["n"]
    outs, rows = {}, {}
    for name, ins, sweep in wl["jobs"]:
        r = len(inds[name].expand_grid(sweep))  # the library's own grid expansion
        rows[name] = r
        nout = len(V.N.INDICATORS[name][1])
        outs[name] = [torch.empty((r, n), dtype=torch.float32, device=dev) for _ in range(nout)]
    out_per_step = sum(rows[nm] * n * len(outs[nm]) for nm in rows)

    kernel_ms = {nm: [] for nm in rows}
    call_ev = {nm: [] for nm in rows}
    kernel_names = {}

    # The device entry points return once their work is queued (like the
    # crate's x_batch_device), so the timed steps run back to back on the
    # stream with no host wait between calls.
    def step(record=False):
        for name, ins, sweep in wl["jobs"]:
            if record:
                ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                ev[0].record(stream)
            inds[name].batch_device([d_series[k] for k in ins], n, firsts[name], sweep, outs[name])
            if not record:  # (warm-up steps) the path each call took
                kernel_names[name] = ctx.last_kernel
            if record:
                ev[1].record(stream)
                call_ev[name].append(ev)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    launches0 = V.launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        torch.cuda.synchronize()
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            step(record=True)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    launches = V.launch_count() - launches0
    ms = e0.elapsed_time(e1)
    ms_per_step = ms / args.steps
    value = out_per_step / (ms_per_step / 1e3)
    # the dominant kernel of each call (the library's events around it): one
    # call at a time after the timed steps, each read once its call is done
    for _ in range(min(args.steps, 5)):
        for name, ins, sweep in wl["jobs"]:
            inds[name].batch_device([d_series[k] for k in ins], n, firsts[name], sweep, outs[name])
            ctx.synchronize()
            kernel_ms[name].append(ctx.kernel_ms)

    # roofline of the dominant kernel: algorithmic bytes per launch / event-timed duration
    dom = wl["dominant"]
    dom_ms = float(np.mean([x for x in kernel_ms[dom] if x > 0]))
    in_bytes = sum(wl["series"][k].nbytes for k in dict((j[0], j[1]) for j in wl["jobs"])[dom])
    dom_bytes = rows[dom] * n * 4 * len(outs[dom]) + in_bytes
    hbm, src = peaks()
    achieved = dom_bytes / (dom_ms / 1e3) / 1e9
    share = {nm: float(np.mean(v)) for nm, v in kernel_ms.items()}
    # whole calls (every kernel of the call and the gaps between them), CUDA
    # events on the calls' stream around each call of the timed steps
    call_ms = {nm: float(np.mean([a.elapsed_time(b) for a, b in v])) for nm, v in call_ev.items()}
    calls = {}
    for name, ins, _ in wl["jobs"]:
        b = rows[name] * n * 4 * len(outs[name]) + sum(wl["series"][k].nbytes for k in ins)
        calls[name] = {"call_ms": call_ms[name], "kernel_ms": share[name], "bytes": b,
                       "call_frac": b / (call_ms[name] / 1e3) / 1e9 / hbm, "kernel": kernel_names.get(name)}

    # e2e through the host-in / host-out C-ABI calls, pinned host buffers
    e2e = None
    if not args.no_e2e:
        e2e = e2e_bench(args, wl, inds, rows, out_per_step)
    return {
        "value": value, "ms_per_step": ms_per_step, "gpu_launches": int(launches), "clocks": clk.summary(),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": TRAFFIC.get(wl["name"]),
                     "kernel": KERNEL_NAME.get(wl["name"]), "peak_source": src,
                     "bytes_per_launch": dom_bytes, "ms_per_launch": dom_ms,
                     "call_ms": call_ms[dom], "call_frac": calls[dom]["call_frac"]},
        "kernel_ms_per_call": share, "calls": calls, "outputs_per_step": out_per_step, "e2e": e2e,
        "_state": {"inds": inds, "outs": outs, "rows": rows},
    }


PLAN_BYTES = {"atr": 16, "adx": 16, "supertrend": 20, "percentile_nearest_rank": 8}  # per (series, row)
PLAIN_PARAMS = {"atr": {"period": 14}, "adx": {"period": 14}, "supertrend": {"period": 10, "factor": 3.0},
                "percentile_nearest_rank": {"length": 50, "percentage": 50.0}}


def gpu_bench_plan(args, wl):
    """Many-series plan: every step replays the plan's graph over all series.
    Beside it, the plain per-request path: the four many-series entry points
    one after another over the same padded matrix."""
    import torch

    from vectorta_gb300 import cuda as V

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ctx = V.Context(0)
    stream = torch.cuda.Stream(device=dev)  # as in gpu_bench: one dedicated stream
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_policy("timing", "on")
    tm, lens = wl["tm"], wl["lens"]
    rows, cols = tm["close"].shape
    d_in = [torch.from_numpy(tm[k]).to(dev) for k in ("high", "low", "close")]
    outs, jobs = [], []
    for kind, p, prm, nout in wl["plan_jobs"]:
        o = [torch.empty(rows, cols, device=dev) for _ in range(nout)]
        outs.append(o)
        jobs.append({"kind": kind, "period": p, "param": prm, "out0": o[0], "out1": o[1] if nout > 1 else None})
    t0 = time.perf_counter()
    plan = V.TmPlan(*d_in, cols, rows, lens, jobs, ctx=ctx)
    create_s = time.perf_counter() - t0
    sum_len = int(lens.sum())
    out_per_step = sum_len * sum(j[3] for j in wl["plan_jobs"])
    for _ in range(args.warmup):
        plan.run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    graph_ms = []
    with ClockSampler(0) as clk:
        barrier()
        e0.record(stream)
        for _ in range(args.steps):
            plan.run()
            graph_ms.append(ctx.kernel_ms)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    ms = e0.elapsed_time(e1) / args.steps
    info = plan.info()
    g_ms = float(np.median(graph_ms))
    alg = sum_len * sum(PLAN_BYTES[j[0]] for j in wl["plan_jobs"])
    hbm, src = peaks()

    # plain per-request path: one many-series call per indicator, padded matrix,
    # with the plain sequential kernels (policy recur_chunk=sequential)
    pctx = V.Context(0)
    pctx.set_stream(stream.cuda_stream)
    pctx.set_policy("recur_chunk", "sequential")
    inds = {k: V.CLASSES[k](0, ctx=pctx) for k in PLAIN_PARAMS}
    p_out = {k: [torch.empty(rows, cols, device=dev) for _ in range(2 if k == "supertrend" else 1)]
             for k in PLAIN_PARAMS}

    def plain_step():
        for k, ind in inds.items():
            ins = [d_in[2]] if k == "percentile_nearest_rank" else d_in
            ind.many_series_one_param_device(ins, cols, rows, PLAIN_PARAMS[k], p_out[k])

    for _ in range(max(1, args.warmup)):
        plain_step()
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        plain_step()
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1) / args.steps

    e2e = None
    if not args.no_e2e:
        h_in = [torch.from_numpy(tm[k]).pin_memory() for k in ("high", "low", "close")]
        h_out = [torch.empty(rows, cols).pin_memory() for o in outs for _ in o]
        d_out = [t for o in outs for t in o]
        plan.run()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for d, h in zip(d_in, h_in):
                d.copy_(h, non_blocking=True)
            plan.run()
            for h, d in zip(h_out, d_out):
                h.copy_(d, non_blocking=True)
            torch.cuda.synchronize()
        dt = (time.perf_counter() - t0) / args.steps
        e2e = {"value": out_per_step / dt, "unit": "outputs/s", "ms_per_step": dt * 1e3,
               "h2d_bytes_per_step": int(sum(t.numel() * 4 for t in h_in)),
               "d2h_bytes_per_step": int(sum(t.numel() * 4 for t in h_out)), "steps": args.steps}
    plan.close()
    return {
        "value": out_per_step / (ms / 1e3), "ms_per_step": ms, "gpu_launches": 3 * args.steps,
        "clocks": clk.summary(),
        "roofline": {"bound": "hbm", "achieved": alg / (g_ms / 1e3) / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": alg / (g_ms / 1e3) / 1e9 / hbm, "traffic": TRAFFIC.get(wl["name"]),
                     "kernel": "tm plan graph (k_plan_first + k_tm_plan + k_tm_fixup)", "peak_source": src,
                     "bytes_per_launch": alg, "ms_per_launch": g_ms},
        "kernel_ms_per_call": {"plan_graph": g_ms}, "outputs_per_step": out_per_step, "e2e": e2e,
        "plan": {"create_s": create_s, "tuned": info["tuned"], "chunk": info["chunk"][:len(jobs)],
                 "n_items": info["n_items"], "fixups_last_run": info["fixups"]},
        "plain_per_request": {"ms_per_step": plain_ms, "value": out_per_step / (plain_ms / 1e3),
                              "note": "ATR/ADX/SuperTrend/percentile many-series entry points, one call each, "
                                      "over the padded matrix, plain sequential kernels"},
    }


SERVED_INDS = ["alma", "ema", "rsi", "adx", "bollinger_bands"]
N_OUT = {"alma": 1, "ema": 1, "rsi": 1, "adx": 1, "bollinger_bands": 3}


def stream_store(n_series=10000, seed=5):
    """Lengths (log-uniform 1e3..1e6), NaN leads (U[0, 500]) and generator
    seeds of the served stream's store."""
    from vectorta_gb300 import datagen

    lens = np.floor(1000.0 * 1000.0 ** datagen.uniform(seed, 20, n_series)).astype(np.int64)
    leads = np.floor(datagen.uniform(seed, 21, n_series) * 501).astype(np.int64)
    seeds = [seed * 100003 + i for i in range(n_series)]
    return lens, leads, seeds


def served_sweep(name, n, valid):
    """Sweep of about n combos of indicator `name` from the other workloads' grids,
    capped at the grid size and at what a series with `valid` bars allows."""
    if name == "alma":
        npd = max(1, min(256, n))
        rem = -(-n // npd)
        no = min(10, rem)
        ns = min(7, -(-rem // no))
        return {"period": (5, 5 + npd - 1, 1), "offset": (0.5, 0.5 + 0.05 * (no - 1), 0.05),
                "sigma": (3.0, 3.0 + (ns - 1), 1.0)}, npd * no * ns
    if name in ("ema", "rsi"):
        m = max(1, min(n, 999, valid - 2))
        return {"period": (2, 1 + m, 1)}, m
    if name == "adx":
        m = max(1, min(n, valid // 2 - 2))
        return {"period": (2, 1 + m, 1)}, m
    m = max(1, min(n, 100, valid // 5))
    return {"period": (5, 5 * m, 5), "devup": (2.0, 2.0, 0.0), "devdn": (2.0, 2.0, 0.0)}, m


def served_requests(duration, rate=2000.0, seed=5, n_series=10000, lens=None, leads=None):
    rng = np.random.default_rng(seed)
    n = int(rate * duration)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    ind = rng.integers(0, len(SERVED_INDS), n)
    ser = rng.integers(0, n_series, n)
    size = np.floor(np.exp(rng.uniform(0.0, np.log(4096.0), n))).astype(np.int64)
    reqs = []
    for i in range(n):
        name = SERVED_INDS[ind[i]]
        valid = int(lens[ser[i]] - leads[ser[i]])
        sw, rows = served_sweep(name, int(size[i]), valid)
        reqs.append({"t": float(t[i]), "name": name, "series": int(ser[i]), "sweep": sw, "rows": rows,
                     "outputs": rows * int(lens[ser[i]]) * N_OUT[name]})
    return reqs


def gpu_bench_server(args, wl):
    """Three runs over one request mix: Poisson-paced (latency), backlogged
    (capacity) and the plain per-request kernels one at a time."""
    import threading

    import torch

    from vectorta_gb300 import cuda as V
    from vectorta_gb300 import datagen

    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    lens, leads, seeds = stream_store()
    srv = V.Server(0, slots=args.slots)
    kept = []  # the generated device series (also used by the plain run)
    t0 = time.perf_counter()
    i = 0
    while i < len(lens):
        j, tot = i, 0
        while j < len(lens) and tot + lens[j] <= 200_000_000:
            tot += int(lens[j])
            j += 1
        j = max(j, i + 1)
        h, l, c, offs = datagen.ohlc_many_torch(lens[i:j], seeds[i:j], leads[i:j], device=dev)
        for q in range(j - i):
            o = int(offs[q]) * 4
            srv.add_series_device(c.data_ptr() + o, int(lens[i + q]), h.data_ptr() + o, l.data_ptr() + o)
        kept.append((i, j, h, l, c, offs))
        i = j
    store_s = time.perf_counter() - t0
    reqs = served_requests(args.duration, lens=lens, leads=leads)
    n_req = len(reqs)

    def run(batch, paced):
        lat, outs, times = [], 0, []
        pending = {}
        lock = threading.Lock()
        finished = threading.Event()

        failed = []

        def poller():
            got = 0
            while got < len(batch):
                for cpl in srv.poll(256, wait_ms=2):
                    with lock:
                        pending.pop(cpl["ticket"], None)
                    if cpl["status"] != 0:
                        failed.append(cpl["ticket"])
                    lat.append(cpl["t_done"] - cpl["t_submit"])
                    times.append((cpl["t_submit"], cpl["t_done"]))
                    srv.release(cpl["ticket"])
                    got += 1
            finished.set()

        th = threading.Thread(target=poller, daemon=True)
        th.start()
        base = time.perf_counter()
        for r in batch:
            if paced:
                delay = base + r["t"] - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
            with lock:
                tk = srv.submit(r["name"], r["series"], r["sweep"])
                pending[tk] = r
            outs += r["outputs"]
        if not finished.wait(timeout=900):
            raise RuntimeError("served stream: requests did not complete")
        if failed:
            raise RuntimeError(f"served stream: {len(failed)} requests failed")
        span = max(t for _, t in times) - min(t for t, _ in times)
        lat = np.array(lat)
        return {"requests": len(batch), "outputs": outs, "seconds": span, "outputs_per_s": outs / span,
                "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "max_ms": float(lat.max() * 1e3)}

    # warm-up: a few requests of every indicator (workspaces, module loading)
    run(reqs[: min(50, n_req)], paced=False)
    launches0 = V.launch_count()
    st0 = srv.stats()
    with ClockSampler(0) as clk:
        cap = run(reqs[: min(n_req, 4000)], paced=False)
    launches = V.launch_count() - launches0
    served = run(reqs, paced=True)
    st1 = srv.stats()

    # plain per-request kernels, one request at a time, on the same requests
    ctx = V.Context(0)
    ctx.set_policy("wma_batch", "plain")
    ctx.set_policy("recur_chunk", "sequential")
    inds = {k: V.CLASSES[k](0, ctx=ctx) for k in SERVED_INDS}

    def series_views(sid):
        for a, b, h, l, c, offs in kept:
            if a <= sid < b:
                o, n = int(offs[sid - a]), int(lens[sid])
                return h[o:o + n], l[o:o + n], c[o:o + n]

    sample = reqs[: min(n_req, 400)]
    p_out, p_t = 0, 0.0
    for r in sample:
        h, l, c = series_views(r["series"])
        ins = [h, l, c] if r["name"] == "adx" else [c]
        n = int(lens[r["series"]])
        outs_t = [torch.empty(r["rows"], n, device=dev) for _ in range(N_OUT[r["name"]])]
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        inds[r["name"]].batch_device(ins, n, int(leads[r["series"]]), r["sweep"], outs_t)
        inds[r["name"]].synchronize()
        p_t += time.perf_counter() - t1
        p_out += r["outputs"]
        del outs_t
    plain = {"requests": len(sample), "outputs_per_s": p_out / p_t, "seconds": p_t,
             "note": "the same requests one at a time through the plain FP32 kernels (wma_batch=plain, "
                     "recur_chunk=sequential)"}
    cap_bytes = cap["outputs"] * 4
    hbm, src = peaks()
    srv.close()
    return {
        "value": cap["outputs_per_s"], "ms_per_step": cap["seconds"] * 1e3 / cap["requests"],
        "gpu_launches": int(launches), "clocks": clk.summary(),
        "roofline": {"bound": "hbm", "achieved": cap_bytes / cap["seconds"] / 1e9, "peak": hbm, "unit": "GB/s",
                     "frac": cap_bytes / cap["seconds"] / 1e9 / hbm, "traffic": None,
                     "kernel": "all kernels of the backlogged run (output bytes / makespan)", "peak_source": src,
                     "bytes_per_launch": None, "ms_per_launch": None},
        "kernel_ms_per_call": {}, "outputs_per_step": cap["outputs"] / cap["requests"], "e2e": None,
        "served": dict(served, rate_req_s=2000.0, duration_s=args.duration,
                       admitted=st1["admitted"] - st0["admitted"], deferred=st1["deferred"] - st0["deferred"]),
        "capacity": cap, "plain_per_request": dict(plain, speedup=cap["outputs_per_s"] / plain["outputs_per_s"]),
        "store": {"series": int(len(lens)), "bars": int(lens.sum()), "build_s": store_s},
    }


def cpu_sample_server(wl, n=40):
    """The first n requests of the served stream, each reduced to the first
    combo of its sweep over its whole series, through the oracle."""
    from oracle import oracle as O
    from vectorta_gb300 import datagen

    lens, leads, seeds = stream_store()
    tasks = []
    for r in served_requests(1.0, lens=lens, leads=leads)[:n]:
        sid = r["series"]
        d = datagen.ohlcv(int(lens[sid]), seeds[sid], nan_lead=int(leads[sid]))
        h, l, c = d["high"], d["low"], d["close"]
        p = int(r["sweep"]["period"][0])
        L = int(lens[sid])
        if r["name"] == "alma":
            tasks.append((lambda c=c, p=p, o=r["sweep"]["offset"][0], sg=r["sweep"]["sigma"][0]: O.alma(c, p, o, sg), L))
        elif r["name"] == "ema":
            tasks.append((lambda c=c, p=p: O.ema(c, p), L))
        elif r["name"] == "rsi":
            tasks.append((lambda c=c, p=p: O.rsi_batch(c, [p]), L))
        elif r["name"] == "adx":
            tasks.append((lambda h=h, l=l, c=c, p=p: O.adx(h, l, c, p), L))
        else:
            tasks.append((lambda c=c, p=p: O.bollinger(c, p, 2.0, 2.0), 3 * L))
    return tasks


def cpu_tasks(wl):
    kind = wl.get("kind")
    return cpu_sample_plan(wl) if kind == "plan" else cpu_sample_server(wl) if kind == "server" else cpu_sample(wl)


def cpu_sample_plan(wl, every=64):
    """Every `every`-th series of the plan workload through the oracle."""
    from oracle import oracle as O

    tm, lens = wl["tm"], wl["lens"]
    tasks = []
    for s in range(0, tm["close"].shape[1], every):
        L = int(lens[s])
        h, l, c = (tm[k][:L, s].astype(np.float64) for k in ("high", "low", "close"))
        tasks.append((lambda h=h, l=l, c=c: O.atr(h, l, c, 14), L))
        tasks.append((lambda h=h, l=l, c=c: O.adx(h, l, c, 14), L))
        tasks.append((lambda h=h, l=l, c=c: O.supertrend(h, l, c, 10, 3.0), 2 * L))
        tasks.append((lambda c=c: O.percentile_nearest_rank(c, 50, 50.0), L))
    return tasks


def err_rows(name, n_rows):
    """Rows whose every bar is compared with the oracle: every row of the
    100-combo window sweeps, every 10th row (and the last) of the 999-combo
    recurrence sweeps, 64 rows spread over the ALMA grid."""
    if name == "alma":
        return sorted(set(np.linspace(0, n_rows - 1, 64).round().astype(int).tolist()))
    if n_rows <= 128:
        return list(range(n_rows))
    return sorted(set(range(0, n_rows, 10)) | {n_rows - 1})


def measure_err(wl, state):
    """Error of this run's device outputs against the oracle (CPU-baseline
    leg; outside every timed region).  Per indicator: max abs and rel error
    over every bar of the sampled rows (oracle/parity.py gives the
    definitions), and for StdDev / Z-score the same against the exact window
    statistics plus the crate's own drift from them."""
    from oracle import parity as P

    inds, outs, rows = state["inds"], state["outs"], state["rows"]
    res = {}
    for name, ins, sweep in wl["jobs"]:
        combos = [tuple(c.values()) for c in inds[name].expand_grid(sweep)]

        def fetch(r, name=name):
            return np.concatenate([o[r].cpu().numpy() for o in outs[name]])

        series = {k: wl["series"][k] for k in set(ins) | {"close"} if k in wl["series"]}
        t0 = time.perf_counter()
        res[name] = P.sweep_err(name, series, combos, fetch, err_rows(name, rows[name]))
        res[name]["seconds"] = time.perf_counter() - t0
    return res


def e2e_bench(args, wl, inds, rows, out_per_step):
    import ctypes as C

    import torch

    from vectorta_gb300 import _native as N

    L = N.lib()
    n = wl["n"]
    # pinned host inputs
    host_in = {}
    for k, v in wl["series"].items():
        p = C.c_void_p()
        N.check(L.vta_pinned_alloc(v.nbytes, C.byref(p)))
        a = np.ctypeslib.as_array((C.c_float * v.size).from_address(p.value))
        a[:] = v
        host_in[k] = (p, a)
    biggest = max(rows[nm] * n for nm in rows)
    nout_max = max(len(N.INDICATORS[nm][1]) for nm in rows)
    host_out = []
    for _ in range(nout_max):
        p = C.c_void_p()
        N.check(L.vta_pinned_alloc(biggest * 4, C.byref(p)))
        host_out.append(p)
    h2d = sum(sum(wl["series"][k].nbytes for k in ins) for _, ins, _ in wl["jobs"])
    d2h = out_per_step * 4

    def step():
        for name, ins, sweep in wl["jobs"]:
            ind = inds[name]
            nout = len(N.INDICATORS[name][1])
            import vectorta_gb300.cuda as V

            s = V._to_sweep(ind._fam, sweep)
            r, c = C.c_size_t(), C.c_size_t()
            N.check(ind._fn("batch_into_host_f32")(
                ind.ctx.handle, *[host_in[k][0].value for k in ins], n, C.byref(s),
                *[host_out[i].value for i in range(nout)], rows[name] * n, C.byref(r), C.byref(c)))

    steps = max(1, args.steps)
    step()  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / steps
    for p, _ in host_in.values():
        L.vta_pinned_free(p)
    for p in host_out:
        L.vta_pinned_free(p)
    return {"value": out_per_step / dt, "unit": "outputs/s", "h2d_bytes_per_step": int(h2d),
            "d2h_bytes_per_step": int(d2h), "ms_per_step": dt * 1e3, "steps": steps}


# DRAM bytes (read + write) per launch of the dominant kernel, from one ncu
# capture each of the EMA sweep on 200,000 bars and of the ALMA grid on 20,000
# bars (ema_small / alma_small).  Their per-launch bytes are scaled by the
# output count to the full workloads (x5 and x10): these kernels' traffic is
# linear in the outputs they write.
TRAFFIC = {
    "recurrence_window_sweeps": (5.659392e6 + 737.656320e6) * 5,
    "ema_small": 5.659392e6 + 737.656320e6,
    "alma_grid": (24.602112e6 + 1374.316e6) * 10,
    "alma_small": 24.602112e6 + 1374.316e6,
}
KERNEL_NAME = {"recurrence_window_sweeps": "k_recur<OpEma, batch, EMIT>", "alma_grid": "k_wwma_tc<fp16x3>",
               "ema_small": "k_recur<OpEma, batch, EMIT>", "alma_small": "k_wwma_tc<fp16x3>",
               "adx_sweep": "k_hlc_chunk<adx> + k_adx_scan passes + fix-up", "wwma_family": "k_wwma_tc<fp16x3> (CWMA)",
               "windows_small": "k_prefix_window_batch (StdDev)", "recur_small": "k_recur<OpEma, batch, EMIT>",
               "wma_long": "k_wwma_tc<fp16x3> (K slices)", "tema_small": "k_recur<OpTema, batch, EMIT>",
               "percentile_small": "k_percentile (register window)"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="sweeps", choices=sorted(WORKLOADS))
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--duration", type=float, default=60.0, help="served_stream: seconds of Poisson arrivals")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload: skip the ALMA-grid and served-stream figures")
    ap.add_argument("--no-err", action="store_true", help="skip the error measurement against the oracle")
    ap.add_argument("--tune", default="on", choices=["on", "off", "cached"],
                    help="batch-sweep autotuner policy (off: untuned defaults, e.g. for profiling)")
    ap.add_argument("--slots", type=int, default=8, help="served_stream: concurrent server slots")
    ap.add_argument("--recur-agg", default="auto", choices=["auto", "cuda", "tc"],
                    help="chunk aggregates of the EMA/DEMA/TEMA/RSI sweeps: tensor cores where eligible "
                         "(auto), CUDA cores only, or tensor cores required")
    args = ap.parse_args()

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    wl = WORKLOADS[args.workload]()
    cfg = dict(wl["config"], l2="each step writes >> 129 MB of outputs, flushing L2",
               parallelism="replicas" if world > 1 else "single GPU")
    base = {"metric": "indicator outputs/s at stated err vs FP64 oracle", "unit": "outputs/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded random walk)",
            "config": cfg}

    if args.impl == "reference":
        if rank != 0:
            return
        threads = os.cpu_count() or 1
        tasks = cpu_tasks(wl)
        run_cpu(tasks[: max(1, len(tasks) // 8)], threads)  # warm caches / page in
        vals = []
        for _ in range(max(1, args.warmup)):
            run_cpu(tasks, threads)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            v, dt, outs = run_cpu(tasks, threads)
            vals.append(v)
        wall = (time.perf_counter() - t0) / args.steps
        v = float(np.median(vals))
        line = dict(base, impl="reference", value=v, ms_per_step=wall * 1e3,
                    cpu_baseline={"value": v, "unit": "outputs/s", "cores": threads, "kind": "port",
                                  "sample": sample_desc(wl, tasks, outs, None, threads)},
                    e2e={"value": v, "unit": "outputs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
        print(json.dumps(line))
        return

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        import torch

        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    kind = wl.get("kind")
    res = (gpu_bench_plan(args, wl) if kind == "plan" else
           gpu_bench_server(args, wl) if kind == "server" else gpu_bench(args, wl))
    state = res.pop("_state", None)
    if world > 1:
        combine_ranks(res, world)
    if rank != 0:
        return
    cpu = None
    err = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        tasks = cpu_tasks(wl)
        v, dt, outs = run_cpu(tasks, threads)
        cpu = {"value": v, "unit": "outputs/s", "cores": threads, "kind": "port",
               "sample": sample_desc(wl, tasks, outs, dt, threads)}
        if state is not None and not args.no_err:
            err = measure_err(wl, state)
    state = None
    line = dict(base, value=res["value"], ms_per_step=res["ms_per_step"], gpu_launches=res["gpu_launches"],
                clocks=res["clocks"], roofline=res["roofline"], cpu_baseline=cpu, e2e=res["e2e"],
                kernel_ms_per_call=res["kernel_ms_per_call"], outputs_per_step=res["outputs_per_step"])
    if err is not None:
        line["err"] = err
    for k in ("calls", "plan", "plain_per_request", "served", "capacity", "store"):
        if k in res:
            line[k] = res[k]
    if args.workload == "sweeps" and world == 1 and not args.no_extras:
        line.update(extras(args))
    print(json.dumps(line))


def extras(args):
    """The two other headline figures of the default run, each measured as
    its own workload with its own clock record: the ALMA grid (17,920 combos x
    200,000 bars on the tensor-core contraction, with its error against the
    oracle) and the served mixed request stream (Poisson 2,000 req/s for
    --duration seconds, p50/p99 latency, against plain per-request kernels)."""
    import gc

    import torch

    out = {}
    gc.collect()
    torch.cuda.empty_cache()
    wl = workload_alma_grid()
    r = gpu_bench(args, wl)
    st = r.pop("_state")
    e = None if (args.no_cpu or args.no_err) else measure_err(wl, st)["alma"]
    st = None
    out["alma_grid"] = {"config": wl["config"], "value": r["value"], "unit": "outputs/s",
                        "ms_per_step": r["ms_per_step"], "roofline": r["roofline"], "clocks": r["clocks"],
                        "err": e, "e2e": r["e2e"], "gpu_launches": r["gpu_launches"]}
    r = None
    gc.collect()
    torch.cuda.empty_cache()
    wl = workload_served_stream()
    r = gpu_bench_server(args, wl)
    out["served_stream"] = {"config": dict(wl["config"], duration_s=args.duration), "clocks": r["clocks"],
                            "served": r["served"], "capacity": r["capacity"],
                            "plain_per_request": r["plain_per_request"], "store": r["store"],
                            "roofline": r["roofline"], "gpu_launches": r["gpu_launches"]}
    gc.collect()
    torch.cuda.empty_cache()
    return out


if __name__ == "__main__":
    main()

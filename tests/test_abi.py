"""CPU-only checks of the C ABI boundary: the library loads, exports every
symbol the public header declares, and its parameter-grid expansion matches
the oracle's restatement of each indicator's expand_grid (no GPU needed)."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from vectorta_gb300 import _native as N
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen


def test_library_exports_every_header_symbol():
    syms = N.header_symbols()
    assert len(syms) >= 140
    L = N.lib()
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_every_indicator_has_six_entry_points():
    L = N.lib()
    for name in N.INDICATORS:
        for suffix in ("expand_grid", "batch_dev", "batch_device", "batch_into_host_f32",
                       "many_series_one_param_time_major_dev", "many_series_one_param_device"):
            assert hasattr(L, f"vta_{name}_{suffix}"), (name, suffix)


def test_version_and_device_count_without_gpu():
    assert N.lib().vta_version().startswith(b"vta_gb300")
    assert N.lib().vta_device_count() >= 0


def test_oom_payload_is_empty_unless_the_last_failure_was_out_of_memory():
    # (no GPU needed: nothing has failed with OutOfMemory on this thread)
    r, f, h = C.c_size_t(7), C.c_size_t(7), C.c_size_t(7)
    assert N.lib().vta_last_error_oom(C.byref(r), C.byref(f), C.byref(h)) == 4
    assert (r.value, f.value, h.value) == (0, 0, 0)
    assert N.lib().vta_last_error_oom(None, None, None) == 4


def test_rust_binding_declares_every_entry_point():
    """The generated Rust crate (not compiled here: no Rust toolchain) declares
    each C entry point of the indicators and of the context, with as many
    parameters as the header gives it."""
    import os
    import re

    src = open(os.path.join(os.path.dirname(N.HEADER), "..", "vectorta_gb300", "rust", "vta_sys", "src",
                            "lib.rs")).read()
    hdr = open(N.HEADER).read()
    rust = {m.group(1): m.group(2) for m in re.finditer(r"pub fn (vta_\w+)\(([^)]*)\)", src)}
    want = [f"vta_{n}_{s}" for n in N.INDICATORS for s in (
        "expand_grid", "batch_dev", "batch_device", "batch_into_host_f32",
        "many_series_one_param_time_major_dev", "many_series_one_param_device")]
    want += ["vta_ctx_create", "vta_ctx_destroy", "vta_ctx_synchronize", "vta_ctx_set_policy",
             "vta_last_error", "vta_last_error_oom", "vta_device_array_free"]
    for name in want:
        assert name in rust, name
        m = re.search(name + r"\(([^;]*)\);", hdr)
        assert m, name
        n_c = 0 if m.group(1).strip() in ("void", "") else m.group(1).count(",") + 1
        n_r = 0 if not rust[name].strip() else rust[name].count(",") + 1
        assert n_c == n_r, (name, n_c, n_r)


def test_ctx_create_fails_loudly_without_gpu():
    if V.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(N.VtaError):
        V.Context(0)


def _grid(name, sweep):
    kind, outs, fam = N.INDICATORS[name]
    s = V._to_sweep(fam, sweep)
    L = N.lib()
    n = C.c_size_t()
    getattr(L, f"vta_{name}_expand_grid")(C.byref(s), None, 0, C.byref(n))
    P = N.PARAMS[fam]
    buf = (P * max(n.value, 1))()
    N.check(getattr(L, f"vta_{name}_expand_grid")(C.byref(s), buf, n.value, C.byref(n)))
    return [tuple(getattr(buf[i], f) for f, _ in P._fields_) for i in range(n.value)]


RANGES = [(5, 260, 1), (10, 50, 5), (2, 1000, 1), (50, 10, 15), (40, 9, 7), (7, 7, 0), (9, 12, 0), (30, 2, 4)]
PERIOD_ONLY = [k for k, v in N.INDICATORS.items() if v[2] == "period"]


@pytest.mark.parametrize("name", PERIOD_ONLY)
@pytest.mark.parametrize("rng", RANGES)
def test_period_grid_matches_oracle(name, rng):
    got = [g[0] for g in _grid(name, {"period": rng})]
    assert got == O.periods_of(name, rng)


def test_alma_grid_order_and_float_accumulation():
    g = _grid("alma", {"period": (5, 260, 1), "offset": (0.50, 0.95, 0.05), "sigma": (3.0, 9.0, 1.0)})
    assert len(g) == 256 * 10 * 7 == 17920
    offs = O.axis_f64((0.50, 0.95, 0.05))
    sig = O.axis_f64((3.0, 9.0, 1.0))
    exp = [(p, o, s) for p in range(5, 261) for o in offs for s in sig]
    assert g == exp  # bit-identical offsets (accumulated x += step)
    g6 = _grid("alma", {"period": (9, 9, 0), "offset": (0.5, 1.0, 0.1), "sigma": (6, 6, 0)})
    assert len(g6) == 6


def test_multi_param_grids():
    assert len(_grid("stddev", {"period": (5, 500, 5), "nbdev": (1.0, 2.0, 0.5)})) == 100 * 3
    bb = _grid("bollinger_bands", {"period": (20, 22, 1), "devup": (1.0, 2.0, 1.0), "devdn": (2.0, 2.0, 0.0)})
    assert bb == [(p, u, 2.0) for p in (20, 21, 22) for u in (1.0, 2.0)]
    st = _grid("supertrend", {"period": (10, 12, 2), "factor": (2.0, 3.0, 0.5)})
    assert st == [(p, f, ) + () for p in (10, 12) for f in (2.0, 2.5, 3.0)]
    pn = _grid("percentile_nearest_rank", {"length": (15, 17, 1), "percentage": (25.0, 75.0, 25.0)})
    assert pn == [(l, q) for l in (15, 16, 17) for q in (25.0, 50.0, 75.0)]


def test_datagen_deterministic_and_shaped():
    a = datagen.random_walk(1000, seed=1, nan_lead=50)
    b = datagen.random_walk(1000, seed=1, nan_lead=50)
    assert np.array_equal(a, b, equal_nan=True)
    assert np.isnan(a[:50]).all() and np.isfinite(a[50:]).all()
    r = np.diff(np.log(datagen.random_walk(200000, seed=2)))
    assert abs(r.std() - 0.01) < 2e-4 and abs(r.mean()) < 1e-4
    d, lens, leads = datagen.ragged_many_series(8, seed=3, min_len=100, max_len=400, max_nan_lead=20)
    assert d["close"].shape == (int(lens.max()), 8)
    for s in range(8):
        col = d["close"][:, s]
        assert np.isnan(col[: leads[s]]).all() and np.isfinite(col[leads[s]: lens[s]]).all()
        assert np.isnan(col[lens[s]:]).all()
        assert (d["high"][leads[s]:lens[s], s] >= d["low"][leads[s]:lens[s], s]).all()


def test_ma_computer_names_without_gpu():
    """vta_ma_supported mirrors supports_vram_kernel_ma (vram_ma.rs:68-76) for
    the MAs this library has kernels for (trimmed, case-insensitive)."""
    L = N.lib()
    for name in ("sma", " EMA ", "wma", "alma", "dema", "tema", "swma", "trima", "sinwma", "epma", "wilders",
                 "cwma", "fwma", "pwma", "srwma", "sqwma", "vpwma"):
        assert L.vta_ma_supported(name.encode()) == 1, name
    for name in ("hma", "jma", "vwma", "frama", "nosuch", ""):
        assert L.vta_ma_supported(name.encode()) == 0, name


"""The MA computer (the crate's VramMaComputer, vram_ma.rs:87-160, 574, 2153):
name dispatch over an arbitrary period list on a device-resident series,
row-major and time-major outputs, against the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

from test_gpu_parity import TOL, assert_close

pytestmark = pytest.mark.gpu

PERIODS = [17, 5, 30, 5, 9]  # unordered, with a repeat
CASES = {
    "sma": lambda x, p, prm: O.sma(x, p), "ema": lambda x, p, prm: O.ema(x, p),
    "wma": lambda x, p, prm: O.wma(x, p), "dema": lambda x, p, prm: O.dema(x, p),
    "tema": lambda x, p, prm: O.tema(x, p), "swma": lambda x, p, prm: O.swma(x, p),
    "trima": lambda x, p, prm: O.trima(x, p), "sinwma": lambda x, p, prm: O.sinwma(x, p),
    "wilders": lambda x, p, prm: O.wilders(x, p), "cwma": lambda x, p, prm: O.cwma(x, p),
    "fwma": lambda x, p, prm: O.fwma(x, p), "pwma": lambda x, p, prm: O.pwma(x, p, True),
    "srwma": lambda x, p, prm: O.srwma(x, p), "sqwma": lambda x, p, prm: O.sqwma(x, p),
    "alma": lambda x, p, prm: O.alma(x, p, prm.get("offset", 0.85), prm.get("sigma", 6.0)),
    "epma": lambda x, p, prm: O.epma(x, p, int(round(prm.get("offset", 0.0)))),
    "vpwma": lambda x, p, prm: O.vpwma(x, p, prm.get("power", 0.382)),
}
PARAMS = {"alma": {"offset": 0.9, "sigma": 5.0}, "epma": {"offset": 2.0}, "vpwma": {"power": 0.5}}


@pytest.fixture(scope="module")
def series():
    import torch

    x = datagen.random_walk(3000, seed=41, nan_lead=11).astype(np.float32)
    return x, torch.from_numpy(x).cuda()


@pytest.mark.parametrize("name", sorted(CASES))
def test_ma_computer_matches_oracle(name, series):
    import torch

    x, dx = series
    periods = [p for p in PERIODS if not (name == "trima" and p <= 3)]
    first = int(np.argmax(~np.isnan(x)))
    mc = V.VramMaComputer(0)
    prm = PARAMS.get(name, {})
    out = torch.empty(len(periods), x.size, device="cuda")
    mc.compute_period_ma_into(name.upper() if name == "ema" else name, prm, dx, x.size, first, periods, out)
    got = out.cpu().numpy()
    xd = x.astype(np.float64)
    exp = np.stack([CASES[name](xd, p, prm) for p in periods])
    assert_close(got, exp, TOL[name], f"ma computer {name}")
    tm = torch.empty(x.size, len(periods), device="cuda")
    mc.compute_period_ma_into(name, prm, dx, x.size, first, periods, tm, time_major=True)
    assert np.array_equal(tm.cpu().numpy(), got.T, equal_nan=True)


def test_ma_computer_errors(series):
    import torch

    x, dx = series
    mc = V.VramMaComputer(0)
    out = torch.empty(2, x.size, device="cuda")
    with pytest.raises(RuntimeError, match="not implemented|NotImplemented|no kernel"):
        mc.compute_period_ma_into("hma", None, dx, x.size, 11, [5, 9], out)
    with pytest.raises(RuntimeError):
        mc.compute_period_ma_into("nosuchma", None, dx, x.size, 11, [5, 9], out)
    with pytest.raises(RuntimeError):
        mc.compute_period_ma_into("ema", None, dx, x.size, 11, [0, 9], out)


def test_ma_selector_single_and_sweep(series):
    """CudaMaSelector: one period and a descending sweep (the selector's range
    rule) from host prices, to device and to host, against the oracle."""
    x, _ = series
    xd = x.astype(np.float64)
    sel = V.CudaMaSelector(0)
    one = sel.ma_to_device("sinwma", x, 14).to_host()
    assert one.shape == (1, x.size)
    assert_close(one[0], O.sinwma(xd, 14), TOL["sinwma"], "selector single")
    h, rows, cols = sel.ma_sweep_to_host_f32("alma", x, 30, 10, 7, {"offset": 0.8, "sigma": 4.0})
    assert (rows, cols) == (3, x.size)  # 30, 23, 16 (next 9 < 10)
    exp = np.stack([O.alma(xd, p, 0.8, 4.0) for p in (30, 23, 16)])
    assert_close(h, exp, TOL["alma"], "selector sweep")
    d = sel.ma_sweep_to_device("epma", x, 12, 20, 4, {"offset": 3}).to_host()
    assert_close(d, np.stack([O.epma(xd, p, 3) for p in (12, 16, 20)]), TOL["epma"], "selector epma")
    h1 = sel.ma_to_host_f32("ema", x, 21)
    assert_close(h1, O.ema(xd, 21), TOL["ema"], "selector to host")


def test_shared_context_buffers_survive_host_io_growth(series):
    # the MA computer's time-major staging buffer and the into-host I/O buffer
    # live in the same context: growing one leaves the other usable
    import torch

    x, dx = series
    ctx = V.Context(0)
    mc = V.VramMaComputer(0, ctx=ctx)
    first = int(np.argmax(~np.isnan(x)))
    periods = [5, 9, 30]
    tm1 = torch.empty(x.size, len(periods), device="cuda")
    mc.compute_period_ma_into("ema", {}, dx, x.size, first, periods, tm1, time_major=True)
    ema = V.CLASSES["ema"](0, ctx=ctx)
    for hi in (50, 400):  # the second call needs a larger I/O buffer
        h, rows, cols = ema.batch_into_host_f32(x, sweep={"period": (2, hi, 1)})
        assert rows == hi - 1 and cols == x.size
    tm2 = torch.empty(x.size, len(periods), device="cuda")
    mc.compute_period_ma_into("ema", {}, dx, x.size, first, periods, tm2, time_major=True)
    ctx.synchronize()
    assert np.array_equal(tm1.cpu().numpy(), tm2.cpu().numpy(), equal_nan=True)
    exp = np.stack([O.ema(x.astype(np.float64), p) for p in periods])
    assert_close(tm2.cpu().numpy().T, exp, TOL["ema"], "ma computer after host I/O growth")

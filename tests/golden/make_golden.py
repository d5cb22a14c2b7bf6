"""Regenerate the golden fixtures in this folder from the VectorTA sources.

Run where a checkout of the VectorTA project exists; its root is the
required argument (or the VECTORTA_ROOT environment variable):

    python tests/golden/make_golden.py <path to the VectorTA checkout>

Produces:

* ``bitfinex_4h.npz``  -- OHLCV columns (float64) of the crate's fixture
  ``src/data/2018-09-01-2024-Bitfinex_Spot-4h.csv``, loaded with the crate's
  own Python loader ``tests/python/test_utils.py::load_test_data``;
* ``expected.json``   -- the crate's golden last-5 values per indicator with
  the parameters, the tolerance the crate's test uses, and the file:line they
  were read from.  Values come from ``EXPECTED_OUTPUTS`` in test_utils.py when
  present there, otherwise they are parsed from the Rust unit test bodies.

The tests read only the two output files, never the reference checkout.
"""
from __future__ import annotations

import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def rust_array(path: str, anchor: str, line_hint: int) -> tuple[list[float], int]:
    """Parse the first `[...]` float list after `anchor` at or after line_hint."""
    lines = open(path).read().splitlines()
    for i in range(max(0, line_hint - 3), len(lines)):
        if anchor in lines[i]:
            text = "\n".join(lines[i:i + 12])
            m = re.search(r"\[([^\]]*)\]", text, re.S)
            vals = [float(v) for v in re.findall(r"-?\d+\.?\d*(?:e-?\d+)?", m.group(1))]
            return vals, i + 1
    raise RuntimeError(f"{anchor} not found in {path}")


def main(ref: str):
    sys.path.insert(0, os.path.join(ref, "tests", "python"))
    import test_utils  # the crate's own test helper

    cd = test_utils.load_test_data()
    np.savez_compressed(
        os.path.join(HERE, "bitfinex_4h.npz"),
        open=cd["open"], high=cd["high"], low=cd["low"], close=cd["close"],
        volume=cd["volume"],
    )
    E = test_utils.EXPECTED_OUTPUTS
    ind = os.path.join(ref, "src", "indicators")
    ma = os.path.join(ind, "moving_averages")
    gold: dict[str, dict] = {}

    def from_py(name, key, params, tol, rust_src):
        e = E[key]
        vals = e["last_5_values"] if "last_5_values" in e else e["last_five"]
        gold[name] = {"params": params, "last5": [float(v) for v in vals],
                      "tol": tol, "source": f"tests/python/test_utils.py EXPECTED_OUTPUTS['{key}']",
                      "rust_test": rust_src}

    def from_rs(name, path, anchor, hint, params, tol, rel):
        vals, line = rust_array(path, anchor, hint)
        gold[name] = {"params": params, "last5": vals, "tol": tol, "source": f"{rel}:{line}"}

    from_py("alma", "alma", {"period": 9, "offset": 0.85, "sigma": 6.0}, 1e-8, "alma.rs:1835-1841")
    gold["alma_reinput"] = {"params": {"period": 9, "offset": 0.85, "sigma": 6.0},
                            "last5": [float(v) for v in E["alma"]["reinput_last_5"]],
                            "tol": 1e-8, "source": "tests/python/test_utils.py alma.reinput_last_5",
                            "rust_test": "alma.rs:2005-2011"}
    from_py("ema", "ema", {"period": 9}, 1e-1, "ema.rs:971")
    from_py("dema", "dema", {"period": 30}, 1e-6, "dema.rs:1179-1185")
    from_py("tema", "tema", {"period": 9}, 1e-8, "tema.rs:799-805")
    from_py("wma", "wma", {"period": 30}, 1e-6, "wma.rs:860-866")
    from_py("swma", "swma", {"period": 5}, 1e-8, "swma.rs:1301-1307")
    from_py("pwma", "pwma", {"period": 5}, 1e-3, "pwma.rs:1423")
    from_py("sinwma", "sinwma", {"period": 14}, 1e-6, "sinwma.rs:1410-1416")
    from_py("trima", "trima", {"period": 30}, 1e-6, "trima.rs:1882-1888")
    gold["trima_reinput"] = {"params": {"period": 30}, "second_period": 10,
                             "last5": [float(v) for v in E["trima"]["reinput_last_5"]],
                             "tol": 1e-6, "rtol": True,
                             "source": "tests/python/test_utils.py trima.reinput_last_5; "
                                       "periods 30 then 10 as in tests/python/test_trima.py:118-137"}
    from_py("sma", "sma", {"period": 9}, 1e-1, "sma.rs:1628")
    from_py("cwma", "cwma", {"period": 14}, 1e-9, "cwma.rs:2147-2160")
    from_py("srwma", "srwma", {"period": 14}, 1e-8, "srwma.rs:1476-1490")
    from_py("sqwma", "sqwma", {"period": 14}, 1e-5, "sqwma.rs:1066-1090")
    from_py("epma", "epma", {"period": 11, "offset": 4}, 1e-1, "epma.rs:1217-1225")
    from_py("vpwma", "vpwma", {"period": 14, "power": 0.382}, 1e-2, "vpwma.rs:1690-1707")
    from_py("wilders", "wilders", {"period": 5}, 1e-8, "wilders.rs:1229-1235")
    from_py("atr", "atr", {"length": 14}, 1e-2, "atr.rs:1422")
    from_py("adx", "adx", {"period": 14}, 1e-1, "adx.rs:2163")
    from_py("zscore", "zscore", {"period": 14, "nbdev": 1.0}, 1e-8, "-")
    from_py("percentile_nearest_rank", "percentile_nearest_rank",
            {"length": 15, "percentage": 50.0}, 1e-6, "percentile_nearest_rank.rs:1411")
    pk = E["percentile_nearest_rank"]
    gold["percentile_known_answers"] = {
        "basic": pk["basic_test"], "percentiles": pk["percentile_tests"],
        "source": "tests/python/test_utils.py percentile_nearest_rank.basic_test/percentile_tests"}

    from_rs("rsi", os.path.join(ind, "rsi.rs"), "expected_last_five", 1144, {"period": 14}, 1e-2,
            "src/indicators/rsi.rs")
    from_rs("stddev", os.path.join(ind, "stddev.rs"), "expected_last_five", 1741,
            {"period": 5, "nbdev": 1.0}, 1e-1, "src/indicators/stddev.rs")
    from_rs("willr", os.path.join(ind, "willr.rs"), "expected_last_five", 1985, {"period": 14},
            1e-8, "src/indicators/willr.rs")
    from_rs("fwma", os.path.join(ind, "moving_averages", "fwma.rs"), "expected_last_five", 1266,
            {"period": 5}, 1e-8, "src/indicators/moving_averages/fwma.rs")
    st, line = rust_array(os.path.join(ind, "supertrend.rs"), "expected_last_five_trend", 2419)
    ch, _ = rust_array(os.path.join(ind, "supertrend.rs"), "expected_last_five_changed", 2419)
    gold["supertrend"] = {"params": {"period": 10, "factor": 3.0}, "last5_trend": st,
                          "last5_changed": ch, "tol": 1e-4,
                          "source": f"src/indicators/supertrend.rs:{line}"}
    bbp = os.path.join(ind, "bollinger_bands.rs")
    mid, line = rust_array(bbp, "expected_middle", 1706)
    low, _ = rust_array(bbp, "expected_lower", 1706)
    up, _ = rust_array(bbp, "expected_upper", 1706)
    gold["bollinger"] = {"params": {"period": 20, "devup": 2.0, "devdn": 2.0},
                         "last5_upper": up, "last5_middle": mid, "last5_lower": low,
                         "tol": 1e-4, "source": f"src/indicators/bollinger_bands.rs:{line}"}
    dp = os.path.join(ind, "donchian.rs")
    du, line = rust_array(dp, "expected_last_five_upper", 1386)
    dm, _ = rust_array(dp, "expected_last_five_middle", 1386)
    dl, _ = rust_array(dp, "expected_last_five_lower", 1386)
    gold["donchian"] = {"params": {"period": 20}, "last5_upper": du, "last5_middle": dm,
                        "last5_lower": dl, "tol": 1e-1,
                        "source": f"src/indicators/donchian.rs:{line}"}
    gold["donchian_reinput"] = {
        "params": {"period": 20},
        "last5_upper": [float(v) for v in E["donchian"]["reinput_last_5_upper"]],
        "last5_middle": [float(v) for v in E["donchian"]["reinput_last_5_middle"]],
        "last5_lower": [float(v) for v in E["donchian"]["reinput_last_5_lower"]],
        "tol": 1e-1, "source": "tests/python/test_utils.py donchian.reinput_last_5_*"}
    gold["pwma_formula"] = {"params": {"period": 3}, **E["pwma"]["formula_test"],
                            "source": "tests/python/test_utils.py pwma.formula_test"}
    with open(os.path.join(HERE, "expected.json"), "w") as f:
        json.dump(gold, f, indent=1, sort_keys=True)
    print(f"wrote {len(gold)} golden entries, {cd['close'].size} bars")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VECTORTA_ROOT")
    if not root:
        sys.exit("usage: make_golden.py <path to the VectorTA checkout> (or set VECTORTA_ROOT)")
    main(root)

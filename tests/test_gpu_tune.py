"""The batch-sweep autotuner: the first call with a new (indicator, log2
length, log2 sweep size) times the launch candidates and keeps the fastest;
later calls take the cached choice and give bit-identical results; the choice
is reported by last_kernel and, with VTA_TUNE_CACHE, kept in a file that a new
process reads back."""
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _tag(kernel):
    m = re.search(r"\((.*)\)$", kernel)
    assert m, kernel
    return m.group(1)


@pytest.mark.parametrize("name,sweep,n", [
    ("ema", {"period": (2, 700, 1)}, 150_001),    # chunked recurrence: warps-per-SM knob
    ("willr", {"period": (5, 400, 5)}, 700_001),  # sliding min/max: tile knob
])
def test_cache_hit_is_bit_identical(name, sweep, n):
    c = datagen.random_walk(n, seed=21, nan_lead=13)
    hi, lo = datagen.high_low(c, seed=22)
    ins = {"ema": [c], "willr": [hi, lo, c]}[name]
    ins = [np.asarray(a, np.float32) for a in ins]
    ind = V.CLASSES[name](0)
    first = ind.batch_dev(*ins, sweep=sweep).to_host()
    tag1 = _tag(ind.last_kernel)
    assert tag1.endswith("tuned") or tag1.endswith("cached"), ind.last_kernel
    second = ind.batch_dev(*ins, sweep=sweep).to_host()
    tag2 = _tag(ind.last_kernel)
    assert tag2.endswith("cached"), ind.last_kernel
    # the same choice both times (the tuned run leaves the winner's outputs)
    assert tag1.rsplit(",", 1)[0] == tag2.rsplit(",", 1)[0]
    assert np.array_equal(first, second, equal_nan=True)
    ind.set_policy("tune", "off")
    ind.batch_dev(*ins, sweep=sweep)
    assert _tag(ind.last_kernel).endswith("default"), ind.last_kernel


_CHILD = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from vectorta_gb300 import cuda as V, datagen
x = datagen.random_walk(90_001, seed=5, nan_lead=3).astype(np.float32)
ind = V.CudaEma(0)
ind.ema_batch_dev(x, sweep={"period": (2, 300, 1)})
print(ind.last_kernel)
"""


def test_choices_persist_across_processes(tmp_path):
    env = dict(os.environ, VTA_TUNE_CACHE=str(tmp_path / "tune.txt"))
    runs = [subprocess.run([sys.executable, "-c", _CHILD, ROOT], env=env, capture_output=True, text=True,
                           timeout=300) for _ in range(2)]
    for r in runs:
        assert r.returncode == 0, r.stderr[-2000:]
    k1, k2 = (r.stdout.strip().splitlines()[-1] for r in runs)
    assert _tag(k1).endswith("tuned"), k1
    assert _tag(k2).endswith("cached"), k2
    assert k1.rsplit(",", 1)[0] == k2.rsplit(",", 1)[0]
    lines = (tmp_path / "tune.txt.sweeps").read_text().split("\n")
    assert len([ln for ln in lines if ln.strip()]) == 1

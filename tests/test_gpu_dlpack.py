"""DLPack export of device arrays (the crate's DeviceArrayF32Py::__dlpack__,
dlpack_cuda.rs:265-374): zero-copy hand-over to torch, the buffer moves into
the capsule, and an unconsumed capsule frees it."""
import ctypes as C

import numpy as np
import pytest

from vectorta_gb300 import cuda as V
from vectorta_gb300 import datagen

pytestmark = pytest.mark.gpu


def _array(seed=21, n=3000):
    x = datagen.random_walk(n, seed=seed, nan_lead=5).astype(np.float32)
    return V.CudaEma(0).batch_dev(x, sweep={"period": (5, 40, 5)})


def test_torch_from_dlpack_shares_the_buffer():
    import torch

    a = _array()
    ptr, shape, host = a.ptr, a.shape, a.to_host()
    assert a.__dlpack_device__() == (2, 0)
    t = torch.from_dlpack(a)
    assert t.is_cuda and t.dtype == torch.float32 and tuple(t.shape) == shape
    assert t.data_ptr() == ptr  # zero copy
    assert np.array_equal(t.cpu().numpy(), host, equal_nan=True)
    # the array handed its buffer over
    assert a.ptr == 0 and a.shape == (0, 0)
    del t
    torch.cuda.synchronize()


@pytest.mark.parametrize("versioned", [0, 1])
def test_unconsumed_capsule_frees_its_tensor(versioned):
    import torch

    valid = C.PYFUNCTYPE(C.c_int, C.py_object, C.c_char_p)(("PyCapsule_IsValid", C.pythonapi))
    name = b"dltensor_versioned" if versioned else b"dltensor"
    ind = V.CudaEma(0)
    x = datagen.random_walk(1_000_000, seed=30, nan_lead=5).astype(np.float32)
    ind.batch_dev(x, sweep={"period": (5, 40, 5)}).free()  # context workspace at its size
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    caps = []
    for k in range(4):
        a = ind.batch_dev(x, sweep={"period": (5, 40, 5)})  # 8 x 1M f32 = 32 MB
        caps.append(a.__dlpack__(max_version=(1, 0) if versioned else None))
        assert valid(caps[-1], name) == 1
        assert a.ptr == 0
    mid = torch.cuda.mem_get_info()[0]
    assert mid <= free0 - (96 << 20)  # the four buffers live in the capsules
    del caps  # destructors run the managed tensors' deleters
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    # none of the four 32 MB buffers may stay allocated (allow 8 MB of slack)
    assert free1 >= free0 - (8 << 20)


def test_dl_device_mismatch_is_rejected():
    a = _array()
    with pytest.raises(ValueError):
        a.__dlpack__(dl_device=(2, 7))
    assert a.ptr != 0  # nothing was handed over

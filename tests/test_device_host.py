"""Device-array plumbing of the Python fronts, on the host (no GPU).

``caustica_gb300.device.as_device`` reads the two exchange protocols; these
checks use stand-in objects that expose ``__cuda_array_interface__`` with no
stream (so no CUDA call is made) and NumPy's own DLPack export, which names
the host and must be refused as a device array.
"""

from __future__ import annotations

import numpy as np
import pytest

from caustica_gb300.device import DeviceView, as_device, is_device_array


class FakeCAI:
    def __init__(self, shape, typestr, strides=None, ptr=0x7F0000000000):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (ptr, False),
                                         "strides": strides, "version": 3}


def test_a_cuda_array_interface_object_becomes_a_non_owning_view():
    obj = FakeCAI((4, 5), "<f4")
    assert is_device_array(obj)
    v = as_device(obj, dtype=np.float32, shape=(4, 5))
    assert isinstance(v, DeviceView)
    assert v.shape == (4, 5) and v.dtype == np.float32 and v.nbytes == 80
    assert v.ptr.value == 0x7F0000000000
    v.close()  # frees nothing: the producer owns the memory
    assert v.ptr is None


def test_layout_dtype_and_shape_are_checked():
    with pytest.raises(ValueError, match="C-contiguous"):
        as_device(FakeCAI((4, 5), "<f4", strides=(4, 16)), what="q")
    as_device(FakeCAI((4, 5), "<f4", strides=(20, 4)))  # explicit C strides are fine
    with pytest.raises(ValueError, match="need float32"):
        as_device(FakeCAI((3,), "<f8"), dtype=np.float32)
    with pytest.raises(ValueError, match=r"need \(3, 2\)"):
        as_device(FakeCAI((2, 3), "|u1"), shape=(3, 2))


def test_host_arrays_are_not_device_arrays():
    a = np.zeros((3, 3), np.float32)
    assert not is_device_array(a)  # NumPy's DLPack export names the CPU
    with pytest.raises(ValueError, match="expected a device array"):
        as_device(a)
    with pytest.raises(ValueError, match="expected a device array"):
        as_device([1.0, 2.0])

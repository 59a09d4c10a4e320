"""Device-resident inputs for the Python fronts.

The C ABI takes host or device pointers alike. This module lets the Python
fronts take device arrays from any framework through the two standard
exchange protocols -- ``__cuda_array_interface__`` (CuPy, Numba, PyTorch)
and DLPack (``__dlpack__`` / ``__dlpack_device__``) -- and hand their device
pointers to the library without a host round trip:

* :func:`as_device` wraps such an object as a non-owning
  :class:`DeviceView` (the producer keeps the memory; the view keeps the
  producer alive);
* :class:`DeviceLabelMedium` is a medium whose uint8 label map lives on the
  device, with one (alpha, rho, c, beta) row per label -- the shape of the
  reference's ``Medium.from_id_map`` (medium.py:57-81). The solver copies
  the labels device to device; host volumes are formed only if a caller
  asks for ``alpha``/``rho``/``c``/``beta``.

Heating terms, initial temperatures and doses given as device arrays go
straight to the Pennes calls; steering phases given as device arrays are
read back (a few KB) so the source scale is formed with the same float32
host arithmetic as for host phases.
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

_KDL_CUDA, _KDL_CUDA_MANAGED = 2, 13
_DL_CODES = {0: "i", 1: "u", 2: "f"}


class _DLDevice(C.Structure):
    _fields_ = [("device_type", C.c_int32), ("device_id", C.c_int32)]


class _DLDataType(C.Structure):
    _fields_ = [("code", C.c_uint8), ("bits", C.c_uint8), ("lanes", C.c_uint16)]


class _DLTensor(C.Structure):
    _fields_ = [("data", C.c_void_p), ("device", _DLDevice), ("ndim", C.c_int32), ("dtype", _DLDataType),
                ("shape", C.POINTER(C.c_int64)), ("strides", C.POINTER(C.c_int64)), ("byte_offset", C.c_uint64)]


class _DLManagedTensor(C.Structure):
    _fields_ = [("dl_tensor", _DLTensor), ("manager_ctx", C.c_void_p), ("deleter", C.c_void_p)]


_capsule_ptr = C.pythonapi.PyCapsule_GetPointer
_capsule_ptr.restype = C.c_void_p
_capsule_ptr.argtypes = [C.py_object, C.c_char_p]


class DeviceView(_lib.DeviceArray):
    """A non-owning view of another framework's device array (C-contiguous)."""

    def __init__(self, ptr: int, shape, dtype, owner):  # noqa: D107 - no allocation here
        self.shape = tuple(int(n) for n in shape)
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape, dtype=np.int64)) * self.dtype.itemsize
        self.ptr = C.c_void_p(int(ptr))
        self._owner = owner  # keeps the producer's memory alive

    def close(self) -> None:  # the producer frees its memory
        self.ptr = None
        self._owner = None


def is_device_array(obj) -> bool:
    """True for objects exposing device memory through either protocol."""
    if isinstance(obj, _lib.DeviceArray):
        return True
    if hasattr(obj, "__cuda_array_interface__"):
        return True
    if hasattr(obj, "__dlpack_device__"):
        try:
            return int(obj.__dlpack_device__()[0]) in (_KDL_CUDA, _KDL_CUDA_MANAGED)
        except Exception:  # noqa: BLE001 - not a device array then
            return False
    return False


def _contiguous(shape, strides, itemsize) -> bool:
    if strides is None:
        return True
    want = itemsize
    for n, st in zip(reversed(shape), reversed(strides)):
        if n > 1 and st != want:
            return False
        want *= n
    return True


def as_device(obj, dtype=None, shape=None, what: str = "array") -> DeviceView:
    """Wrap a device array (either protocol) as a :class:`DeviceView`.

    The producer's pending work on the stream it names is waited for, so the
    library's own streams read finished data. Raises ``ValueError`` for host
    arrays, non-contiguous layouts or a dtype/shape other than the one asked."""
    if isinstance(obj, _lib.DeviceArray):
        view = obj
    elif hasattr(obj, "__cuda_array_interface__"):
        cai = obj.__cuda_array_interface__
        ptr, _ro = cai["data"]
        dt = np.dtype(cai["typestr"])
        shp = tuple(cai["shape"])
        if not _contiguous(shp, cai.get("strides"), dt.itemsize):
            raise ValueError(f"{what}: device arrays must be C-contiguous")
        stream = cai.get("stream")
        if stream is not None and stream != 0:
            _lib.call("cg_stream_synchronize", C.c_void_p(int(stream)))
        view = DeviceView(ptr or 0, shp, dt, obj)
    elif hasattr(obj, "__dlpack__") and is_device_array(obj):
        cap = obj.__dlpack__()
        mt = _DLManagedTensor.from_address(_capsule_ptr(cap, b"dltensor"))
        t = mt.dl_tensor
        if t.dtype.lanes != 1 or t.dtype.code not in _DL_CODES:
            raise ValueError(f"{what}: unsupported DLPack dtype (code {t.dtype.code}, lanes {t.dtype.lanes})")
        dt = np.dtype(f"{_DL_CODES[t.dtype.code]}{t.dtype.bits // 8}")
        shp = tuple(int(t.shape[i]) for i in range(t.ndim))
        strides = None if not t.strides else tuple(int(t.strides[i]) * dt.itemsize for i in range(t.ndim))
        if not _contiguous(shp, strides, dt.itemsize):
            raise ValueError(f"{what}: device arrays must be C-contiguous")
        _lib.call("cg_stream_synchronize", None)  # DLPack's default: ready on the legacy stream
        view = DeviceView((t.data or 0) + t.byte_offset, shp, dt, (obj, cap))
    else:
        raise ValueError(f"{what}: expected a device array (__cuda_array_interface__ or DLPack), "
                         f"got {type(obj).__name__}")
    if dtype is not None and view.dtype != np.dtype(dtype):
        raise ValueError(f"{what}: device array is {view.dtype}, need {np.dtype(dtype)}")
    if shape is not None and tuple(view.shape) != tuple(shape):
        raise ValueError(f"{what}: device array has shape {view.shape}, need {tuple(shape)}")
    return view


def to_host(obj, dtype=None) -> np.ndarray:
    """A host copy of a device array (small inputs such as phases)."""
    v = as_device(obj, dtype=dtype)
    return v.to_host()


class DeviceLabelMedium:
    """A medium whose label map lives on the device.

    ``labels``: uint8 device array of the grid's shape (either protocol);
    ``table``: ``{label: (alpha [Np/m], rho, c, beta)}`` covering every label
    that occurs. The labels present are counted on the device once, so the
    time step and the nonlinearity switch follow the materials that occur,
    as they would for the equivalent host ``Medium``.
    """

    def __init__(self, labels, table: dict):
        self.labels = as_device(labels, dtype=np.uint8, what="labels")
        self.shape = tuple(self.labels.shape)
        counts = np.zeros(256, np.uint64)
        _lib.call("cg_label_counts", self.labels.ptr, int(np.prod(self.shape)), _lib.ptr(counts))
        self.present = np.flatnonzero(counts)
        missing = [int(i) for i in self.present if int(i) not in table]
        if missing:
            raise ValueError(f"label map contains labels {missing} that are missing from the table")
        self.table = {int(k): tuple(float(x) for x in v) for k, v in table.items()}
        rows = np.zeros((256, 4), np.float32)
        for k, v in self.table.items():
            if not 0 <= k < 256:
                raise ValueError(f"label {k} does not fit a uint8 label map")
            rows[k] = np.asarray(v, np.float32)
        self.rows = rows  # float32, per label value
        self._host = None

    # the facts the solver needs, from the labels that occur
    @property
    def c_min(self) -> float:
        return float(self.rows[self.present, 2].min())

    @property
    def c_max(self) -> float:
        return float(self.rows[self.present, 2].max())

    @property
    def is_linear(self) -> bool:
        return bool((self.rows[self.present, 3] == 0).all())

    def labels_at(self, idx: np.ndarray) -> np.ndarray:
        """Labels at integer voxel indices (n, ndim), gathered on the device."""
        idx = np.asarray(idx, np.int64)
        flat = np.ascontiguousarray(np.ravel_multi_index(tuple(idx.T), self.shape).astype(np.int64))
        out = np.zeros(len(flat), np.uint8)
        _lib.call("cg_gather_u8", self.labels.ptr, _lib.ptr(flat), len(flat), _lib.ptr(out))
        return out

    # host volumes for callers that want them (formed once, on request)
    def _volumes(self):
        if self._host is None:
            lab = self.labels.to_host()
            self._host = [np.ascontiguousarray(self.rows[:, k][lab]) for k in range(4)] + [lab]
        return self._host

    @property
    def alpha(self):
        return self._volumes()[0]

    @property
    def rho(self):
        return self._volumes()[1]

    @property
    def c(self):
        return self._volumes()[2]

    @property
    def beta(self):
        return self._volumes()[3]

    @property
    def id_map(self):
        return self._volumes()[4]

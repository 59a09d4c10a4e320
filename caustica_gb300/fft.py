"""Batched 3-D real FFT on GB300 (the solver's own axis passes).

``FFT3D(shape, batch).forward(x)`` returns the half spectrum of
``scipy.fft.rfftn(x, axes=(-3, -2, -1))`` in the solver's layout
``[batch][x][kz][y]``; :meth:`FFT3D.to_numpy_layout` transposes it to
``[batch][x][y][kz]``. ``inverse`` is unnormalised (divide by nx*ny*nz for
``irfftn``). Replaces the backend FFT calls of the reference step
(solvers/kspace/engine.py:459-469).
"""

from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib


class FFT3D:
    def __init__(self, shape, batch: int = 1):
        self.shape = tuple(int(s) for s in shape)
        if len(self.shape) != 3:
            raise ValueError("shape must be (nx, ny, nz)")
        self.batch = int(batch)
        nx, ny, nz = self.shape
        self.spec_shape = (self.batch, nx, nz // 2 + 1, ny)
        h = C.c_void_p()
        _lib.check(_lib.load().cg_fft3d_create(nx, ny, nz, self.batch, C.byref(h)), "cg_fft3d_create")
        self.h = h

    def forward(self, x: np.ndarray) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32).reshape((self.batch, *self.shape))
        out = np.zeros(self.spec_shape, np.complex64)
        _lib.call("cg_fft3d_forward", self.h, _lib.ptr(x), _lib.ptr(out))
        return out

    def inverse(self, spec: np.ndarray) -> np.ndarray:
        spec = np.ascontiguousarray(spec, np.complex64).reshape(self.spec_shape)
        out = np.zeros((self.batch, *self.shape), np.float32)
        _lib.call("cg_fft3d_inverse", self.h, _lib.ptr(spec), _lib.ptr(out))
        return out

    @staticmethod
    def to_numpy_layout(spec: np.ndarray) -> np.ndarray:
        return np.ascontiguousarray(np.swapaxes(spec, -1, -2))

    @staticmethod
    def from_numpy_layout(spec: np.ndarray) -> np.ndarray:
        return np.ascontiguousarray(np.swapaxes(spec, -1, -2))

    def close(self) -> None:
        if getattr(self, "h", None):
            _lib.load().cg_fft3d_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover
        try:
            self.close()
        except Exception:
            pass

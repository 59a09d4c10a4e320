"""ctypes binding of ``libcaustica_gb300.so`` (the C ABI in ``include/caustica_gb300.h``).

The library is the only compute path: if it is missing or cannot be loaded
the import of anything that needs it raises. There is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libcaustica_gb300.so"

CG_OK = 0
CG_ERR_INVALID = 1
CG_ERR_OOM = 2
CG_ERR_CUDA = 3
CG_ERR_NONFINITE = 4
CG_ERR_TIMEOUT = 5


class CGError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, code: int, func: str, msg: str):
        super().__init__(f"{func} failed (code {code}): {msg}")
        self.code = code


class CGInvalidArgument(CGError, ValueError):
    """The library refused its arguments (CG_ERR_INVALID)."""


class SolverConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("batch", C.c_int), ("nonlinear", C.c_int), ("spp", C.c_int), ("max_periods", C.c_int),
        ("n_harmonics", C.c_int), ("harmonics", C.c_int * 8),
        ("pml", C.c_int * 3), ("pml_edge", C.c_double),
        ("dx", C.c_double), ("dt", C.c_double), ("c_ref", C.c_double),
        ("rec_lo", C.c_int * 3), ("rec_hi", C.c_int * 3),
        ("conv_lo", C.c_int * 3), ("conv_hi", C.c_int * 3),
    ]


class PennesConfig(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("dirichlet", C.c_int), ("dose", C.c_int),
        ("theta_wall", C.c_float), ("t_ref", C.c_float), ("half_dt_min", C.c_float),
        ("n_labels", C.c_int),
    ]


class QField(C.Structure):
    _fields_ = [("data", C.c_void_p), ("n", C.c_longlong), ("stride", C.c_longlong)]


class FocusInput(C.Structure):
    _fields_ = [
        ("p1", C.c_void_p), ("p2", C.c_void_p), ("pmax", C.c_void_p),
        ("shape", C.c_int * 3), ("lo", C.c_int * 3), ("hi", C.c_int * 3), ("probe", C.c_int * 3),
        ("offset", C.c_int * 3), ("dx", C.c_double),
    ]


class FocusReport(C.Structure):
    _fields_ = [
        ("peak", C.c_longlong), ("p_peak", C.c_float), ("p_max_at_peak", C.c_float),
        ("n_above_half", C.c_longlong), ("p_probe", C.c_float), ("has_a2", C.c_int),
        ("a2_at_peak", C.c_float), ("a2_peak", C.c_float), ("a2_peak_index", C.c_longlong),
        ("truncated", C.c_int * 3), ("left", C.c_double * 3), ("right", C.c_double * 3),
    ]


class HeatingSpec(C.Structure):
    _fields_ = [
        ("n_terms", C.c_int), ("harmonics", C.c_int * 8), ("phasor", C.c_void_p * 8), ("shape", C.c_int * 3),
        ("n_labels", C.c_int), ("coef", C.c_void_p), ("labels", C.c_void_p),
        ("alpha", C.c_void_p), ("rho", C.c_void_p), ("c", C.c_void_p), ("alpha_factor", C.c_double * 8),
        ("map_shape", C.c_int * 3), ("map_origin", C.c_int * 3),
        ("q_shape", C.c_int * 3), ("q_origin", C.c_int * 3), ("scale", C.c_float),
    ]


_P = C.c_void_p
_I = C.c_int
_LL = C.c_longlong

# name -> (argtypes); every function returns int unless listed in _RESTYPE
SIGNATURES = {
    "cg_last_error": [],
    "cg_version": [],
    "cg_set_device": [_I],
    "cg_solver_create": [C.POINTER(SolverConfig), C.POINTER(_P)],
    "cg_solver_destroy": [_P],
    "cg_solver_set_medium_labels": [_P, _P, _I, _P],
    "cg_solver_set_medium_dense": [_P, _P, _P, _P, _P],
    "cg_solver_set_source": [_P, _I, _P, _P, _P],
    "cg_solver_set_drive": [_P, _I, _P],
    "cg_solver_reset": [_P],
    "cg_solver_run": [_P, _I, _I],
    "cg_solver_run_periods": [_P, _I, _I],
    "cg_solver_begin_record": [_P],
    "cg_solver_read_peaks": [_P, _I, _I, _P],
    "cg_solver_finalize": [_P, _I, _P, _P],
    "cg_solver_get_state": [_P, _P, _P],
    "cg_solver_set_state": [_P, _P, _P, _LL],
    "cg_solver_synchronize": [_P],
    "cg_solver_query": [_P, _P],
    "cg_solver_info": [_P, _P],
    "cg_solver_timed_run": [_P, _I, _I, _I, _P],
    "cg_solver_profile": [_P, _I, _I, _P],
    "cg_solver_autotune": [_P, _I, _P],
    "cg_solver_set_slabs": [_P, _I],
    "cg_solver_set_zstaging": [_P, _I],
    "cg_solver_get_zstaging": [_P, _P],
    "cg_solver_get_config": [_P, _P],
    "cg_fft3d_create": [_I, _I, _I, _I, C.POINTER(_P)],
    "cg_fft3d_destroy": [_P],
    "cg_fft3d_forward": [_P, _P, _P],
    "cg_fft3d_inverse": [_P, _P, _P],
    "cg_fft3d_forward_noalloc": [_I, _I, _I, _I, _P, _P, _P],
    "cg_pennes_create": [C.POINTER(PennesConfig), C.POINTER(_P)],
    "cg_pennes_destroy": [_P],
    "cg_pennes_set_coefficients": [_P, _P, _P, _P, _P, _P, _P, _P, _P],
    "cg_pennes_set_labels": [_P, _P, _I, _P, C.c_float, _I, _I, _P],
    "cg_pennes_set_state": [_P, _P, _P, _P],
    "cg_pennes_run": [_P, _I],
    "cg_pennes_timed_run": [_P, _I, _P],
    "cg_pennes_set_temperature": [_P, _P, _P, _P],
    "cg_pennes_get_temperature": [_P, _P, _P, _P],
    "cg_pennes_check_finite": [_P, _P],
    "cg_pennes_get_state": [_P, _P, _P, _P],
    "cg_focus_metrics": [C.POINTER(FocusInput), C.POINTER(FocusReport), _P],
    "cg_solver_focus_metrics": [_P, _I, C.POINTER(FocusInput), C.POINTER(FocusReport)],
    "cg_heating_q": [C.POINTER(HeatingSpec), _P, _P, _P],
    "cg_solver_heating_q": [_P, _I, C.POINTER(HeatingSpec), _P, _P],
    "cg_quantize_f16": [C.POINTER(QField), _I, C.c_double, _P, _P, _P, _P],
    "cg_solver_quantize": [_P, _I, C.c_double, _P, _P, _P],
    "cg_label_counts": [_P, _LL, _P],
    "cg_gather_u8": [_P, _P, _I, _P],
    "cg_stream_synchronize": [_P],
    "cg_buffer_alloc": [C.c_size_t, C.POINTER(_P)],
    "cg_buffer_free": [_P],
    "cg_buffer_copy": [_P, _P, C.c_size_t],
}
_RESTYPE = {"cg_last_error": C.c_char_p}

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load the library (once) and declare every exported signature."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(
            f"{p} is missing: build it with `python -m caustica_gb300.build` "
            f"(there is no CPU fallback for this solver)"
        )
    lib = C.CDLL(str(p))
    for name, args in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = _RESTYPE.get(name, C.c_int)
    _lib = lib
    return lib


def last_error() -> str:
    return load().cg_last_error().decode(errors="replace")


def check(code: int, func: str) -> None:
    if code != CG_OK:
        msg = last_error()
        if code == CG_ERR_INVALID:
            raise CGInvalidArgument(code, func, msg)
        raise CGError(code, func, msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)


def ptr(a: np.ndarray | None):
    """Host pointer of a C-contiguous array (None -> NULL)."""
    if a is None:
        return None
    if not a.flags.c_contiguous:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data_as(C.c_void_p)


class DeviceArray:
    """A device buffer of the library (``cg_buffer_alloc``) with a NumPy shape and dtype.

    Carries fields between device calls without a host copy (phasors into
    the focal metrics, Q into the Pennes step); ``to_host`` reads it back.
    """

    def __init__(self, shape, dtype):
        self.shape = tuple(int(n) for n in shape)
        self.dtype = np.dtype(dtype)
        self.nbytes = int(np.prod(self.shape, dtype=np.int64)) * self.dtype.itemsize
        h = C.c_void_p()
        check(load().cg_buffer_alloc(self.nbytes, C.byref(h)), "cg_buffer_alloc")
        self.ptr = h

    @classmethod
    def from_host(cls, a: np.ndarray) -> "DeviceArray":
        a = np.ascontiguousarray(a)
        d = cls(a.shape, a.dtype)
        if d.nbytes:
            call("cg_buffer_copy", d.ptr, ptr(a), d.nbytes)
        return d

    def to_host(self) -> np.ndarray:
        out = np.empty(self.shape, self.dtype)
        if self.nbytes:
            call("cg_buffer_copy", ptr(out), self.ptr, self.nbytes)
        return out

    def close(self) -> None:
        if getattr(self, "ptr", None):
            load().cg_buffer_free(self.ptr)
            self.ptr = None

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

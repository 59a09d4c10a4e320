"""Oracle: dynamic float16 quantisation of a stored result field (NumPy).

TEST INFRASTRUCTURE ONLY (see :mod:`oracle`). Restates ``try_float16``
(``io/quantize.py:45-67``, paths relative to ``src/caustica/``): the field is
divided by its own absolute peak, cast to float16, reconstructed and measured
against the original; the float16 copy is kept when the largest round-trip
error, as a fraction of the peak, is within ``max_norm_err`` (``1e-3`` by
default, ``io/quantize.py:21``), else the float32 values are kept with scale
1. A zero peak (or an empty field) stores the plain cast. Every operation is
NumPy's float32 arithmetic on the float32 array with the peak as a Python
float, as in the reference, so a test compares the device's output with
this one bit for bit. ``store_order`` restates the order in which
``save_result`` writes the quantised datasets (``io/store.py:146-151``).
"""

from __future__ import annotations

from typing import NamedTuple

import numpy as np

DEFAULT_MAX_NORM_ERR = 1e-3


class Quantized(NamedTuple):
    stored: np.ndarray
    scale: float
    dtype_name: str
    norm_err: float


def try_float16(arr, max_norm_err: float = DEFAULT_MAX_NORM_ERR) -> Quantized:
    a = np.asarray(arr, dtype=np.float32)
    peak = float(np.abs(a).max()) if a.size else 0.0
    if peak <= 0.0:
        return Quantized(a.astype(np.float16), 1.0, "float16", 0.0)
    q = (a / peak).astype(np.float16)
    err = float(np.abs(q.astype(np.float32) * peak - a).max() / peak)
    if err <= max_norm_err:
        return Quantized(q, peak, "float16", err)
    return Quantized(a, 1.0, "float32", 0.0)


def restore(stored, scale: float) -> np.ndarray:
    return np.asarray(stored).astype(np.float32) * np.float32(scale)


def store_order(phasors: dict, p_max) -> list[tuple[str, np.ndarray]]:
    """(dataset name, float32 field) in the order the store writes them."""
    out = []
    for h in sorted(phasors):
        ph = np.asarray(phasors[h])
        out.append((f"p_real_h{h}", np.ascontiguousarray(ph.real, dtype=np.float32)))
        out.append((f"p_imag_h{h}", np.ascontiguousarray(ph.imag, dtype=np.float32)))
    out.append(("p_max", np.asarray(p_max, dtype=np.float32)))
    return out

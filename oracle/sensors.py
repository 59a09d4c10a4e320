"""Oracle: volumetric heating Q from recorded phasors (NumPy, FP64).

TEST INFRASTRUCTURE ONLY (see :mod:`oracle`). Restates
``HeatingSource.from_phasors`` (sensors.py:193-295): Q = sum_n alpha_n
|P_n|^2 / (rho c) in float64, returned as float32.
"""

from __future__ import annotations

import numpy as np


def heating_q(phasors: dict, *, alpha, rho, c, harmonics=None, alpha_power_law_y=None, exact_amp=False):
    """Q [W/m^3] (sensors.py:259-273); alpha_n = alpha_f0 n^y when y is given (sensors.py:393-402).

    ``exact_amp`` takes |P| as the correctly rounded float32 (float64 square
    root of the exact sum of squares) instead of NumPy's complex ``abs``.
    """
    requested = tuple(sorted(phasors)) if harmonics is None else tuple(harmonics)
    shape = np.shape(phasors[requested[0]])
    alpha_f0 = np.broadcast_to(np.asarray(alpha, np.float64), shape)
    rho_map = np.broadcast_to(np.asarray(rho, np.float64), shape)
    c_map = np.broadcast_to(np.asarray(c, np.float64), shape)
    if any(n >= 2 for n in requested) and alpha_power_law_y is None:
        raise ValueError("harmonics above the fundamental need an absorption model")
    inv_rho_c = 1.0 / (rho_map * c_map)
    q = np.zeros(shape, dtype=np.float64)
    for n in requested:
        a_n = alpha_f0 if alpha_power_law_y is None else alpha_f0 * float(n) ** alpha_power_law_y
        p = np.asarray(phasors[n])
        if exact_amp:
            re, im = p.real.astype(np.float64), p.imag.astype(np.float64)
            amp = np.sqrt(re * re + im * im).astype(np.float32)
        else:
            amp = np.abs(p).astype(np.float32)
        p2 = amp.astype(np.float64) ** 2
        q += a_n * p2 * inv_rho_c
    return np.ascontiguousarray(q, dtype=np.float32)

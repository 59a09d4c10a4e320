"""Oracle: focal metrics of a CW result (NumPy).

TEST INFRASTRUCTURE ONLY (see :mod:`oracle`). Restates
``report/metrics.py`` (paths relative to ``src/caustica/``): the interior
box (:96-120), the interior argmax (:123-127), the -6 dB crossing (:130-152),
the plane-wave intensity (:155-157), the PML distance (:171-184) and
``focus_metrics`` (:192-313), on plain arrays. The golden fixtures
``tests/golden/focus_*.npz`` hold the reference's own output for the same
inputs.

``amp`` may be supplied so that the device's correctly rounded amplitudes
can be checked without NumPy's vectorised complex ``abs`` (which may differ
from them by a unit in the last place).
"""

from __future__ import annotations

import numpy as np

HALF_PRESSURE = 0.5
A2_PML_MARGIN_WARN_VOX = 8


def interior(origin, shape, grid_shape, pml_vox, extra=2):
    """Record-frame slices with the sponge plus ``extra`` voxels removed (metrics.py:96-120)."""
    margin = pml_vox + extra
    out = []
    for d, (o, n) in enumerate(zip(origin, shape)):
        lo = max(0, margin - o)
        hi = min(n, grid_shape[d] - margin - o)
        if hi <= lo:
            raise ValueError(f"axis {d}: the record region lies entirely inside the PML margin")
        out.append(slice(lo, hi))
    return tuple(out)


def argmax_in(field, box):
    """First maximum in C order of ``field[box]``, in the full-array frame (metrics.py:123-127)."""
    sub = field[box]
    loc = np.unravel_index(int(np.argmax(sub)), sub.shape)
    return tuple(int(i) + s.start for i, s in zip(loc, box))


def crossing(coord, prof, i0, level):
    """First coordinate right of ``i0`` where ``prof`` falls below ``level`` (metrics.py:130-137)."""
    for i in range(i0, prof.size - 1):
        if prof[i + 1] < level <= prof[i]:
            t = (prof[i] - level) / (prof[i] - prof[i + 1])
            return float(coord[i] + t * (coord[i + 1] - coord[i]))
    return None


def extent(coord, prof, i0):
    """-6 dB extent around ``i0`` (metrics.py:140-152)."""
    level = HALF_PRESSURE * float(prof[i0])
    right = crossing(coord, prof, i0, level)
    left = crossing(coord[::-1], prof[::-1], prof.size - 1 - i0, level)
    if right is None or left is None:
        return {"left_mm": None, "right_mm": None, "width_mm": None, "truncated": True}
    return {"left_mm": round(left * 1e3, 3), "right_mm": round(right * 1e3, 3),
            "width_mm": round((right - left) * 1e3, 3), "truncated": False}


def edge_distance(vox, grid_shape, pml_vox):
    """Voxels to the nearest sponge face (metrics.py:171-184)."""
    return min(min(int(i) - pml_vox, (n - pml_vox - 1) - int(i)) for i, n in zip(vox, grid_shape))


def a2_warning(d):
    """The a2-near-the-absorber caveat (metrics.py:187-193); the text is part of the output."""
    return (
        f"the a2 peak lies {d} voxels from the PML edge "
        f"(< {A2_PML_MARGIN_WARN_VOX}) — likely a harmonic-DFT edge artifact rather "
        f"than physics (an edge residue grows LINEARLY with drive, a real second "
        f"harmonic quadratically); a2_at_fundamental_peak_pa is the trustworthy number."
    )


def focus_metrics(p1, *, origin, grid_shape, pml_vox, apex, dx, focus=None, p2=None, p_max=None,
                  rho=None, c=None, source_amplitude=None, run=None, amp=None, amp2=None):
    """The metrics dictionary of ``focus_metrics`` (metrics.py:192-313).

    ``rho``/``c`` are grid-frame maps (ISPPA), ``run`` the ``run`` section
    (copied through), ``amp``/``amp2`` optional precomputed amplitudes.
    """
    a = np.abs(p1).astype(np.float32) if amp is None else amp
    box = interior(origin, a.shape, grid_shape, pml_vox)
    pk = argmax_in(a, box)
    pk_g = tuple(i + o for i, o in zip(pk, origin))
    peak = float(a[pk])
    coords = [(np.arange(a.shape[d]) + origin[d] - apex[d]) * dx for d in range(3)]
    prof = [a[:, pk[1], pk[2]], a[pk[0], :, pk[2]], a[pk[0], pk[1], :]]
    volume = float((a[box] >= HALF_PRESSURE * peak).sum() * (dx * 1e3) ** 3)
    isppa = None
    if rho is not None:
        isppa = round(float(peak ** 2 / (2.0 * float(rho[pk_g]) * float(c[pk_g])) / 1e4), 1)
    m = {"peak": {
        "p_pa": round(peak, 1),
        "p_mpa": round(peak / 1e6, 4),
        "voxel_grid": [int(i) for i in pk_g],
        "position_mm_from_apex": {k: round(float(coords[d][pk[d]]) * 1e3, 3) for d, k in enumerate("xyz")},
        "gain_vs_source": None if source_amplitude is None else round(peak / source_amplitude, 2),
        "isppa_w_cm2": isppa,
        "p_max_time_domain_pa": None if p_max is None else round(float(p_max[pk]), 1),
    }}
    if focus is not None:
        t = tuple(int(f) - o for f, o in zip(focus, origin))
        inside = all(0 <= i < n for i, n in zip(t, a.shape))
        pt = float(a[t]) if inside else float("nan")
        m["target"] = {
            "voxel_grid": [int(i) for i in focus],
            "p_pa": None if np.isnan(pt) else round(pt, 1),
            "hit_ratio": None if np.isnan(pt) else round(pt / peak, 4),
            "displacement_mm": {k: round((pk_g[d] - focus[d]) * dx * 1e3, 3) for d, k in enumerate("xyz")},
            "displacement_norm_mm": round(float(np.linalg.norm(np.array(pk_g) - np.array(focus)) * dx * 1e3), 3),
        }
    m["focal_spot"] = {
        "axial_6db": extent(coords[2], prof[2], pk[2]),
        "lateral_x_6db": extent(coords[0], prof[0], pk[0]),
        "lateral_y_6db": extent(coords[1], prof[1], pk[1]),
        "volume_above_6db_mm3": round(volume, 3),
    }
    if run is not None:
        m["run"] = run
    warns = []
    if p2 is not None or amp2 is not None:
        a2 = np.abs(p2).astype(np.float32) if amp2 is None else amp2
        pk2 = argmax_in(a2, box)
        pk2_g = tuple(i + o for i, o in zip(pk2, origin))
        d = edge_distance(pk2_g, grid_shape, pml_vox)
        m["harmonics"] = {
            "a2_at_fundamental_peak_pa": round(float(a2[pk]), 1),
            "a2_over_a1_at_peak_pct": round(100.0 * float(a2[pk]) / float(a[pk]), 2),
            "a2_peak_pa": round(float(a2[pk2]), 1),
            "a2_peak_voxel_grid": [int(i) for i in pk2_g],
            "a2_peak_distance_to_pml_vox": d,
        }
        if d < A2_PML_MARGIN_WARN_VOX:
            warns.append(a2_warning(d))
    m["warnings"] = warns
    return m


def exact_amp(p):
    """Correctly rounded float32 |p| (float64 square root of the exact sum of squares)."""
    re = p.real.astype(np.float64)
    im = p.imag.astype(np.float64)
    return np.sqrt(re * re + im * im).astype(np.float32)

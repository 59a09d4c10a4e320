"""Focal metrics of a CW result, reduced on the GPU.

Mirrors ``caustica.report.metrics`` (report/metrics.py:37-313): the same
:class:`FieldFrame`, the same ``focus_metrics`` signature and the same
JSON-ready dictionary. The field-sized work -- the interior argmax of
|P1| (and |P2|), the count of interior voxels at or above half the peak,
the three profiles through the peak -- runs in ``cg_focus_metrics``
(``csrc/cg_post.cu``); the host only turns the handful of numbers it returns
into the dictionary, with the reference's rounding.

Amplitudes are the correctly rounded float32 |P|. NumPy's vectorised complex
``abs`` may differ from them by one or two units in the last place, so a
result can differ from the reference's only where two interior amplitudes
(or an amplitude and half the peak) lie that close.

``device_focus_metrics`` computes the same from a live solver handle's
phasors without copying the field to the host (the serving loop's path).
"""

from __future__ import annotations

import ctypes as C
from collections.abc import Mapping
from dataclasses import dataclass
from typing import Any

import numpy as np

from . import _lib

HALF_PRESSURE = 0.5  # -6 dB in pressure (metrics.py:23)
A2_PML_MARGIN_WARN_VOX = 8  # metrics.py:33


@dataclass(frozen=True)
class FieldFrame:
    """Where a solved field sits on the grid (metrics.py:36-75)."""

    dx: float
    grid_shape: tuple[int, ...]
    pml_vox: int
    apex_vox: tuple[int, int, int]
    focus_vox: tuple[int, int, int] | None = None

    @classmethod
    def from_geometry(cls, geo: Mapping[str, Any]) -> "FieldFrame":
        focus = geo.get("focus_vox")
        return cls(dx=float(geo["dx"]), grid_shape=tuple(int(v) for v in geo["grid_shape"]),
                   pml_vox=int(geo["pml_vox"]), apex_vox=tuple(int(v) for v in geo["apex_vox"]),
                   focus_vox=None if focus is None else tuple(int(v) for v in focus))


def region_origin(result) -> tuple[int, ...]:
    return tuple(int(sl.start) for sl in result.region)


def interior_slices(result, frame: FieldFrame, *, extra: int = 2) -> tuple[slice, ...]:
    """Record-region slices without the sponge and ``extra`` voxels (metrics.py:96-120)."""
    return _interior(region_origin(result), np.shape(result.phasor), frame, extra)


def _interior(org, shape, frame, extra=2):
    margin = frame.pml_vox + extra
    out = []
    for d, (o, n) in enumerate(zip(org, shape)):
        lo = max(0, margin - o)
        hi = min(n, frame.grid_shape[d] - margin - o)
        if hi <= lo:
            raise ValueError(f"axis {d}: the record region lies entirely inside the PML margin "
                             f"({margin} voxels); nothing to analyze.")
        out.append(slice(lo, hi))
    return tuple(out)


def intensity_w_cm2(pressure_pa: float, rho: float, c: float) -> float:
    """Plane-wave CW intensity p^2 / (2 rho c) in W/cm^2 (metrics.py:155-157)."""
    return float(pressure_pa ** 2 / (2.0 * rho * c) / 1e4)


def pml_edge_distance(voxel_grid, frame: FieldFrame) -> int:
    """Voxels to the nearest sponge face (metrics.py:171-184)."""
    pml = frame.pml_vox
    return min(min(int(i) - pml, (n - pml - 1) - int(i)) for i, n in zip(voxel_grid, frame.grid_shape))


def a2_edge_warning(distance_vox: int) -> str:
    """Caveat for an a2 maximum on the absorber (metrics.py:187-193); the text is part of the output."""
    return (
        f"the a2 peak lies {distance_vox} voxels from the PML edge "
        f"(< {A2_PML_MARGIN_WARN_VOX}) — likely a harmonic-DFT edge artifact rather "
        f"than physics (an edge residue grows LINEARLY with drive, a real second "
        f"harmonic quadratically); a2_at_fundamental_peak_pa is the trustworthy number."
    )


def _query(org, shape, frame: FieldFrame) -> _lib.FocusInput:
    if len(shape) != 3:
        raise ValueError(f"focal metrics need a 3-D record region, got shape {tuple(shape)}")
    box = _interior(org, shape, frame)
    q = _lib.FocusInput()
    for a in range(3):
        q.shape[a] = int(shape[a])
        q.lo[a], q.hi[a] = box[a].start, box[a].stop
        q.offset[a] = int(org[a]) - int(frame.apex_vox[a])
        q.probe[a] = -1
    if frame.focus_vox is not None:
        t = [int(f) - o for f, o in zip(frame.focus_vox, org)]
        if all(0 <= i < n for i, n in zip(t, shape)):
            for a in range(3):
                q.probe[a] = t[a]
    q.dx = float(frame.dx)
    return q


def _extent(rep, a) -> dict:
    if rep.truncated[a]:
        return {"left_mm": None, "right_mm": None, "width_mm": None, "truncated": True}
    left, right = rep.left[a], rep.right[a]
    return {"left_mm": round(left * 1e3, 3), "right_mm": round(right * 1e3, 3),
            "width_mm": round((right - left) * 1e3, 3), "truncated": False}


def _assemble(rep: _lib.FocusReport, result, frame: FieldFrame, org, shape, *, source_amplitude, medium,
              solver) -> dict:
    dx = frame.dx
    pk = np.unravel_index(int(rep.peak), shape)
    pk_g = tuple(int(i) + o for i, o in zip(pk, org))
    p_peak = float(np.float32(rep.p_peak))
    isppa = None
    if medium is not None:
        isppa = round(intensity_w_cm2(p_peak, float(medium.rho[pk_g]), float(medium.c[pk_g])), 1)
    pos = {k: round(float((int(pk[a]) + org[a] - frame.apex_vox[a]) * dx) * 1e3, 3) for a, k in enumerate("xyz")}
    m: dict = {"peak": {
        "p_pa": round(p_peak, 1),
        "p_mpa": round(p_peak / 1e6, 4),
        "voxel_grid": [int(i) for i in pk_g],
        "position_mm_from_apex": pos,
        "gain_vs_source": None if source_amplitude is None else round(p_peak / source_amplitude, 2),
        "isppa_w_cm2": isppa,
        "p_max_time_domain_pa": round(float(np.float32(rep.p_max_at_peak)), 1),
    }}
    focus = frame.focus_vox
    if focus is not None:
        pt = float(np.float32(rep.p_probe))
        m["target"] = {
            "voxel_grid": [int(i) for i in focus],
            "p_pa": None if np.isnan(pt) else round(pt, 1),
            "hit_ratio": None if np.isnan(pt) else round(pt / p_peak, 4),
            "displacement_mm": {k: round((pk_g[a] - focus[a]) * dx * 1e3, 3) for a, k in enumerate("xyz")},
            "displacement_norm_mm": round(float(np.linalg.norm(np.array(pk_g) - np.array(focus)) * dx * 1e3), 3),
        }
    m["focal_spot"] = {
        "axial_6db": _extent(rep, 2),
        "lateral_x_6db": _extent(rep, 0),
        "lateral_y_6db": _extent(rep, 1),
        "volume_above_6db_mm3": round(float(int(rep.n_above_half) * (dx * 1e3) ** 3), 3),
    }
    m["run"] = {
        "solver": solver if solver is not None else str(result.meta.get("solver", "")),
        "dt_s": result.dt,
        "steps_per_period": result.spp,
        "steps_total": result.steps_total,
        "t_end_us": round(result.t_end_s * 1e6, 3),
        "tof_periods": result.tof_periods,
        "converged_period": result.converged_period,
        "settle_capped": bool(result.settle_capped),
        "harmonics_recorded": sorted(result.phasors),
    }
    warns: list[str] = []
    if rep.has_a2:
        a2_pk = float(np.float32(rep.a2_at_peak))
        pk2 = np.unravel_index(int(rep.a2_peak_index), shape)
        pk2_g = tuple(int(i) + o for i, o in zip(pk2, org))
        edge = pml_edge_distance(pk2_g, frame)
        m["harmonics"] = {
            "a2_at_fundamental_peak_pa": round(a2_pk, 1),
            "a2_over_a1_at_peak_pct": round(100.0 * a2_pk / p_peak, 2),
            "a2_peak_pa": round(float(np.float32(rep.a2_peak)), 1),
            "a2_peak_voxel_grid": [int(i) for i in pk2_g],
            "a2_peak_distance_to_pml_vox": edge,
        }
        if edge < A2_PML_MARGIN_WARN_VOX:
            warns.append(a2_edge_warning(edge))
    m["warnings"] = warns
    return m


def focus_metrics(result, frame: FieldFrame, *, source_amplitude: float | None = None, medium: Any | None = None,
                  solver: str | None = None) -> dict:
    """All scalar focal metrics of one run (metrics.py:192-313), reduced on the GPU.

    ``result`` is a ``SolverResult`` (host phasors; they are copied to the
    device once). Without ``frame.focus_vox`` there is no ``target``
    section, without ``medium`` no ISPPA, as in the reference.
    """
    org = region_origin(result)
    p1 = np.ascontiguousarray(result.phasors.get(1, result.phasor) if result.phasors else result.phasor,
                              np.complex64)
    shape = p1.shape
    q = _query(org, shape, frame)
    bufs = [_lib.DeviceArray.from_host(p1)]
    q.p1 = bufs[0].ptr
    if result.phasors and 2 in result.phasors:
        bufs.append(_lib.DeviceArray.from_host(np.ascontiguousarray(result.phasors[2], np.complex64)))
        q.p2 = bufs[-1].ptr
    bufs.append(_lib.DeviceArray.from_host(np.ascontiguousarray(result.p_max, np.float32)))
    q.pmax = bufs[-1].ptr
    rep = _lib.FocusReport()
    try:
        _lib.call("cg_focus_metrics", C.byref(q), C.byref(rep), None)
    finally:
        for b in bufs:
            b.close()
    return _assemble(rep, result, frame, org, shape, source_amplitude=source_amplitude, medium=medium,
                     solver=solver)


def device_focus_metrics(dev, member: int, result, frame: FieldFrame, *, source_amplitude: float | None = None,
                         medium: Any | None = None, solver: str | None = None) -> dict:
    """``focus_metrics`` on member ``member`` of a live ``DeviceSolver`` after its finalize.

    The field never leaves the device; ``result`` supplies the run section
    and the record region (it may hold its phasors or not).
    """
    org = region_origin(result)
    shape = tuple(int(h - l) for l, h in zip(dev.plan.rec_lo, dev.plan.rec_hi))
    if len(result.region) != 3:
        raise ValueError("focal metrics need a 3-D record region")
    q = _query(org, shape, frame)
    rep = _lib.FocusReport()
    _lib.call("cg_solver_focus_metrics", dev.h, int(member), C.byref(q), C.byref(rep))
    return _assemble(rep, result, frame, org, shape, source_amplitude=source_amplitude, medium=medium,
                     solver=solver)

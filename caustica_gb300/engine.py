"""Host orchestration of the GB300 CW solve over the C ABI.

Mirrors ``run_cw_kspace_pstd`` (reference solvers/kspace/engine.py:167-586):
the discretisation, padded maps, source scaling, settle bounds, convergence
and record regions and the settle / record loop semantics are the
reference's; every step runs in ``libcaustica_gb300.so``. Only host-side
set-up and the once-per-period bookkeeping live here.
"""

from __future__ import annotations

import ctypes as C
import logging
import os
import time
import warnings
from dataclasses import dataclass, field
from itertools import product
from math import ceil, floor, isfinite

import numpy as np

from . import _lib
from .contract import SolverDivergedError, SolverResult, ramp_envelope

log = logging.getLogger("caustica")


# ------------------------------------------------------------------ set-up --
def optimal_fft_size(n: int) -> int:
    """Smallest 2/3/5-smooth size >= n (operators.py:23-34)."""
    if n < 1:
        raise ValueError(f"n must be >= 1, got {n}")
    while True:
        m = n
        for p in (2, 3, 5):
            while m % p == 0:
                m //= p
        if m == 1:
            return n
        n += 1


def pad_shape(shape):
    return tuple(optimal_fft_size(n) for n in shape)


def pad_volume(vol: np.ndarray, padded) -> np.ndarray:
    """High-end edge replication (operators.py:42-57)."""
    pad = [(0, want - have) for have, want in zip(vol.shape, padded, strict=True)]
    if all(p == (0, 0) for p in pad):
        return vol
    return np.pad(vol, pad, mode="edge")


def cw_discretization(dx, c_max, f0, spec, harmonics=(1,)):
    """Exact-period (spp, dt) under the CFL limit (engine.py:86-113)."""
    period = 1.0 / f0
    dt_cfl = spec.cfl * dx / c_max
    spp = max(2, int(floor(period / dt_cfl)))
    dt = period / spp
    while dt * c_max / dx > spec.cfl_hard_max + 1e-12 and spp < 1024:
        spp += 1
        dt = period / spp
    h_max = max(harmonics)
    if 2 * h_max >= spp:
        raise ValueError(
            f"harmonic {h_max} is at/above the temporal Nyquist for spp={spp} "
            f"(need 2*h < spp); refine dx or lower cfl to raise spp."
        )
    return spp, dt


def cw_tof_periods(shape, dx, c_min, f0, indices, reference_point=None) -> int:
    """Periods of flight to the farthest corner or the reference (engine.py:116-134)."""
    period = 1.0 / f0
    src_pos = np.asarray(indices).astype(np.float64) * dx
    if reference_point is not None:
        refs = np.asarray(reference_point, np.float64)[None, :] * dx
    else:
        refs = np.array(list(product(*((0, n - 1) for n in shape))), np.float64) * dx
    dmax = max(float(np.sqrt(((src_pos - r) ** 2).sum(axis=1)).max()) for r in refs)
    return max(1, int(ceil(dmax / c_min / period)))


def normalize_record_region(region, shape):
    """engine.py:65-83."""
    if len(region) != len(shape):
        raise ValueError(f"record_region rank {len(region)} != grid rank {len(shape)}")
    out = []
    for sl, n_ax in zip(region, shape, strict=True):
        start, stop, step = sl.indices(n_ax)
        if step != 1:
            raise ValueError(f"record_region does not support strides, got {sl}")
        if stop <= start:
            raise ValueError(f"record_region slice {sl} is empty on an axis of {n_ax}")
        out.append(slice(start, stop))
    return tuple(out)


def material_coefficients(alpha, rho, c, beta, dt, nonlinear_active):
    """(dt/rho, rho c^2 dt, exp(-alpha c dt), 2 beta dt) with the reference's
    float32 host arithmetic (engine.py:239-249)."""
    alpha = np.asarray(alpha, np.float32)
    rho = np.asarray(rho, np.float32)
    c = np.asarray(c, np.float32)
    beta = np.asarray(beta, np.float32)
    dtr = np.asarray(dt / rho, dtype=np.float32)
    rc2 = np.asarray(rho * c.astype(np.float64) ** 2 * dt, dtype=np.float32)
    ab = np.asarray(np.exp(-(alpha * c) * dt), dtype=np.float32)
    b2 = np.asarray(beta * (2.0 * dt), dtype=np.float32) if nonlinear_active else np.zeros_like(dtr)
    return dtr, rc2, ab, b2


def _first_occurrence(inv: np.ndarray, n: int, chunk: int = 1 << 20) -> np.ndarray:
    """Index of the first element equal to each label 0..n-1 (chunked scan)."""
    first = np.full(n, -1, np.int64)
    missing = n
    for s0 in range(0, inv.size, chunk):
        part = inv[s0:s0 + chunk]
        for lab in np.flatnonzero(np.bincount(part, minlength=n)[:n] > 0):
            if first[lab] < 0:
                first[lab] = s0 + int(np.argmax(part == lab))
                missing -= 1
        if missing == 0:
            break
    return first


def _uniform(flat) -> bool:
    """Every volume bitwise equal to its own first value, checked in chunks on
    a few host threads (the NumPy compares release the GIL)."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    bits = [f.view(np.uint32) for f in flat]
    first = [b[0] for b in bits]
    n = bits[0].size
    nt = max(1, min(8, os.cpu_count() or 1))
    step = max(1 << 18, (n + 4 * nt - 1) // (4 * nt))

    def chunk(a):
        b = min(n, a + step)
        return all(not np.any(x[a:b] != v) for x, v in zip(bits, first))

    if n <= step:
        return chunk(0)
    with ThreadPoolExecutor(nt) as ex:
        return all(ex.map(chunk, range(0, n, step)))


# material counts up to which label_volumes assigns labels by direct
# comparison scans (one pass per material) instead of sorting every cell
_SCAN_MATERIALS = 24


def _scan_labels(bits, rows: np.ndarray):
    """Labels by comparison: every cell gets the index of the row of
    ``rows`` (value tuples as uint32 bit patterns) it equals bit for bit;
    tuples absent from ``rows`` are appended in order of first occurrence.
    Chunks run on a few host threads. None past _SCAN_MATERIALS rows."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    n = bits[0].size
    inv = np.full(n, 255, np.uint8)
    rows = [tuple(int(x) for x in r) for r in rows]
    nt = max(1, min(8, os.cpu_count() or 1))
    step = max(1 << 18, (n + 4 * nt - 1) // (4 * nt))

    def assign(a, first_row):
        b = min(n, a + step)
        part = inv[a:b]
        for m in range(first_row, len(rows)):
            eq = bits[0][a:b] == np.uint32(rows[m][0])
            for f, v in zip(bits[1:], rows[m][1:]):
                eq &= f[a:b] == np.uint32(v)
            part[eq & (part == 255)] = m

    first_row = 0
    while True:
        with ThreadPoolExecutor(nt) as ex:
            list(ex.map(lambda a: assign(a, first_row), range(0, n, step)))
        left = np.flatnonzero(inv == 255)
        if left.size == 0:
            break
        if len(rows) >= _SCAN_MATERIALS:
            return None
        first_row = len(rows)
        rows.append(tuple(int(f[left[0]]) for f in bits))
    props = np.array(rows, np.uint32).view(np.float32).reshape(len(rows), len(bits))
    return inv, props.copy()


def _labels_match(props: np.ndarray, inv: np.ndarray, vols) -> bool:
    """props[inv] == vols bit for bit, checked in chunks on a few host threads
    (the NumPy gathers and compares release the GIL)."""
    import os
    from concurrent.futures import ThreadPoolExecutor

    flat = [v.reshape(-1).view(np.uint32) for v in vols]
    luts = [np.ascontiguousarray(props[:, i]).view(np.uint32) for i in range(len(vols))]
    n = inv.size
    nt = max(1, min(8, os.cpu_count() or 1))
    step = max(1 << 16, (n + 4 * nt - 1) // (4 * nt))

    def chunk(a):
        b = min(n, a + step)
        return all(np.array_equal(np.take(lut, inv[a:b]), f[a:b]) for lut, f in zip(luts, flat))

    if n <= step:
        return chunk(0)
    with ThreadPoolExecutor(nt) as ex:
        return all(ex.map(chunk, range(0, n, step)))


def label_volumes(vols, id_map=None, max_labels: int = 256):
    """Exact label decomposition of equally shaped float32 volumes.

    Returns ``(labels uint8, props (n, len(vols)) float32)`` when at most
    ``max_labels`` distinct value tuples occur (``props[labels] == vols``),
    else None. An integer ``id_map`` is tried first (O(N)); ids spanning at
    most ``max_labels`` values become labels directly (id - min), the rows
    of ids that do not occur repeat an occurring row.
    """
    vols = [np.ascontiguousarray(v, np.float32) for v in vols]
    nv = len(vols)
    if id_map is not None:
        ids_flat = np.asarray(id_map).reshape(-1)
        if ids_flat.size == vols[0].size and ids_flat.dtype.kind in "iu":
            lo, hi = int(ids_flat.min()), int(ids_flat.max())
            if hi - lo < max_labels:
                inv = (ids_flat - lo).astype(np.uint8) if lo else ids_flat.astype(np.uint8)
                n = hi - lo + 1
                first = _first_occurrence(inv, n)
                first[first < 0] = first[first >= 0][0]
                props = np.stack([v.reshape(-1)[first] for v in vols], axis=1).astype(np.float32)
                if _labels_match(props, inv, vols):
                    return inv.reshape(vols[0].shape), props
            elif hi - lo < (1 << 20):
                present = np.flatnonzero(np.bincount(ids_flat - lo, minlength=hi - lo + 1))
                if len(present) <= max_labels:
                    lut = np.zeros(hi - lo + 1, np.uint8)
                    lut[present] = np.arange(len(present))
                    inv = lut[ids_flat - lo]
                    first = _first_occurrence(inv, len(present))
                    props = np.stack([v.reshape(-1)[first] for v in vols], axis=1).astype(np.float32)
                    if _labels_match(props, inv, vols):
                        return inv.reshape(vols[0].shape), props
    flat = [v.reshape(-1) for v in vols]
    if _uniform(flat):
        return (np.zeros(vols[0].shape, np.uint8),
                np.array([[f[0] for f in flat]], np.float32))
    stride = max(1, flat[0].size // 4096)
    for f in flat:
        if len(np.unique(f.view(np.uint32)[::stride])) > max_labels:
            return None
    sample = np.unique(np.stack([f.view(np.uint32)[::stride] for f in flat], axis=1), axis=0)
    if len(sample) <= _SCAN_MATERIALS:
        got = _scan_labels([f.view(np.uint32) for f in flat], sample)
        if got is not None:
            inv, props = got
            return inv.reshape(vols[0].shape), props
    bits = [f.view(np.uint32).astype(np.uint64) for f in flat]
    keys = [(bits[i] << np.uint64(32)) | (bits[i + 1] if i + 1 < nv else np.uint64(0)) for i in range(0, nv, 2)]
    code = None
    for k in keys:
        u, inv_k = np.unique(k, return_inverse=True)
        if len(u) > max_labels:
            return None
        code = inv_k.astype(np.int64) if code is None else code * len(u) + inv_k
    u, inv = np.unique(code, return_inverse=True)
    if len(u) > max_labels:
        return None
    first = _first_occurrence(inv, len(u))
    props = np.stack([f[first] for f in flat], axis=1).astype(np.float32)
    return inv.astype(np.uint8).reshape(vols[0].shape), props


def label_medium(medium, max_labels: int = 256):
    """Labels of the acoustic property volumes (alpha, rho, c, beta), or None.

    A medium built by ``Medium.from_labels`` carries its decomposition with
    read-only maps; it is used as it is while the medium still holds those
    very arrays (nothing can have changed them). Any other medium is
    decomposed and verified against its maps."""
    vols = [getattr(medium, k) for k in ("alpha", "rho", "c", "beta")]
    cached = getattr(medium, "_label_cache", None)
    if cached is not None:
        maps, labels, rows = cached
        if all(v is m for v, m in zip(vols, maps)) and not any(m.flags.writeable for m in maps):
            return labels, rows
    return label_volumes(vols, getattr(medium, "id_map", None), max_labels)


def _embed3(shape):
    """Map a 1/2/3-D active shape onto the solver's 3-D (x, y, z) frame."""
    nd = len(shape)
    return (1,) * (3 - nd) + tuple(shape)


@dataclass
class Plan:
    """Everything the device solve needs, derived once on the host."""

    name: str
    shape: tuple
    padded: tuple
    padded3: tuple
    nd: int
    dx: float
    spp: int
    dt: float
    f0: float
    omega: float
    period: float
    c_max: float
    nonlinear_active: bool
    harmonics: tuple
    tof: int
    eff_min: int
    eff_max: int
    spec: object
    rec: tuple
    rec_lo: tuple
    rec_hi: tuple
    conv_lo: tuple
    conv_hi: tuple
    pml3: tuple
    pml_edge: float
    src_xyz: np.ndarray
    src_scale: np.ndarray
    src_phase: np.ndarray
    amplitude: float
    ramp_periods: float
    labels: np.ndarray | None = None
    label_table: np.ndarray | None = None
    label_props: np.ndarray | None = None  # (n, 4) float32 alpha, rho, c, beta per label
    labels_dev: object | None = None  # device label map (a device.DeviceView) instead of host labels
    dense: tuple | None = None
    label: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def extra_periods_cap(self) -> int:
        if self.spec.t_end_min_us is None:
            return 0
        need = ceil(self.spec.t_end_min_us * 1e-6 / self.period) - self.spec.n_record_periods
        return max(0, need)

    @property
    def max_periods(self) -> int:
        return max(self.eff_max, self.extra_periods_cap) + self.spec.n_record_periods + 2

    @property
    def ncell(self) -> int:
        return int(np.prod(self.padded3))

    def drive_table(self, n_steps: int | None = None) -> np.ndarray:
        """(amp ramp(t), sin wt, cos wt, 0) per step (engine.py:478-482, sources.py:98-102)."""
        n_steps = self.max_periods * self.spp if n_steps is None else int(n_steps)
        out = np.zeros((n_steps, 4), np.float32)
        for n in range(n_steps):
            t = n * self.dt
            env = ramp_envelope(t, self.period, self.ramp_periods)
            out[n, 0] = np.float32(self.amplitude * env)
            wt = self.omega * t
            out[n, 1] = np.sin(wt)
            out[n, 2] = np.cos(wt)
        return out

    def source_amplitudes(self, phases: np.ndarray | None = None) -> tuple[np.ndarray, np.ndarray]:
        """(2 c dt/dx) cos/sin(phase) per member and voxel, float32 [B][S]."""
        ph = self.src_phase[None, :] if phases is None else np.atleast_2d(np.asarray(phases, np.float32))
        sc = self.src_scale.astype(np.float64)[None, :]
        ph64 = ph.astype(np.float64)
        return (np.ascontiguousarray((sc * np.cos(ph64)).astype(np.float32)),
                np.ascontiguousarray((sc * np.sin(ph64)).astype(np.float32)))


def make_plan(name, grid, medium, source, spec, *, record_region=None, reference_point=None,
              nonlinear=False, harmonics=(1,)) -> Plan:
    """Host set-up of one solve (engine.py:211-301)."""
    harmonics = tuple(dict.fromkeys(int(h) for h in harmonics))
    if not harmonics or harmonics[0] != 1 or any(h < 1 for h in harmonics):
        raise ValueError(f"harmonics must start with 1 (fundamental), got {harmonics}")
    if len(harmonics) > 8:
        raise ValueError("at most 8 harmonics per solve")
    shape = tuple(int(s) for s in grid.shape)
    nd = len(shape)
    if reference_point is not None:
        ref = tuple(reference_point)
        if len(ref) != nd or any(not float(r).is_integer() or not 0 <= int(r) < n
                                 for r, n in zip(ref, shape, strict=True)):
            raise ValueError(f"reference_point must be integer VOXEL indices inside {shape}, "
                             f"got {reference_point} (did you pass meters?)")
    dx = float(grid.dx)
    device_medium = hasattr(medium, "labels_at")  # a device.DeviceLabelMedium
    c_max = medium.c_max if device_medium else float(np.max(medium.c))
    c_min = medium.c_min if device_medium else float(np.min(medium.c))
    spp, dt = cw_discretization(dx, c_max, source.f0, spec, harmonics)
    padded = pad_shape(shape)
    padded3 = _embed3(padded)
    pml_vox = int(grid.pml_vox)
    pml_edge = float(grid.pml.edge) if getattr(grid, "pml", None) is not None else 2.0
    if grid.pml_vox == 0:
        log.warning("grid has no PML: the FFT domain is PERIODIC and waves wrap around.")
    for n in padded:
        if 2 * pml_vox > n:
            raise ValueError(f"sponge width {pml_vox} does not fit twice into length {n}")
    pml3 = (0,) * (3 - nd) + (pml_vox,) * nd
    if device_medium:
        return _device_medium_plan(name, grid, medium, source, spec, record_region=record_region,
                                   reference_point=reference_point, nonlinear=nonlinear, harmonics=harmonics,
                                   shape=shape, padded=padded, padded3=padded3, dx=dx, spp=spp, dt=dt,
                                   c_max=c_max, c_min=c_min, pml3=pml3, pml_edge=pml_edge, pml_vox=pml_vox)
    beta = np.asarray(medium.beta, np.float32)
    nonlinear_active = bool(nonlinear) and not bool((beta == 0).all())

    # medium: exact labels when few materials, else dense float32 maps
    labels = table = dense = props = None
    lab = label_medium(medium)
    if lab is not None:
        lab_vol, props = lab
        dtr, rc2, ab, b2 = material_coefficients(props[:, 0], props[:, 1], props[:, 2], props[:, 3], dt,
                                                 nonlinear_active)
        table = np.ascontiguousarray(np.stack([dtr, rc2, ab, b2], axis=1).astype(np.float32))
        labels = np.ascontiguousarray(pad_volume(lab_vol, padded).reshape(padded3))
    else:
        maps = material_coefficients(pad_volume(np.asarray(medium.alpha, np.float32), padded),
                                     pad_volume(np.asarray(medium.rho, np.float32), padded),
                                     pad_volume(np.asarray(medium.c, np.float32), padded),
                                     pad_volume(beta, padded), dt, nonlinear_active)
        dense = tuple(np.ascontiguousarray(m.reshape(padded3)) for m in maps)

    idx = np.asarray(source.indices, np.int64)
    c_src = np.asarray(medium.c, np.float32)[tuple(idx[:, d] for d in range(nd))]
    return _finish_plan(name, grid, source, spec, record_region=record_region, reference_point=reference_point,
                        harmonics=harmonics, shape=shape, padded=padded, padded3=padded3, dx=dx, spp=spp, dt=dt,
                        c_max=c_max, c_min=c_min, pml3=pml3, pml_edge=pml_edge, pml_vox=pml_vox,
                        nonlinear_active=nonlinear_active, idx=idx, c_src=c_src, labels=labels, table=table,
                        props=props, dense=dense)


def _device_medium_plan(name, grid, medium, source, spec, *, record_region, reference_point, nonlinear, harmonics,
                        shape, padded, padded3, dx, spp, dt, c_max, c_min, pml3, pml_edge, pml_vox) -> "Plan":
    """Plan over a label map that stays on the device (device.DeviceLabelMedium):
    the per-label coefficient table is formed on the host from the rows of
    the labels that occur, and the map itself goes device to device into the
    solver."""
    if tuple(padded) != tuple(shape):
        raise ValueError(f"a device label map needs a 2/3/5-smooth grid (got {shape}, the FFT size would be "
                         f"{padded}); pad it on the device first")
    nonlinear_active = bool(nonlinear) and not medium.is_linear
    present = medium.present
    n_lab = int(present.max()) + 1
    rows = np.array(medium.rows[:n_lab], np.float32)
    rows[np.setdiff1d(np.arange(n_lab), present)] = rows[present[0]]  # absent labels: any valid row
    dtr, rc2, ab, b2 = material_coefficients(rows[:, 0], rows[:, 1], rows[:, 2], rows[:, 3], dt, nonlinear_active)
    table = np.ascontiguousarray(np.stack([dtr, rc2, ab, b2], axis=1).astype(np.float32))
    idx = np.asarray(source.indices, np.int64)
    c_src = rows[medium.labels_at(idx).astype(np.int64), 2]
    plan = _finish_plan(name, grid, source, spec, record_region=record_region, reference_point=reference_point,
                        harmonics=harmonics, shape=shape, padded=padded, padded3=padded3, dx=dx, spp=spp, dt=dt,
                        c_max=c_max, c_min=c_min, pml3=pml3, pml_edge=pml_edge, pml_vox=pml_vox,
                        nonlinear_active=nonlinear_active, idx=idx, c_src=c_src, labels=None, table=table,
                        props=rows, dense=None)
    plan.labels_dev = medium.labels
    plan.meta["present_labels"] = present
    return plan


def _finish_plan(name, grid, source, spec, *, record_region, reference_point, harmonics, shape, padded, padded3,
                 dx, spp, dt, c_max, c_min, pml3, pml_edge, pml_vox, nonlinear_active, idx, c_src, labels, table,
                 props, dense) -> "Plan":
    nd = len(shape)
    src_scale = np.asarray(2.0 * c_src.astype(np.float64) * dt / dx, dtype=np.float32)
    src_xyz = np.zeros((idx.shape[0], 3), np.int32)
    src_xyz[:, 3 - nd:] = idx

    tof = cw_tof_periods(shape, dx, c_min, source.f0, idx, reference_point)
    eff_min = tof + max(spec.min_settle_periods, int(ceil(source.ramp_periods)) + 1)
    eff_max = max(tof + spec.max_settle_periods, eff_min)
    margin = pml_vox + 2
    if any(n <= 2 * margin for n in shape):
        margin = 0
    conv_lo = (0,) * (3 - nd) + (margin,) * nd
    conv_hi = (1,) * (3 - nd) + tuple(n - margin for n in shape)
    active = tuple(slice(0, n) for n in shape)
    rec = normalize_record_region(record_region, shape) if record_region is not None else active
    rec_lo = (0,) * (3 - nd) + tuple(s.start for s in rec)
    rec_hi = (1,) * (3 - nd) + tuple(s.stop for s in rec)
    return Plan(
        name=name, shape=shape, padded=padded, padded3=padded3, nd=nd, dx=dx, spp=spp, dt=dt, f0=source.f0,
        omega=2.0 * np.pi * source.f0, period=1.0 / source.f0, c_max=c_max, nonlinear_active=nonlinear_active,
        harmonics=harmonics, tof=tof, eff_min=eff_min, eff_max=eff_max, spec=spec, rec=rec, rec_lo=rec_lo,
        rec_hi=rec_hi, conv_lo=conv_lo, conv_hi=conv_hi, pml3=pml3, pml_edge=pml_edge, src_xyz=src_xyz,
        src_scale=src_scale, src_phase=np.asarray(source.phases, np.float32), amplitude=float(source.amplitude),
        ramp_periods=float(source.ramp_periods), labels=labels, label_table=table, label_props=props,
        dense=dense,
        label=getattr(source, "label", ""),
        meta={"reference_point": None if reference_point is None else [int(r) for r in reference_point]},
    )


def device_footprint(plan: "Plan", batch: int) -> int:
    """Device bytes of one solver handle (the serving loop's admission
    estimate; the record accumulators are counted although they are only
    allocated at the record window)."""
    nx, ny, nz = plan.padded3
    ncell = nx * ny * nz
    nspec = nx * (nz // 2 + 1) * ny
    nrec = int(np.prod([h - l for l, h in zip(plan.rec_lo, plan.rec_hi)]))
    per_member = 16 * ncell + 24 * nspec + 8 * plan.spp * nrec + 4 * nrec + 8 * len(plan.harmonics) * nrec
    medium = ncell if (plan.labels is not None or plan.labels_dev is not None) else 16 * ncell
    return batch * per_member + medium + 16 * plan.max_periods * plan.spp + (64 << 10)


# ----------------------------------------------------------------- device --
class DeviceSolver:
    """One ``cg_solver`` handle: B right-hand sides over one medium."""

    def __init__(self, plan: Plan, batch: int = 1, phases: np.ndarray | None = None, autotune: bool | None = None):
        self.plan = plan
        self.batch = int(batch)
        lib = _lib.load()
        cfg = _lib.SolverConfig()
        cfg.nx, cfg.ny, cfg.nz = plan.padded3
        cfg.batch = self.batch
        cfg.nonlinear = int(plan.nonlinear_active)
        cfg.spp = plan.spp
        cfg.max_periods = plan.max_periods
        cfg.n_harmonics = len(plan.harmonics)
        for i, h in enumerate(plan.harmonics):
            cfg.harmonics[i] = h
        for i in range(3):
            cfg.pml[i] = plan.pml3[i]
            cfg.rec_lo[i], cfg.rec_hi[i] = plan.rec_lo[i], plan.rec_hi[i]
            cfg.conv_lo[i], cfg.conv_hi[i] = plan.conv_lo[i], plan.conv_hi[i]
        cfg.pml_edge = plan.pml_edge
        cfg.dx, cfg.dt, cfg.c_ref = plan.dx, plan.dt, plan.c_max
        h = C.c_void_p()
        _lib.check(lib.cg_solver_create(C.byref(cfg), C.byref(h)), "cg_solver_create")
        self.h = h
        try:
            if plan.labels_dev is not None:  # device label map: copied device to device
                _lib.call("cg_solver_set_medium_labels", h, plan.labels_dev.ptr, len(plan.label_table),
                          _lib.ptr(plan.label_table))
            elif plan.labels is not None:
                _lib.call("cg_solver_set_medium_labels", h, _lib.ptr(plan.labels), len(plan.label_table),
                          _lib.ptr(plan.label_table))
            else:
                dtr, rc2, ab, b2 = plan.dense
                _lib.call("cg_solver_set_medium_dense", h, _lib.ptr(dtr), _lib.ptr(rc2), _lib.ptr(ab),
                          _lib.ptr(b2) if plan.nonlinear_active else None)
            self.set_phases(phases)
            self.drive = plan.drive_table()
            _lib.call("cg_solver_set_drive", h, len(self.drive), _lib.ptr(self.drive))
        except Exception:
            self.close()
            raise
        self.tuning = None
        if autotune is None:
            autotune = os.environ.get("CG_AUTOTUNE", "1") != "0"
        if autotune:
            # launch configuration timed on this (fresh) handle, remembered per shape
            out = np.zeros(4, np.int32)
            # a large batch's step is long enough to time in one step per trial
            _lib.call("cg_solver_autotune", h, 4 if self.batch < 8 else 1, _lib.ptr(out))
            cfg4 = np.zeros(4, np.int32)
            _lib.call("cg_solver_get_config", h, _lib.ptr(cfg4))
            self.tuning = {"fused_transverse": bool(out[0]), "persistent_z": bool(out[1]), "slabs": int(cfg4[2]),
                           "tma_staging": self._zstaging(), "configurations_timed": int(out[2]),
                           "cached": bool(out[3])}
        info = np.zeros(8, np.int64)
        _lib.call("cg_solver_info", h, _lib.ptr(info))
        self.nrec = int(info[2])
        self.launches_per_step = int(info[7])

    def set_phases(self, phases: np.ndarray | None) -> None:
        ac, as_ = self.plan.source_amplitudes(phases)
        if ac.shape[0] == 1 and self.batch > 1:
            ac = np.ascontiguousarray(np.repeat(ac, self.batch, axis=0))
            as_ = np.ascontiguousarray(np.repeat(as_, self.batch, axis=0))
        if ac.shape[0] != self.batch:
            raise ValueError(f"phases for {ac.shape[0]} members given to a batch of {self.batch}")
        xyz = np.ascontiguousarray(self.plan.src_xyz)
        _lib.call("cg_solver_set_source", self.h, int(xyz.shape[0]), _lib.ptr(xyz), _lib.ptr(ac), _lib.ptr(as_))

    def set_slabs(self, k: int) -> None:
        """Run the plane-local passes in ``k`` x-slabs (1: the plain step); bit-identical results."""
        _lib.call("cg_solver_set_slabs", self.h, int(k))
        info = np.zeros(8, np.int64)
        _lib.call("cg_solver_info", self.h, _lib.ptr(info))
        self.launches_per_step = int(info[7])

    def set_zstaging(self, tma: bool) -> None:
        """Stage the persistent z-tiles by tensor-map copies (True) or cp.async (False); bit-identical results."""
        _lib.call("cg_solver_set_zstaging", self.h, int(bool(tma)))

    def _zstaging(self) -> bool:
        v = C.c_int(0)
        _lib.call("cg_solver_get_zstaging", self.h, C.byref(v))
        return bool(v.value)

    def config(self) -> dict:
        out = np.zeros(4, np.int32)
        _lib.call("cg_solver_get_config", self.h, _lib.ptr(out))
        return {"fused_transverse": bool(out[0]), "persistent_z": bool(out[1]), "slabs": int(out[2]),
                "launches_per_step": int(out[3]), "tma_staging": self._zstaging()}

    def extend_drive(self, n_steps: int) -> None:
        """Drive table covering ``n_steps`` steps (the default covers one solve's schedule)."""
        self.drive = self.plan.drive_table(n_steps)
        _lib.call("cg_solver_set_drive", self.h, len(self.drive), _lib.ptr(self.drive))

    def close(self) -> None:
        if getattr(self, "h", None):
            _lib.load().cg_solver_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):  # pragma: no cover - best effort
        try:
            self.close()
        except Exception:
            pass

    # thin wrappers
    def reset(self):
        _lib.call("cg_solver_reset", self.h)

    def run_periods(self, n: int, record: bool = False, graph: bool = True):
        if n <= 0:
            return
        if graph:
            _lib.call("cg_solver_run_periods", self.h, int(n), int(record))
        else:
            _lib.call("cg_solver_run", self.h, int(n) * self.plan.spp, int(record))

    def run_steps(self, n: int, record: bool = False):
        _lib.call("cg_solver_run", self.h, int(n), int(record))

    def begin_record(self):
        _lib.call("cg_solver_begin_record", self.h)

    def read_peaks(self, first: int, count: int) -> np.ndarray:
        out = np.zeros((self.batch, count), np.float32)
        if count:
            _lib.call("cg_solver_read_peaks", self.h, int(first), int(count), _lib.ptr(out))
        return out

    def finalize(self, n_record_steps: int):
        nh = len(self.plan.harmonics)
        ph = np.zeros((self.batch, nh, self.nrec), np.complex64)
        pm = np.zeros((self.batch, self.nrec), np.float32)
        _lib.call("cg_solver_finalize", self.h, int(n_record_steps), _lib.ptr(ph), _lib.ptr(pm))
        return ph, pm

    def synchronize(self):
        _lib.call("cg_solver_synchronize", self.h)

    def idle(self) -> bool:
        """True when all queued work on this solver's stream has finished (non-blocking)."""
        flag = C.c_int(0)
        _lib.call("cg_solver_query", self.h, C.byref(flag))
        return bool(flag.value)

    def footprint_bytes(self) -> int:
        """Device bytes this handle holds (state, spectra, medium, record buffers)."""
        return device_footprint(self.plan, self.batch)

    def get_state(self):
        n = self.plan.ncell
        p = np.zeros((self.batch, n), np.float32)
        u = np.zeros((3, self.batch, n), np.float32)
        _lib.call("cg_solver_get_state", self.h, _lib.ptr(p), _lib.ptr(u))
        return p, u

    def set_state(self, p: np.ndarray, u: np.ndarray, step: int = 0):
        p = np.ascontiguousarray(p, np.float32)
        u = np.ascontiguousarray(u, np.float32)
        _lib.call("cg_solver_set_state", self.h, _lib.ptr(p), _lib.ptr(u), int(step))


# ------------------------------------------------------------------- solve --
def _guard_finite(peak: float, where: str, solver_name: str) -> None:
    """engine.py:137-164."""
    if isfinite(peak):
        return
    raise SolverDivergedError(
        f"solver '{solver_name}' diverged during {where}: the peak pressure is {peak}, so the field is no "
        f"longer finite. Nothing downstream of this point is a physical result. Usual causes, most common "
        f"first: a time step the scheme cannot integrate for this medium (check the CFL and "
        f"points-per-wavelength of the fastest material), a drive amplitude far outside the range float32 "
        f"can carry, a medium with a non-physical sound speed or density, or a source sitting in or against "
        f"the PML band, where it is damped as fast as it is driven."
    )


def _settle(dev: DeviceSolver, plan: Plan, progress, member: int = 0, t0: float | None = None):
    """Settle loop with the reference's decisions (engine.py:484-510), one batch member's view.

    Periods are launched in runs; the host synchronises only where a decision
    needs the period peak (convergence armed and tol > 0, or a progress
    callback), so a fixed schedule runs without a host round trip.
    """
    spec = plan.spec
    eff_min, eff_max, tof = plan.eff_min, plan.eff_max, plan.tof
    tol = spec.convergence_tol
    prev_peak = None
    converged = False
    converged_period = eff_max
    history = []
    period_idx = 0
    launched = 0
    all_peaks = []
    while not converged and period_idx < eff_max:
        if progress is not None:
            target = period_idx + 1
        elif tol > 0:
            target = max(period_idx + 1, min(eff_max, eff_min))
        else:
            target = eff_max
        if launched < target:
            dev.run_periods(target - launched, record=False)
            launched = target
        peaks = dev.read_peaks(period_idx, target - period_idx)
        for j in range(target - period_idx):
            period_idx += 1
            peak = float(peaks[member, j])
            all_peaks.append(peaks[:, j].copy())
            _guard_finite(peak, f"settling period {period_idx} (step {period_idx * plan.spp})", plan.name)
            rel = abs(peak - prev_peak) / max(prev_peak, 1e-9) if prev_peak is not None else None
            if period_idx >= tof:
                history.append((period_idx, peak, float("nan") if rel is None else rel))
            if period_idx >= eff_min and rel is not None:
                if peak > 0.0 and rel < tol:
                    converged_period = period_idx
                    converged = True
            if not converged:
                prev_peak = peak
            if progress is not None:
                _emit(progress, plan, dev, "settle", period_idx, peak, rel, t0)
            if converged:
                break
    return period_idx, converged, converged_period, history, all_peaks


_progress_warned = [False]


def _emit(progress, plan, dev, stage, period, peak, rel, t0):
    """One payload per period boundary (engine.py:401-434)."""
    periods_expected = max(plan.eff_max, plan.extra_periods_cap) + plan.spec.n_record_periods
    steps_expected = periods_expected * plan.spp
    n = period * plan.spp
    elapsed = time.monotonic() - (t0 or time.monotonic())
    eta = round((steps_expected - n) * (elapsed / n), 1) if n > 0 and steps_expected > n else None

    def snapshot():
        if not getattr(dev, "h", None):
            raise RuntimeError("the solve has finished and released its device state; call snapshot() inside "
                               "the progress callback")
        p, _ = dev.get_state()
        vol = p[0].reshape(plan.padded3)[: 1 if plan.nd < 3 else plan.shape[0]]
        if plan.nd == 1:
            return vol[0, 0, : plan.shape[0]].copy()
        if plan.nd == 2:
            return vol[0, : plan.shape[0], : plan.shape[1]].copy()
        return vol[:, plan.shape[1] // 2, : plan.shape[2]].copy()

    try:
        progress({"period": period, "periods_expected": periods_expected, "step": n,
                  "steps_expected": steps_expected, "peak": peak, "converge_delta": rel,
                  "elapsed_s": round(elapsed, 3), "eta_s": eta, "stage": stage, "snapshot": snapshot})
    except Exception as exc:  # noqa: BLE001 - a widget must not kill a solve
        if not _progress_warned[0]:
            _progress_warned[0] = True
            warnings.warn(f"progress callback raised {type(exc).__name__}: {exc}. The solve continues; further "
                          f"progress failures are silent.", stacklevel=3)


def _results(plan: Plan, dev: DeviceSolver, ph, pm, common: dict, member: int, result_cls) -> SolverResult:
    rshape = tuple(s.stop - s.start for s in plan.rec)
    phasors = {h: ph[member, i].reshape(rshape) for i, h in enumerate(plan.harmonics)}
    return result_cls(phasor=phasors[1], p_max=pm[member].reshape(rshape), region=plan.rec, phasors=phasors,
                      **common)


def member_schedule(peaks: np.ndarray, plan: Plan, name: str | None = None):
    """The settle decisions one member would take alone from its per-period
    peaks (engine.py:484-510): (periods run, converged, converged_period,
    history). Raises on the first non-finite peak."""
    spec = plan.spec
    prev = None
    hist = []
    for j, peak in enumerate(peaks, start=1):
        peak = float(peak)
        _guard_finite(peak, f"settling period {j} (step {j * plan.spp})", name or plan.name)
        rel = abs(peak - prev) / max(prev, 1e-9) if prev is not None else None
        if j >= plan.tof:
            hist.append((j, peak, float("nan") if rel is None else rel))
        if j >= plan.eff_min and rel is not None and peak > 0.0 and rel < spec.convergence_tol:
            return j, True, j, hist
        prev = peak
        if j >= plan.eff_max:
            break
    return len(peaks), False, plan.eff_max, hist


def solve(plan: Plan, *, progress=None, phases: np.ndarray | None = None, result_cls=SolverResult,
          dev: DeviceSolver | None = None, quantize: float | None = None):
    """Run the settle + record schedule; one result per batch member.

    With ``phases`` of shape (B, S) the B members share the medium and the
    voxel set and differ in their drive phases (steering). They run one
    shared schedule, decided by member 0; every other member's own decisions
    are replayed from its period peaks, and a member whose stand-alone run
    would have stopped settling at a different period is solved again on
    its own, so each result equals the one its solo run gives.

    ``quantize`` (a bound on the relative round-trip error) also quantises
    each member's stored fields on the device for the result store and
    attaches them as ``meta["quantized"]``.
    """
    t0 = time.monotonic()
    batch = 1 if phases is None else int(np.atleast_2d(phases).shape[0])
    own = dev is None
    if own:
        dev = DeviceSolver(plan, batch=batch, phases=phases)
    else:
        dev.reset()
        if phases is not None:
            dev.set_phases(phases)
    try:
        spec = plan.spec
        periods_done, converged, converged_period, history, all_peaks = _settle(dev, plan, progress, 0, t0)
        settle_periods = periods_done
        if spec.t_end_min_us is not None:
            need = ceil(spec.t_end_min_us * 1e-6 / plan.period) - spec.n_record_periods
            if periods_done < need:
                dev.run_periods(need - periods_done)
                periods_done = need
        if progress is not None:
            _emit(progress, plan, dev, "record", periods_done, None, None, t0)
        rec_steps = spec.n_record_periods * plan.spp
        dev.begin_record()
        dev.run_periods(spec.n_record_periods, record=True)
        ph, pm = dev.finalize(rec_steps)
        n = (periods_done + spec.n_record_periods) * plan.spp
        peaks = np.array(all_peaks).T if all_peaks else np.zeros((batch, 0), np.float32)  # (B, periods)
        results = []
        redo = []
        for b in range(batch):
            if b == 0:
                sched = (settle_periods, converged, converged_period, history)
            else:
                sched = member_schedule(peaks[b], plan)
                if sched[0] != settle_periods or sched[1] != converged:
                    redo.append(b)
                    results.append(None)
                    continue
            _guard_finite(float(pm[b].max()), f"the record window (step {n})", plan.name)
            common = dict(dt=plan.dt, spp=plan.spp, steps_total=n, t_end_s=n * plan.dt, tof_periods=plan.tof,
                          converged_period=sched[2], settle_capped=not sched[1], convergence_history=sched[3],
                          meta={"solver": plan.name, "backend": "gb300", "padded_shape": plan.padded,
                                "c_ref": plan.c_max, "nonlinear_active": plan.nonlinear_active,
                                "source": plan.label,
                                "medium_storage": "dense" if plan.dense is not None else "labels",
                                "batch": batch, "member": b})
            results.append(_results(plan, dev, ph, pm, common, b, result_cls))
            if quantize is not None:
                from .store import quantize_solver

                tq = time.perf_counter()
                fields = quantize_solver(dev, b, quantize)
                results[-1].meta["quantized"] = {"max_norm_err": float(quantize), "fields": fields,
                                                 "seconds": time.perf_counter() - tq}
    finally:
        if own:
            dev.close()
    for b in redo:
        solo = solve(plan, phases=np.atleast_2d(phases)[b:b + 1], result_cls=result_cls, quantize=quantize)[0]
        solo.meta.update({"batch": batch, "member": b, "solved_alone": True})
        results[b] = solo
    return results

"""Volumetric heating Q from recorded phasors, computed on the GPU.

Mirrors ``caustica.sensors.HeatingSource`` (sensors.py:99-353): the same
constructors, the same refusals (harmonics above the fundamental without an
absorption model, negative alpha, non-positive rho or c, non-finite
phasors), the same provenance ``meta`` and ``embed``. The voxel work,
Q = sum_n alpha_n |P_n|^2 / (rho c) in float64 rounded to float32
(sensors.py:259-273), runs in ``cg_heating_q`` / ``cg_solver_heating_q``
(``csrc/cg_post.cu``).

Media with at most 256 distinct (alpha_1..alpha_N, rho, c) tuples go to the
device as a uint8 label map and a float64 table per material; other media
as three float32 maps with alpha_n = alpha * n^y.

``HeatingSource.from_solver`` builds Q straight from a live solver handle's
phasors into a device buffer placed on the whole grid (zero outside the
record region), which the Pennes step takes as its heating term: the field
never goes to the host between the acoustic and the thermal solve.
"""

from __future__ import annotations

import ctypes as C
import warnings
from dataclasses import dataclass, field
from typing import Any

import numpy as np

from . import _lib

ALPHA_MODEL_F0 = "f0_only"
ALPHA_MODEL_POWER_LAW = "power_law"
ALPHA_MODEL_EXPLICIT = "explicit"
ALPHA_POWER_LAW_Y_RANGE = (0.0, 3.0)


def _as_float_map(value: Any, shape: tuple, what: str) -> np.ndarray:
    """Scalar or full map as float64 (sensors.py:87-96)."""
    arr = np.asarray(value, dtype=np.float64)
    if arr.shape not in ((), shape):
        raise ValueError(f"{what} has shape {arr.shape}, which is neither a scalar nor the field shape {shape}.")
    if not np.isfinite(arr).all():
        raise ValueError(f"{what} contains non-finite values.")
    return np.broadcast_to(arr, shape)


def _resolve_alpha(requested, alpha_f0, *, available, alpha_power_law_y, alpha_at_harmonics):
    """alpha map per requested harmonic (sensors.py:356-430)."""
    if alpha_power_law_y is not None and alpha_at_harmonics is not None:
        raise ValueError("pass EITHER alpha_power_law_y (alpha_n = alpha_f0 * n**y) OR alpha_at_harmonics "
                         "({n: alpha_np_m}), not both.")
    shape = alpha_f0.shape
    high = [n for n in requested if n >= 2]
    if high and alpha_power_law_y is None and alpha_at_harmonics is None:
        raise ValueError(
            f"this result carries harmonics {high} above the fundamental, but alpha is known only at f0; "
            f"heating them with the f0 value would under-report the heating. State the model: "
            f"alpha_power_law_y=y (alpha_n = alpha_f0 * n**y), alpha_at_harmonics={{n: alpha_np_m}}, "
            f"or harmonics=(1,) for the fundamental only.")
    if alpha_power_law_y is not None:
        y = float(alpha_power_law_y)
        lo, hi = ALPHA_POWER_LAW_Y_RANGE
        if not (np.isfinite(y) and lo <= y <= hi):
            raise ValueError(f"alpha_power_law_y={alpha_power_law_y} is outside the physical range [{lo}, {hi}].")
        return {n: alpha_f0 * float(n) ** y for n in requested}, {n: float(n) ** y for n in requested}
    if alpha_at_harmonics is not None:
        keys = {int(n): v for n, v in alpha_at_harmonics.items()}
        missing = [n for n in requested if n >= 2 and n not in keys]
        if missing:
            raise ValueError(f"alpha_at_harmonics is missing harmonic(s) {missing} (given: {sorted(keys)}; "
                             f"requested: {list(requested)}; recorded: {list(available)}).")
        out = {}
        heterogeneous = float(alpha_f0.min()) != float(alpha_f0.max())
        for n in requested:
            if n not in keys:
                out[n] = alpha_f0
                continue
            if heterogeneous and np.asarray(keys[n]).ndim == 0:
                warnings.warn(f"alpha_at_harmonics[{n}] is a single number but the medium's alpha at f0 is "
                              f"heterogeneous: the scalar is applied to every voxel.", stacklevel=4)
            arr = _as_float_map(keys[n], shape, f"alpha_at_harmonics[{n}]")
            if (arr < 0).any():
                raise ValueError(f"alpha_at_harmonics[{n}] must be >= 0 Np/m.")
            out[n] = arr
        return out, None
    return {n: alpha_f0 for n in requested}, {n: 1.0 for n in requested}


def _model_name(requested, alpha_power_law_y, alpha_at_harmonics) -> str:
    if alpha_at_harmonics is not None:
        return ALPHA_MODEL_EXPLICIT
    if alpha_power_law_y is not None and max(requested) > 1:
        return ALPHA_MODEL_POWER_LAW
    return ALPHA_MODEL_F0


def _requested(available, harmonics):
    if harmonics is None:
        req = tuple(available)
    else:
        req = tuple(dict.fromkeys(int(n) for n in harmonics))
        missing = [n for n in req if n not in available]
        if missing:
            raise ValueError(f"harmonics {missing} were asked for but are not in the result "
                             f"(available: {list(available)}).")
    if any(n < 1 for n in req):
        raise ValueError(f"harmonic numbers must be >= 1, got {req}")
    if len(req) > 8:
        raise ValueError("at most 8 harmonics can be summed")
    return req


def _labels_f64(vols, max_labels: int = 256):
    """Exact labels of equally shaped float64 volumes: (uint8 labels, (n, len(vols)) float64) or None."""
    flat = [np.ascontiguousarray(v, np.float64).reshape(-1) for v in vols]
    bits = [f.view(np.uint64) for f in flat]
    for bv in bits:  # cheap early refusal on a sample
        if len(np.unique(bv[:: max(1, bv.size // 4096)])) > max_labels:
            return None
    rows = np.ascontiguousarray(np.stack(bits, axis=1))
    keys = rows.view(np.dtype((np.void, rows.dtype.itemsize * rows.shape[1]))).reshape(-1)
    u, first, inv = np.unique(keys, return_index=True, return_inverse=True)
    if len(u) > max_labels:
        return None
    props = np.stack([f[first] for f in flat], axis=1)
    return inv.astype(np.uint8).reshape(np.shape(vols[0])), props


def _spec(requested, alpha_by_h, factors, alpha_f0, rho_map, c_map, shape3):
    """cg_heating_spec material part: label table (<= 256 distinct tuples) or dense float32 maps.

    Returns the spec and the objects that must outlive the call.
    """
    spec = _lib.HeatingSpec()
    spec.n_terms = len(requested)
    for t, n in enumerate(requested):
        spec.harmonics[t] = n
    for a in range(3):
        spec.map_shape[a] = shape3[a]
    lab = _labels_f64([alpha_by_h[n] for n in requested] + [rho_map, c_map])
    if lab is not None:
        labels, props = lab
        irc = 1.0 / (props[:, -2] * props[:, -1])
        coef = np.ascontiguousarray(np.concatenate([props[:, :len(requested)], irc[:, None]], axis=1))
        lab_dev = _lib.DeviceArray.from_host(np.ascontiguousarray(labels.reshape(shape3)))
        spec.n_labels = coef.shape[0]
        spec.coef = coef.ctypes.data_as(C.c_void_p)
        spec.labels = lab_dev.ptr
        return spec, [coef, lab_dev]
    if factors is None:
        raise ValueError("per-harmonic alpha maps (alpha_at_harmonics) are supported for media of at most 256 "
                         "distinct materials")
    maps = [_lib.DeviceArray.from_host(np.ascontiguousarray(np.reshape(m, shape3), np.float32))
            for m in (alpha_f0, rho_map, c_map)]
    spec.alpha, spec.rho, spec.c = maps[0].ptr, maps[1].ptr, maps[2].ptr
    for t, n in enumerate(requested):
        spec.alpha_factor[t] = factors[n]
    return spec, maps


def _close(objs) -> None:
    for o in objs:
        if isinstance(o, _lib.DeviceArray):
            o.close()


@dataclass(frozen=True, eq=False)
class HeatingSource:
    """Volumetric heat deposition Q [W/m^3] over a record region (sensors.py:99-131).

    ``q`` is the float32 map of the region (read from the device on first
    use); ``device`` holds Q on the device, placed on ``grid_shape`` (the
    region itself unless built with a grid), ready for the Pennes step.
    """

    region: tuple
    dx: float
    harmonics: tuple
    alpha_model: str
    meta: dict = field(default_factory=dict)
    device: Any = None
    grid_shape: tuple | None = None
    region_shape: tuple = ()
    _host: dict = field(default_factory=dict, repr=False)

    @property
    def q(self) -> np.ndarray:
        """float32 Q over the region (read from the device once)."""
        if "q" not in self._host:
            full = self.device.to_host()
            self._host["q"] = np.ascontiguousarray(full[self.region] if self.grid_shape is not None else full)
        return self._host["q"]

    @property
    def shape(self) -> tuple:
        return self.region_shape

    @property
    def q_max(self) -> float:
        return float(self.q.max())

    @property
    def total_power_w(self) -> float:
        """sum(Q) dx^ndim (sensors.py:314-321)."""
        return float(self.q.sum()) * self.dx ** self.q.ndim

    def embed(self, shape) -> np.ndarray:
        """Q on a full grid of ``shape``, zero outside the region (sensors.py:323-343)."""
        shape = tuple(int(s) for s in shape)
        if len(shape) != len(self.region):
            raise ValueError(f"shape {shape} has rank {len(shape)}, need {len(self.region)}")
        if self.grid_shape is not None and shape == tuple(self.grid_shape):
            return self.device.to_host()
        full = np.zeros(shape, dtype=np.float32)
        try:
            full[self.region] = self.q
        except ValueError as exc:
            raise ValueError(f"the region {self.region} does not fit a grid of shape {shape}: {exc}") from None
        return full

    def device_on(self, shape):
        """The device buffer of Q on a grid of ``shape``, or None when it lives on another grid."""
        if self.device is not None and self.grid_shape is not None and tuple(shape) == tuple(self.grid_shape):
            return self.device
        return None

    def close(self) -> None:
        if self.device is not None:
            self.device.close()

    # ---------- constructors ----------

    @classmethod
    def from_phasors(cls, phasors: dict, *, alpha: Any, rho: Any, c: Any, dx: float, region: tuple | None = None,
                     harmonics: tuple | None = None, alpha_power_law_y: float | None = None,
                     alpha_at_harmonics: dict | None = None, grid_shape: tuple | None = None,
                     scale: float = 1.0) -> "HeatingSource":
        """Q from bare phasor arrays (sensors.py:193-295), on the GPU.

        ``grid_shape`` places the device copy on a whole grid (zero outside
        ``region``); ``scale`` multiplies the float32 Q.
        """
        if not phasors:
            raise ValueError("phasors is empty: there is no field to turn into heat.")
        if not (np.isfinite(dx) and dx > 0):
            raise ValueError(f"dx must be a positive finite spacing in meters, got {dx}")
        available = tuple(sorted(int(n) for n in phasors))
        requested = _requested(available, harmonics)
        shape = tuple(np.shape(phasors[requested[0]]))
        for n in requested:
            if tuple(np.shape(phasors[n])) != shape:
                raise ValueError(f"harmonic {n} has shape {np.shape(phasors[n])} but harmonic {requested[0]} has "
                                 f"{shape}: the phasors are not on one grid.")
        alpha_f0, rho_map, c_map = _check_maps(alpha, rho, c, shape)
        alpha_by_h, factors = _resolve_alpha(requested, alpha_f0, available=available,
                                             alpha_power_law_y=alpha_power_law_y,
                                             alpha_at_harmonics=alpha_at_harmonics)
        ph = []
        for n in requested:
            p = np.ascontiguousarray(phasors[n], np.complex64)
            if not np.isfinite(p.view(np.float32)).all():
                raise ValueError(f"the phasor of harmonic {n} contains non-finite values; the run that produced "
                                 f"it did not converge on a physical field.")
            ph.append(p)
        if region is None:
            region = tuple(slice(0, n) for n in shape)
        if grid_shape is not None:
            region = tuple(slice(*sl.indices(g)[:2]) for sl, g in zip(region, grid_shape))
            if tuple(sl.stop - sl.start for sl in region) != shape:
                raise ValueError(f"the region {region} of a grid {tuple(grid_shape)} does not have the phasor "
                                 f"shape {shape}")
        shape3 = _embed3(shape)
        region3 = _embed3_region(region, shape)
        grid3 = _embed3(tuple(grid_shape)) if grid_shape is not None else shape3
        spec, keep = _spec(requested, alpha_by_h, factors, alpha_f0, rho_map, c_map, shape3)
        keep += [_lib.DeviceArray.from_host(p.reshape(shape3)) for p in ph]
        for t in range(len(requested)):
            spec.phasor[t] = keep[-len(requested) + t].ptr
        for a in range(3):
            spec.shape[a] = shape3[a]
            spec.q_shape[a] = grid3[a]
            spec.q_origin[a] = region3[a] if grid_shape is not None else 0
        spec.scale = float(np.float32(scale))
        out = _lib.DeviceArray(tuple(grid_shape) if grid_shape is not None else shape, np.float32)
        sums = np.zeros(8, np.float64)
        try:
            _lib.call("cg_heating_q", C.byref(spec), out.ptr, _lib.ptr(sums), None)
        except Exception:
            out.close()
            raise
        finally:
            _close(keep)
        nvox = int(np.prod(shape))
        meta = _meta(requested, alpha_by_h, alpha_power_law_y, alpha_at_harmonics, available, sums, nvox)
        return cls(region=tuple(region), dx=float(dx), harmonics=requested,
                   alpha_model=_model_name(requested, alpha_power_law_y, alpha_at_harmonics), meta=meta,
                   device=out, grid_shape=tuple(grid_shape) if grid_shape is not None else None,
                   region_shape=shape)

    @classmethod
    def from_result(cls, result, medium, dx: float, *, harmonics: tuple | None = None,
                    alpha_power_law_y: float | None = None, alpha_at_harmonics: dict | None = None,
                    grid_shape: tuple | None = None, scale: float = 1.0) -> "HeatingSource":
        """Q from a CW result and its medium (sensors.py:133-191)."""
        phasors = dict(result.phasors) if result.phasors else {1: result.phasor}
        region = tuple(result.region)
        a, r, cc = medium.alpha, medium.rho, medium.c
        if len(region) != np.ndim(a):
            raise ValueError(f"result.region has rank {len(region)} but the medium is {np.ndim(a)}-D — they are "
                             f"not the same grid.")
        maps = {"alpha": a[region], "rho": r[region], "c": cc[region]}
        shape = tuple(np.shape(phasors[next(iter(phasors))]))
        for name, vol in maps.items():
            if vol.shape != shape:
                raise ValueError(f"medium.{name} sliced by result.region has shape {vol.shape} but the recorded "
                                 f"phasor has shape {shape}.")
        return cls.from_phasors(phasors, alpha=maps["alpha"], rho=maps["rho"], c=maps["c"], dx=dx, region=region,
                                harmonics=harmonics, alpha_power_law_y=alpha_power_law_y,
                                alpha_at_harmonics=alpha_at_harmonics, grid_shape=grid_shape, scale=scale)

    @classmethod
    def from_solver(cls, dev, member: int, result, medium, dx: float, *, harmonics: tuple | None = None,
                    alpha_power_law_y: float | None = None, alpha_at_harmonics: dict | None = None,
                    scale: float = 1.0) -> "HeatingSource":
        """Q from member ``member`` of a live ``DeviceSolver`` after its finalize, on the whole grid.

        The phasors stay on the device. When the solve ran on a label medium
        (and no per-harmonic maps are given) the solver's own label map and
        its per-material alpha, rho, c serve, and the checks of the
        reference run on the materials present in the record region;
        otherwise ``medium``'s alpha, rho and c maps are checked and uploaded.
        """
        plan = dev.plan
        available = tuple(sorted(int(n) for n in plan.harmonics))
        requested = _requested(available, harmonics)
        grid = tuple(plan.shape)
        grid3 = _embed3(grid)
        region = tuple(slice(*sl.indices(g)[:2]) for sl, g in zip(result.region, grid))
        region3 = _embed3_region(region, grid)
        props = plan.label_props
        labelled = plan.labels is not None or plan.labels_dev is not None
        if labelled and props is not None and alpha_at_harmonics is None:
            if plan.labels is not None:
                sub = (slice(None),) * (3 - len(grid)) + region
                present = np.flatnonzero(np.bincount(plan.labels[sub].reshape(-1), minlength=256))
            else:  # a device label map: the labels counted over the whole grid (a superset of the region's)
                present = np.asarray(plan.meta["present_labels"])
            pr = np.asarray(props, np.float64)
            alpha_l, rho_l, c_l = _check_maps(pr[present, 0], pr[present, 1], pr[present, 2], (len(present),))
            alpha_by_h, factors = _resolve_alpha(requested, np.asarray(pr[:, 0]), available=available,
                                                 alpha_power_law_y=alpha_power_law_y, alpha_at_harmonics=None)
            irc = 1.0 / (pr[:, 1] * pr[:, 2])
            coef = np.ascontiguousarray(np.stack([alpha_by_h[n] for n in requested] + [irc], axis=1))
            keep = [coef]
            spec = _lib.HeatingSpec()
            spec.n_terms = len(requested)
            for t, n in enumerate(requested):
                spec.harmonics[t] = n
            spec.n_labels = coef.shape[0]
            spec.coef = coef.ctypes.data_as(C.c_void_p)
            ranges = {n: np.asarray(alpha_by_h[n])[present] for n in requested}
        else:
            alpha_f0, rho_map, c_map = _check_maps(medium.alpha, medium.rho, medium.c, grid)
            alpha_by_h, factors = _resolve_alpha(requested, alpha_f0, available=available,
                                                 alpha_power_law_y=alpha_power_law_y,
                                                 alpha_at_harmonics=alpha_at_harmonics)
            spec, keep = _spec(requested, alpha_by_h, factors, alpha_f0, rho_map, c_map, grid3)
            for a in range(3):
                spec.map_origin[a] = region3[a]
            ranges = {n: np.asarray(alpha_by_h[n])[region] for n in requested}
        for a in range(3):
            spec.q_shape[a] = grid3[a]
            spec.q_origin[a] = region3[a]
        spec.scale = float(np.float32(scale))
        out = _lib.DeviceArray(grid, np.float32)
        sums = np.zeros(8, np.float64)
        try:
            _lib.call("cg_solver_heating_q", dev.h, int(member), C.byref(spec), out.ptr, _lib.ptr(sums))
        except Exception:
            out.close()
            raise
        finally:
            _close(keep)
        rshape = tuple(sl.stop - sl.start for sl in region)
        meta = _meta(requested, ranges, alpha_power_law_y, alpha_at_harmonics, available, sums,
                     int(np.prod(rshape)))
        return cls(region=region, dx=float(dx), harmonics=requested,
                   alpha_model=_model_name(requested, alpha_power_law_y, alpha_at_harmonics), meta=meta,
                   device=out, grid_shape=grid, region_shape=rshape)


def _check_maps(alpha, rho, c, shape):
    alpha_f0 = _as_float_map(alpha, shape, "alpha")
    rho_map = _as_float_map(rho, shape, "rho")
    c_map = _as_float_map(c, shape, "c")
    if (alpha_f0 < 0).any():
        raise ValueError("alpha must be >= 0 Np/m (absorption cannot be negative).")
    if (rho_map <= 0).any() or (c_map <= 0).any():
        raise ValueError("rho and c must be > 0 everywhere to convert |P|^2 into intensity.")
    return alpha_f0, rho_map, c_map


def _embed3(shape):
    return (1,) * (3 - len(shape)) + tuple(int(n) for n in shape)


def _embed3_region(region, shape):
    return (0,) * (3 - len(shape)) + tuple(int(s.start or 0) for s in region)


def _meta(requested, alpha_by_h, y, explicit, available, sums, nvox):
    return {
        "alpha_model": _model_name(requested, y, explicit),
        "alpha_power_law_y": y,
        "alpha_np_m_range": {n: (float(np.min(alpha_by_h[n])), float(np.max(alpha_by_h[n]))) for n in requested},
        "mean_q_by_harmonic_w_m3": {n: float(sums[t] / nvox) for t, n in enumerate(requested)},
        "harmonics_available": list(available),
        "intensity_model": "local plane wave: I = |P|^2 / (2 rho c)",
        "alpha_meaning": "absorption (not total attenuation)",
        "device": "cg_heating_q",
    }

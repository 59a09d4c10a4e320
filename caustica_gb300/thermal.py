"""Pennes bioheat + CEM43 on GB300, with the reference's ``PennesSolver`` interface.

``PennesSolverGB300(...).solve(temperature0, q, medium, dt, n_steps, *,
record_every=None, dose=False, dose0=None)`` follows thermal/pennes.py:
289-689: the same constructor options (blood constants, boundary,
reference temperature, ``on_unstable``, ``finite_check_every``), the same
stability bound and refusals, state carried as the rise above the reference
temperature, CEM43 accumulated in the loop by the trapezoid rule, float32
outputs. Each sub-step is one launch of the fused stencil + dose kernel in
``libcaustica_gb300.so``; the dose sum is Kahan-compensated.
"""

from __future__ import annotations

import ctypes as C
import logging
from collections.abc import Sequence
from dataclasses import dataclass, field
from math import ceil
from typing import Any

import numpy as np

from . import _lib
from .device import as_device, is_device_array


def _qptr(q):
    """Host or device pointer of a field (the library copies either); None -> NULL."""
    if q is None:
        return None
    return q.ptr if isinstance(q, _lib.DeviceArray) else _lib.ptr(q)


log = logging.getLogger("caustica")

BLOOD_DENSITY = 1050.0  # pennes.py:118
BLOOD_SPECIFIC_HEAT = 3617.0  # pennes.py:120
ARTERIAL_TEMPERATURE_C = 37.0  # pennes.py:122
SCHEME = "pennes-fd-explicit-gb300/1"


class ThermalDivergedError(RuntimeError):
    """pennes.py:132-133."""


class ThermalStabilityError(ValueError):
    """pennes.py:136-137."""


class ThermalMedium:
    """Per-voxel k / rho / C / w_b plus dx (thermal/properties.py:83-253)."""

    def __init__(self, k, rho, specific_heat, perfusion, dx: float, id_map=None):
        vols = {"k": k, "rho": rho, "specific_heat": specific_heat, "perfusion": perfusion}
        shapes = {n: np.shape(v) for n, v in vols.items()}
        if len(set(shapes.values())) != 1:
            raise ValueError(f"thermal property volumes disagree in shape: {shapes}")
        for n, v in vols.items():
            arr = np.ascontiguousarray(v, dtype=np.float32)
            if not np.isfinite(arr).all():
                raise ValueError(f"thermal volume '{n}' contains non-finite values")
            setattr(self, n, arr)
        for n in ("k", "rho", "specific_heat"):
            if (getattr(self, n) <= 0).any():
                raise ValueError(f"thermal volume '{n}' must be > 0 everywhere")
        if (self.perfusion < 0).any():
            raise ValueError("perfusion must be >= 0")
        if not (np.isfinite(dx) and dx > 0):
            raise ValueError(f"dx must be a positive finite spacing in meters, got {dx}")
        self.dx = float(dx)
        self.id_map = id_map

    @classmethod
    def homogeneous(cls, shape, *, k: float, rho: float, specific_heat: float, perfusion: float, dx: float):
        full = np.ones(shape, dtype=np.float32)
        return cls(full * k, full * rho, full * specific_heat, full * perfusion, dx)

    @property
    def shape(self):
        return self.k.shape

    @property
    def ndim(self):
        return self.k.ndim

    @property
    def volumetric_heat_capacity(self) -> np.ndarray:
        return (self.rho.astype(np.float64) * self.specific_heat).astype(np.float32)

    @property
    def diffusivity(self) -> np.ndarray:
        return (self.k.astype(np.float64) / self.volumetric_heat_capacity).astype(np.float32)

    @property
    def is_perfused(self) -> bool:
        return bool((self.perfusion > 0).any())


@dataclass
class ThermalResult:
    """What a Pennes solve returns (pennes.py:147-201)."""

    temperature: np.ndarray
    temperature_max: np.ndarray
    dose_cem43: np.ndarray | None
    samples: list
    times: list
    dt: float
    n_steps: int
    t_end_s: float
    substeps: int
    meta: dict[str, Any] = field(default_factory=dict)

    @property
    def peak_temperature_c(self) -> float:
        return float(self.temperature_max.max())

    @property
    def peak_dose_cem43(self) -> float | None:
        return None if self.dose_cem43 is None else float(self.dose_cem43.max())

    @staticmethod
    def chain(results: Sequence[ThermalResult]) -> ThermalResult:
        """One result for a multi-phase exposure (pennes.py:203-286)."""
        results = list(results)
        if not results:
            raise ValueError("ThermalResult.chain() needs at least one result")
        if len({r.temperature.shape for r in results}) != 1:
            raise ValueError("the phases are not on one grid")
        dosed = [r.dose_cem43 is not None for r in results]
        if any(dosed) and not all(dosed):
            raise ValueError("some phases accumulated no CEM43 while others did; solve every phase with "
                             "dose=True, passing the previous phase's dose_cem43 as dose0.")
        for i, (prev, nxt) in enumerate(zip(results, results[1:], strict=False)):
            if prev.dose_cem43 is None:
                continue
            slack = 1e-6 * np.maximum(1.0, prev.dose_cem43)
            if not bool((nxt.dose_cem43 >= prev.dose_cem43 - slack).all()):
                raise ValueError(f"phase {i + 1}'s CEM43 map is BELOW phase {i}'s somewhere, so the phases were "
                                 f"not chained. Pass dose0=<previous>.dose_cem43.")
        tmax = results[0].temperature_max.copy()
        for r in results[1:]:
            np.maximum(tmax, r.temperature_max, out=tmax)
        samples, times, offset = [], [], 0.0
        for i, r in enumerate(results):
            for t, s in zip(r.times, r.samples, strict=True):
                if i > 0 and t == 0.0:
                    continue
                times.append(offset + t)
                samples.append(s)
            offset += r.t_end_s
        last = results[-1]
        meta = dict(last.meta)
        meta["q"] = " -> ".join(str(r.meta.get("q")) for r in results)
        meta["chained_phases"] = [{"t_end_s": r.t_end_s, "n_steps": r.n_steps, "dt_s": r.dt} for r in results]
        return ThermalResult(temperature=last.temperature, temperature_max=tmax, dose_cem43=last.dose_cem43,
                             samples=samples, times=times, dt=last.dt, n_steps=sum(r.n_steps for r in results),
                             t_end_s=float(sum(r.t_end_s for r in results)),
                             substeps=max(r.substeps for r in results), meta=meta)


def _ax(a, axis, sl):
    idx = [slice(None)] * a.ndim
    idx[axis] = sl
    return a[tuple(idx)]


def _representative(medium):
    """For a single-material medium, a grid of min(n, 3) cells per axis has
    every distinct Gershgorin row of the full grid (corners, edges, faces,
    interior), so the stable step computed on it is the full grid's, exactly."""
    vols = [np.asarray(getattr(medium, a)) for a in ("k", "rho", "specific_heat", "perfusion")]
    flat = [v.reshape(-1) for v in vols]
    if not all(np.all(f == f[0]) for f in flat):
        return None
    shape = tuple(min(n, 3) for n in vols[0].shape)
    return ThermalMedium(*(np.full(shape, f[0], np.float32) for f in flat), dx=medium.dx)


def thermal_labels(medium, max_labels: int = 256):
    """Exact label decomposition of (k, rho, C, w_b) or None (> max_labels materials)."""
    from .engine import label_volumes

    vols = [np.ascontiguousarray(getattr(medium, a), np.float32) for a in ("k", "rho", "specific_heat", "perfusion")]
    return label_volumes(vols, getattr(medium, "id_map", None), max_labels)


def _embed3(a: np.ndarray) -> np.ndarray:
    return a.reshape((1,) * (3 - a.ndim) + a.shape)


class PennesSolverGB300:
    """Explicit conservative-FD Pennes solver on GB300 (pennes.py:289-372)."""

    name = "pennes_gb300"
    scheme = SCHEME

    def __init__(self, backend: str = "auto", *, blood_density: float = BLOOD_DENSITY,
                 blood_specific_heat: float = BLOOD_SPECIFIC_HEAT,
                 arterial_temperature_c: float = ARTERIAL_TEMPERATURE_C, boundary: str = "insulated",
                 boundary_temperature_c: float | None = None, reference_temperature_c: float | None = None,
                 on_unstable: str = "refuse", finite_check_every: int = 25):
        if boundary not in ("insulated", "dirichlet"):
            raise ValueError(f"boundary must be 'insulated' (zero flux) or 'dirichlet' (walls held at "
                             f"boundary_temperature_c), got {boundary!r}")
        if on_unstable not in ("refuse", "substep"):
            raise ValueError(f"on_unstable must be 'refuse' or 'substep', got {on_unstable!r}. There is "
                             f"deliberately no option that integrates an unstable step.")
        if blood_density <= 0 or blood_specific_heat <= 0:
            raise ValueError("blood_density and blood_specific_heat must be > 0")
        if finite_check_every < 1:
            raise ValueError(f"finite_check_every must be >= 1, got {finite_check_every}")
        self.backend = backend
        self.blood_density = float(blood_density)
        self.blood_specific_heat = float(blood_specific_heat)
        self.arterial_temperature_c = float(arterial_temperature_c)
        self.boundary = boundary
        self.boundary_temperature_c = (float(arterial_temperature_c) if boundary_temperature_c is None
                                       else float(boundary_temperature_c))
        self.reference_temperature_c = (float(arterial_temperature_c) if reference_temperature_c is None
                                        else float(reference_temperature_c))
        if not np.isfinite(self.reference_temperature_c):
            raise ValueError("reference_temperature_c must be finite")
        self.on_unstable = on_unstable
        self.finite_check_every = int(finite_check_every)

    # ---- coefficients, float32 host arithmetic as in pennes.py:404-447 ----
    def _faces(self, k, dx):
        inv_dx2 = 1.0 / (dx * dx)
        return [((2.0 * _ax(k, ax, slice(None, -1)) * _ax(k, ax, slice(1, None))
                  / (_ax(k, ax, slice(None, -1)) + _ax(k, ax, slice(1, None)))) * inv_dx2).astype(np.float32)
                for ax in range(k.ndim)]

    def _walls(self, k, dx):
        inv_dx2 = 1.0 / (dx * dx)
        return [((2.0 * _ax(k, ax, slice(0, 1)) * inv_dx2).astype(np.float32),
                 (2.0 * _ax(k, ax, slice(-1, None)) * inv_dx2).astype(np.float32)) for ax in range(k.ndim)]

    def _perf(self, medium):
        return (medium.perfusion * np.float32(self.blood_density * self.blood_specific_heat)).astype(np.float32)

    def _inv_rho_c(self, medium):
        vhc = (np.asarray(medium.rho, np.float32).astype(np.float64) * medium.specific_heat).astype(np.float32)
        return np.asarray(1.0 / vhc.astype(np.float64), np.float32)

    def _stable(self, medium, faces, walls, perf, inv_rho_c):
        diag = np.zeros(medium.shape, np.float32)
        for ax, kf in enumerate(faces):
            _ax(diag, ax, slice(None, -1))[...] += kf
            _ax(diag, ax, slice(1, None))[...] += kf
        if walls is not None:
            for ax, (lo, hi) in enumerate(walls):
                _ax(diag, ax, slice(0, 1))[...] += lo
                _ax(diag, ax, slice(-1, None))[...] += hi
        diag += perf
        diag *= inv_rho_c
        peak = float(diag.max())
        return float("inf") if peak <= 0.0 else 1.0 / peak

    def stable_dt(self, medium) -> float:
        """Gershgorin positivity bound (pennes.py:376-402)."""
        small = _representative(medium)
        if small is not None:
            medium = small
        k = np.asarray(medium.k, np.float32)
        walls = self._walls(k, medium.dx) if self.boundary == "dirichlet" else None
        return self._stable(medium, self._faces(k, medium.dx), walls, self._perf(medium), self._inv_rho_c(medium))

    def _resolve_substeps(self, dt, dt_stable, medium) -> int:
        """pennes.py:723-754."""
        if dt <= dt_stable:
            return 1
        if self.on_unstable == "substep":
            return int(ceil(dt / dt_stable))
        raise ThermalStabilityError(
            f"dt = {dt:.6g} s is above the stability bound {dt_stable:.6g} s of the explicit scheme for this medium "
            f"(dx = {medium.dx * 1e3:.6g} mm). Pass dt <= {dt_stable:.6g} s, construct the solver with "
            f"on_unstable='substep', or coarsen dx.")

    def _prepare_q(self, q, medium):
        """pennes.py:693-721."""
        if q is None:
            return None, "none"
        shape = medium.shape
        if is_device_array(q):
            # Q already on the device (cg_solver_heating_q / cg_heating_q, or a
            # framework tensor by DLPack / __cuda_array_interface__)
            q = as_device(q, what="Q")
            if q.shape != tuple(shape) or q.dtype != np.float32:
                raise ValueError(f"device Q is {q.dtype}{q.shape} but the thermal medium is float32{shape}.")
            return q, "device"
        dev = q.device_on(shape) if hasattr(q, "device_on") else None
        if dev is not None:
            if abs(q.dx - medium.dx) > 1e-12 * max(q.dx, medium.dx):
                raise ValueError(f"the HeatingSource was built on a grid with dx = {q.dx * 1e3:.6g} mm but this "
                                 f"thermal medium has dx = {medium.dx * 1e3:.6g} mm.")
            return dev, f"HeatingSource({q.alpha_model}, device)"
        if hasattr(q, "q") and hasattr(q, "dx") and hasattr(q, "region"):
            if abs(q.dx - medium.dx) > 1e-12 * max(q.dx, medium.dx):
                raise ValueError(f"the HeatingSource was built on a grid with dx = {q.dx * 1e3:.6g} mm but this "
                                 f"thermal medium has dx = {medium.dx * 1e3:.6g} mm.")
            if q.q.shape != shape:
                raise ValueError(f"the HeatingSource covers the record region {q.region} (shape {q.q.shape}) but "
                                 f"the thermal medium is {shape}; place it with heating_source.embed({shape}).")
            return np.ascontiguousarray(q.q, np.float32), f"HeatingSource({getattr(q, 'alpha_model', '?')})"
        arr = np.asarray(q, dtype=np.float32)
        if arr.ndim == 0:
            arr = np.full(shape, float(arr), dtype=np.float32)
        if arr.shape != shape:
            raise ValueError(f"Q has shape {arr.shape} but the thermal medium is {shape}.")
        if not np.isfinite(arr).all():
            raise ValueError("Q contains non-finite values.")
        return np.ascontiguousarray(arr), "array"

    def solve(self, temperature0, q, medium, dt: float, n_steps: int, *, record_every: int | None = None,
              dose: bool = False, dose0=None, timing: dict | None = None) -> ThermalResult:
        """Integrate ``n_steps`` outer steps of ``dt`` (pennes.py:451-689).

        ``timing``: a dict that receives ``device_ms``, the CUDA-event time of
        all sub-steps on the handle's stream (each run between guards is timed
        and synchronised), and ``substeps``, their count.
        """
        if not all(hasattr(medium, a) for a in ("k", "rho", "specific_heat", "perfusion", "dx")):
            raise TypeError(f"medium must be a ThermalMedium, got {type(medium).__name__}.")
        if not (np.isfinite(dt) and dt > 0):
            raise ValueError(f"dt must be a positive finite number of seconds, got {dt}")
        n_steps = int(n_steps)
        if n_steps < 1:
            raise ValueError(f"n_steps must be >= 1, got {n_steps}")
        if record_every is not None:
            if int(record_every) < 1:
                raise ValueError(f"record_every must be >= 1 or None, got {record_every}")
            record_every = int(record_every)
        if dose0 is not None and not dose:
            raise ValueError("dose0 was given but dose=False, so the dose already accumulated would be dropped. "
                             "Pass dose=True to continue accumulating, or drop dose0 to start fresh.")
        shape = tuple(medium.shape)
        if tuple(np.shape(temperature0)) != shape:
            raise ValueError(f"temperature0 has shape {tuple(np.shape(temperature0))} but the thermal medium is "
                             f"{shape}.")
        t_ref = np.float32(self.reference_temperature_c)
        # theta = T0 - t_ref, its finiteness check (pennes.py:531-536) and
        # T = theta + t_ref on the way out run on the device
        # a device T0 / dose0 (either exchange protocol) goes to the device calls as it is
        temp0 = (as_device(temperature0, dtype=np.float32, shape=shape, what="temperature0")
                 if is_device_array(temperature0) else np.ascontiguousarray(temperature0, dtype=np.float32))
        q_arr, q_kind = self._prepare_q(q, medium)
        ref_minus_ta = np.float32(self.reference_temperature_c - self.arterial_temperature_c)
        theta_wall = np.float32(self.boundary_temperature_c) - t_ref
        lab = thermal_labels(medium)
        if lab is not None:
            # per-material coefficients with the reference's float32 arithmetic
            lab_vol, props = lab
            perfused = bool((props[:, 3] > 0).any())
            pm = ThermalMedium(props[:, 0], props[:, 1], props[:, 2], props[:, 3], dx=medium.dx)
            if len(props) == 1:
                # one material: the bound of its min(n, 3)-cell representative is the grid's
                rep = tuple(min(n, 3) for n in shape)
                dt_stable = self.stable_dt(ThermalMedium(*(np.full(rep, props[0, j], np.float32) for j in range(4)),
                                                         dx=medium.dx))
            else:
                dt_stable = self.stable_dt(medium)
            n_sub = self._resolve_substeps(dt, dt_stable, medium)
            dt_sub = dt / n_sub
            perf_l = self._perf(pm)
            coeff_l = (self._inv_rho_c(pm) * np.float32(dt_sub)).astype(np.float32)
            poff_l = ((perf_l * ref_minus_ta).astype(np.float32) if perfused and float(ref_minus_ta) != 0.0
                      else np.zeros_like(perf_l))
            table = np.ascontiguousarray(np.stack([props[:, 0], coeff_l, perf_l if perfused else 0 * perf_l,
                                                   poff_l], axis=1).astype(np.float32))
            faces = walls = perf = coeff = perf_offset = None
        else:
            perfused = bool(medium.is_perfused)
            k = np.asarray(medium.k, np.float32)
            faces = self._faces(k, medium.dx)
            walls = self._walls(k, medium.dx) if self.boundary == "dirichlet" else None
            perf = self._perf(medium)
            inv_rho_c = self._inv_rho_c(medium)
            dt_stable = self._stable(medium, faces, walls, perf, inv_rho_c)
            n_sub = self._resolve_substeps(dt, dt_stable, medium)
            dt_sub = dt / n_sub
            coeff = (inv_rho_c * np.float32(dt_sub)).astype(np.float32)
            perf_offset = ((perf * ref_minus_ta).astype(np.float32)
                           if perfused and float(ref_minus_ta) != 0.0 else None)
        dose_arr = None
        if dose:
            if dose0 is not None and is_device_array(dose0):
                dose_arr = as_device(dose0, dtype=np.float32, shape=shape, what="dose0")
            else:
                dose_arr = (np.zeros(shape, np.float32) if dose0 is None
                            else np.ascontiguousarray(np.asarray(dose0, np.float32)))
            if dose_arr.shape != shape:
                raise ValueError(f"dose0 has shape {dose_arr.shape} but the medium is {shape}.")

        # 3-D frame (a 2-D grid a x b is 1 x a x b; axes keep their order)
        nd = len(shape)
        s3 = (1,) * (3 - nd) + shape
        kf3 = [None, None, None]
        for ax, kf in enumerate(faces or []):
            kf3[3 - nd + ax] = np.ascontiguousarray(_embed3(kf))
        wall_buf = None
        if walls is not None:
            nx, ny, nz = s3
            planes = {0: (ny * nz,), 1: (nx * nz,), 2: (nx * ny,)}
            parts = []
            for ax3 in range(3):
                ax = ax3 - (3 - nd)
                if ax < 0:
                    parts += [np.zeros(planes[ax3], np.float32)] * 2
                else:
                    lo, hi = walls[ax]
                    parts += [np.ascontiguousarray(_embed3(lo)).reshape(-1).astype(np.float32),
                              np.ascontiguousarray(_embed3(hi)).reshape(-1).astype(np.float32)]
            wall_buf = np.ascontiguousarray(np.concatenate(parts))
        cfg = _lib.PennesConfig()
        cfg.nx, cfg.ny, cfg.nz = s3
        cfg.dirichlet = int(self.boundary == "dirichlet")
        cfg.dose = int(dose)
        cfg.theta_wall = float(theta_wall)
        cfg.t_ref = float(t_ref)
        cfg.half_dt_min = float(np.float32(0.5 * dt_sub / 60.0))
        lib = _lib.load()
        h = C.c_void_p()
        _lib.check(lib.cg_pennes_create(C.byref(cfg), C.byref(h)), "cg_pennes_create")
        try:
            if lab is not None:
                wall_axes = sum(1 << a for a in range(3 - nd, 3))
                _lib.call("cg_pennes_set_labels", h, _lib.ptr(np.ascontiguousarray(lab_vol.reshape(s3))),
                          len(table), _lib.ptr(table), float(np.float32(1.0 / (medium.dx * medium.dx))),
                          int(perfused and float(ref_minus_ta) != 0.0), wall_axes, _qptr(q_arr))
            else:
                _lib.call("cg_pennes_set_coefficients", h, _lib.ptr(kf3[0]), _lib.ptr(kf3[1]), _lib.ptr(kf3[2]),
                          _lib.ptr(wall_buf), _lib.ptr(np.ascontiguousarray(perf)) if perfused else None,
                          _lib.ptr(np.ascontiguousarray(coeff)), _qptr(q_arr),
                          _lib.ptr(np.ascontiguousarray(perf_offset)) if perf_offset is not None else None)
            fin = C.c_int(0)
            _lib.call("cg_pennes_set_temperature", h, _qptr(temp0), _qptr(dose_arr), C.byref(fin))
            if not fin.value:
                raise ValueError("temperature0 contains non-finite values; a solve cannot start from a field that "
                                 "is not a temperature.")
            samples, times = [], []
            buf = np.empty(shape, np.float32)

            def record(step_idx):
                _lib.call("cg_pennes_get_temperature", h, _lib.ptr(buf), None, None)
                samples.append(buf.copy())
                times.append(step_idx * dt)

            def guard(step):
                """pennes.py:756-781: temperature first, then the dose."""
                fin = C.c_int(3)
                _lib.call("cg_pennes_check_finite", h, C.byref(fin))
                for bit, what in ((1, "temperature"), (2, "CEM43 dose")):
                    if not fin.value & bit:
                        raise ThermalDivergedError(
                            f"the {what} field stopped being finite at outer step {step} (t = {step * dt:.6g} s, "
                            f"{n_sub} sub-step(s) per step). Nothing downstream of this point is a physical "
                            f"result. Usual causes, most common first: a heat source far outside the range "
                            f"float32 can carry, a temperature driven above ~170 C where the CEM43 rate "
                            f"R^(43-T) itself overflows float32, or a medium whose k / rho / C make the "
                            f"assembled step unstable in a way the bound could not see (check "
                            f"PennesSolverGB300.stable_dt(medium) against your dt).")

            if record_every is not None:
                record(0)
            step = 0
            while step < n_steps:
                # run up to the next record / guard boundary in one go
                nxt = n_steps
                if record_every is not None:
                    nxt = min(nxt, (step // record_every + 1) * record_every)
                nxt = min(nxt, (step // self.finite_check_every + 1) * self.finite_check_every)
                if timing is None:
                    _lib.call("cg_pennes_run", h, (nxt - step) * n_sub)
                else:
                    ms = C.c_float(0.0)
                    _lib.call("cg_pennes_timed_run", h, (nxt - step) * n_sub, C.byref(ms))
                    timing["device_ms"] = timing.get("device_ms", 0.0) + float(ms.value)
                    timing["substeps"] = timing.get("substeps", 0) + (nxt - step) * n_sub
                step = nxt
                if record_every is not None and step % record_every == 0:
                    record(step)
                if step % self.finite_check_every == 0 and step != n_steps:
                    guard(step)
            guard(n_steps)
            if record_every is not None and (not times or times[-1] != n_steps * dt):
                record(n_steps)
            T = np.empty(shape, np.float32)
            Tm = np.empty(shape, np.float32)
            D = np.empty(shape, np.float32) if dose else None
            _lib.call("cg_pennes_get_temperature", h, _lib.ptr(T), _lib.ptr(Tm), _lib.ptr(D))
        finally:
            lib.cg_pennes_destroy(h)
        return ThermalResult(
            temperature=T, temperature_max=Tm, dose_cem43=D, samples=samples, times=times,
            dt=float(dt), n_steps=n_steps, t_end_s=float(dt * n_steps), substeps=n_sub,
            meta={"scheme": SCHEME, "backend": "gb300", "boundary": self.boundary,
                  "boundary_temperature_c": self.boundary_temperature_c, "dt_stable_s": dt_stable,
                  "dt_sub_s": dt_sub, "q": q_kind, "perfusion_active": perfused,
                  "blood_density": self.blood_density, "blood_specific_heat": self.blood_specific_heat,
                  "arterial_temperature_c": self.arterial_temperature_c,
                  "reference_temperature_c": self.reference_temperature_c, "dose_accumulated": dose,
                  "dose_summation": "kahan", "coefficients": "labels" if lab is not None else "dense"})

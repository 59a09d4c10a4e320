"""Oracle: explicit Pennes bioheat step with in-loop CEM43 dose (NumPy).

TEST INFRASTRUCTURE ONLY (see :mod:`oracle`). Restates
``PennesSolver`` (thermal/pennes.py:289-689) and ``cem43_rate``
(thermal/dose.py:74-89). ``dtype=np.float64`` reproduces the reference run
through an FP64 backend, including the places where the reference forms a
``np.float32`` scalar on the host (pennes.py:524, 565, 571, 596), which keep
their float32 rounding in that run; results are cast to float32 on return
as the reference does (pennes.py:660-667).
"""

from __future__ import annotations

from math import ceil

import numpy as np

BLOOD_DENSITY = 1050.0  # pennes.py:118
BLOOD_SPECIFIC_HEAT = 3617.0  # pennes.py:120
ARTERIAL_TEMPERATURE_C = 37.0  # pennes.py:122


class OracleThermalDiverged(RuntimeError):
    """Mirror of ``ThermalDivergedError`` (pennes.py:132-133)."""


class OracleThermalStability(ValueError):
    """Mirror of ``ThermalStabilityError`` (pennes.py:136-137)."""


def _ax(arr, axis, sl):
    """pennes.py:140-144."""
    idx = [slice(None)] * arr.ndim
    idx[axis] = sl
    return arr[tuple(idx)]


def cem43_rate(t):
    """R^(43 - T), R = 0.5 above 43 C else 0.25 (dose.py:74-89)."""
    t = np.asarray(t)
    scalar = t.dtype.type
    r = np.where(t > 43.0, scalar(0.5), scalar(0.25))
    return r ** (scalar(43.0) - t)


def face_conductances(k, dx, dtype):
    """Harmonic-mean face k over dx^2 per axis (pennes.py:404-412)."""
    inv_dx2 = 1.0 / (dx * dx)
    faces = []
    for ax in range(k.ndim):
        lo = _ax(k, ax, slice(None, -1))
        hi = _ax(k, ax, slice(1, None))
        faces.append(((2.0 * lo * hi / (lo + hi)) * inv_dx2).astype(dtype))
    return faces


def wall_conductances(k, dx, dtype):
    """Dirichlet wall coefficients 2 k_edge / dx^2 (pennes.py:414-426)."""
    inv_dx2 = 1.0 / (dx * dx)
    out = []
    for ax in range(k.ndim):
        lo = (2.0 * _ax(k, ax, slice(0, 1)) * inv_dx2).astype(dtype)
        hi = (2.0 * _ax(k, ax, slice(-1, None)) * inv_dx2).astype(dtype)
        out.append((lo, hi))
    return out


def diagonal(k, faces, walls, dtype):
    """Sum of face coefficients per cell (pennes.py:428-438)."""
    diag = np.zeros(k.shape, dtype=dtype)
    for ax, kf in enumerate(faces):
        _ax(diag, ax, slice(None, -1))[...] += kf
        _ax(diag, ax, slice(1, None))[...] += kf
    if walls is not None:
        for ax, (lo, hi) in enumerate(walls):
            _ax(diag, ax, slice(0, 1))[...] += lo
            _ax(diag, ax, slice(-1, None))[...] += hi
    return diag


def coefficients(k, rho, specific_heat, perfusion, dx, dtype, *, boundary="insulated",
                 blood_density=BLOOD_DENSITY, blood_specific_heat=BLOOD_SPECIFIC_HEAT):
    """Faces, walls, perfusion sink, 1/(rho C) and the stable step (pennes.py:540-555)."""
    k_dev = np.asarray(np.asarray(k, np.float32), dtype=dtype)
    faces = face_conductances(k_dev, dx, dtype)
    walls = wall_conductances(k_dev, dx, dtype) if boundary == "dirichlet" else None
    w = np.asarray(np.asarray(perfusion, np.float32), dtype=dtype)
    perf = (w * np.float32(blood_density * blood_specific_heat)).astype(dtype)
    vhc = (np.asarray(rho, np.float32).astype(np.float64) * np.asarray(specific_heat, np.float32)).astype(
        np.float32
    )
    inv_rho_c = np.asarray(1.0 / vhc.astype(np.float64), dtype=dtype)
    diag = diagonal(k_dev, faces, walls, dtype)
    diag += perf
    diag *= inv_rho_c
    peak = float(diag.max())
    dt_stable = float("inf") if peak <= 0.0 else 1.0 / peak
    return faces, walls, perf, inv_rho_c, dt_stable


def solve(
    temperature0,
    q,
    *,
    k,
    rho,
    specific_heat,
    perfusion,
    dx,
    dt,
    n_steps,
    dose=False,
    dose0=None,
    boundary="insulated",
    boundary_temperature_c=None,
    reference_temperature_c=None,
    on_unstable="refuse",
    blood_density=BLOOD_DENSITY,
    blood_specific_heat=BLOOD_SPECIFIC_HEAT,
    arterial_temperature_c=ARTERIAL_TEMPERATURE_C,
    record_every=None,
    finite_check_every=25,
    dtype=np.float64,
):
    """``PennesSolver.solve`` (pennes.py:451-689); returns a dict of float32 maps."""
    dtype = np.dtype(dtype).type
    shape = tuple(np.shape(k))
    n_steps = int(n_steps)
    if n_steps < 1:
        raise ValueError(f"n_steps must be >= 1, got {n_steps}")
    if dose0 is not None and not dose:
        raise ValueError("dose0 was given but dose=False")
    ref_c = arterial_temperature_c if reference_temperature_c is None else reference_temperature_c
    wall_c = arterial_temperature_c if boundary_temperature_c is None else boundary_temperature_c
    t_ref = np.float32(ref_c)
    theta = np.asarray(np.asarray(temperature0, np.float32), dtype=dtype) - t_ref
    if not bool(np.isfinite(theta).all()):
        raise ValueError("temperature0 contains non-finite values")
    q_dev = None
    if q is not None:
        arr = np.asarray(q, dtype=np.float32)
        if arr.ndim == 0:
            arr = np.full(shape, float(arr), dtype=np.float32)
        q_dev = np.asarray(arr, dtype=dtype)

    faces, walls, perf, inv_rho_c, dt_stable = coefficients(
        k, rho, specific_heat, perfusion, dx, dtype, boundary=boundary,
        blood_density=blood_density, blood_specific_heat=blood_specific_heat,
    )
    perfused = bool((np.asarray(perfusion) > 0).any())
    if dt <= dt_stable:
        n_sub = 1
    elif on_unstable == "substep":
        n_sub = int(ceil(dt / dt_stable))
    else:
        raise OracleThermalStability(f"dt = {dt:.6g} s is above the stability bound {dt_stable:.6g} s")
    dt_sub = dt / n_sub
    coeff = (inv_rho_c * np.float32(dt_sub)).astype(dtype)
    ref_minus_ta = np.float32(ref_c - arterial_temperature_c)
    perf_offset = (perf * ref_minus_ta).astype(dtype) if perfused and float(ref_minus_ta) != 0.0 else None
    theta_wall = np.float32(wall_c) - t_ref

    work = np.zeros(shape, dtype=dtype)
    diff_bufs = [np.zeros(_ax(theta, ax, slice(None, -1)).shape, dtype=dtype) for ax in range(len(shape))]
    theta_max = theta.copy()
    dose_map = None
    rate = None
    if dose:
        dose_map = (
            np.zeros(shape, dtype=dtype)
            if dose0 is None
            else np.asarray(np.asarray(dose0, dtype=np.float32), dtype=dtype).copy()
        )
        rate = cem43_rate(theta + t_ref)
    half_dt_min = np.float32(0.5 * dt_sub / 60.0)
    samples, times = [], []
    if record_every is not None:
        samples.append(np.asarray(theta, np.float32) + t_ref)
        times.append(0.0)

    def guard(step):
        for what, arr in (("temperature", theta), ("CEM43 dose", dose_map)):
            if arr is not None and not bool(np.isfinite(arr).all()):
                raise OracleThermalDiverged(f"the {what} field stopped being finite at outer step {step}")

    for step in range(1, n_steps + 1):
        for _ in range(n_sub):
            work.fill(0)
            for ax, kf in enumerate(faces):
                buf = diff_bufs[ax]
                np.subtract(_ax(theta, ax, slice(1, None)), _ax(theta, ax, slice(None, -1)), out=buf)
                buf *= kf
                _ax(work, ax, slice(None, -1))[...] += buf
                _ax(work, ax, slice(1, None))[...] -= buf
            if walls is not None:
                for ax, (lo, hi) in enumerate(walls):
                    _ax(work, ax, slice(0, 1))[...] += lo * (theta_wall - _ax(theta, ax, slice(0, 1)))
                    _ax(work, ax, slice(-1, None))[...] += hi * (theta_wall - _ax(theta, ax, slice(-1, None)))
            if q_dev is not None:
                work += q_dev
            if perfused:
                work -= perf * theta
                if perf_offset is not None:
                    work -= perf_offset
            work *= coeff
            theta += work
            np.maximum(theta_max, theta, out=theta_max)
            if dose_map is not None:
                new_rate = cem43_rate(theta + t_ref)
                increment = new_rate + rate
                increment *= half_dt_min
                dose_map += increment
                rate = new_rate
        if record_every is not None and step % record_every == 0:
            samples.append(np.asarray(theta, np.float32) + t_ref)
            times.append(step * dt)
        if step % finite_check_every == 0 and step != n_steps:
            guard(step)
    guard(n_steps)
    if record_every is not None and (not times or times[-1] != n_steps * dt):
        samples.append(np.asarray(theta, np.float32) + t_ref)
        times.append(n_steps * dt)
    return {
        "temperature": np.array(theta, dtype=np.float32, copy=True) + t_ref,
        "temperature_max": np.array(theta_max, dtype=np.float32, copy=True) + t_ref,
        "dose_cem43": None if dose_map is None else np.array(dose_map, dtype=np.float32, copy=True),
        "theta": theta,
        "theta_max": theta_max,
        "dose_raw": dose_map,
        "samples": samples,
        "times": times,
        "dt": float(dt),
        "n_steps": n_steps,
        "t_end_s": float(dt * n_steps),
        "substeps": n_sub,
        "dt_stable_s": dt_stable,
    }

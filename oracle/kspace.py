"""Oracle: k-space PSTD CW solve (linear / Westervelt) in NumPy + scipy.fft.

TEST INFRASTRUCTURE ONLY (see :mod:`oracle`). A restatement of the
reference's engine, one function per reference function, each citing the
reference file:line it follows (relative to ``src/caustica/``).

``dtype=np.float64`` is the FP64 oracle: it reproduces the reference engine
run through a backend whose ``xp.float32``/``xp.complex64`` read as
float64/complex128. Host-side NumPy arithmetic that the reference performs on
its float32 medium arrays *before* the backend sees them (``dt / rho``,
``exp(-alpha c dt)``, ``beta * 2 dt``, the float32 phases) keeps its float32
rounding here too, exactly as it does in that run. ``dtype=np.float32`` is
the reference's stock CPU path (the CPU baseline).
"""

from __future__ import annotations

from itertools import product
from math import ceil, floor, isfinite

import numpy as np
import scipy.fft as spfft


class OracleDiverged(RuntimeError):
    """Mirror of ``SolverDivergedError`` (solvers/base.py:34-41)."""


# --------------------------------------------------------------------------
# operators.py
# --------------------------------------------------------------------------


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
    """operators.py:37-39."""
    return tuple(optimal_fft_size(n) for n in shape)


def pad_volume(vol: np.ndarray, padded) -> np.ndarray:
    """High-end edge replication (operators.py:42-57)."""
    pad = [(0, want - have) for have, want in zip(vol.shape, padded, strict=True)]
    if all(p == (0, 0) for p in pad):
        return vol
    return np.pad(vol, pad, mode="edge")


def k_vectors(shape, dx: float, dtype) -> list[np.ndarray]:
    """Broadcast k per axis, rfft layout on the last axis (operators.py:60-73)."""
    ks = []
    nd = len(shape)
    for ax, n in enumerate(shape):
        if ax == nd - 1:
            k = 2.0 * np.pi * np.fft.rfftfreq(n, d=dx)
        else:
            k = 2.0 * np.pi * np.fft.fftfreq(n, d=dx)
        arr = np.asarray(k, dtype=dtype)
        sh = [1] * nd
        sh[ax] = arr.size
        ks.append(arr.reshape(sh))
    return ks


def kappa_sinc(ks, c_ref: float, dt: float, dtype) -> np.ndarray:
    """sinc(c_ref |k| dt / 2) (operators.py:76-87)."""
    k2 = ks[0] ** 2
    for k in ks[1:]:
        k2 = k2 + k**2
    return np.sinc(c_ref * np.sqrt(k2) * (dt / (2.0 * np.pi))).astype(dtype)


def spectral_derivative_factors(ks, kappa, shape, cdtype) -> list[np.ndarray]:
    """i k_ax kappa with the Nyquist bin zeroed on even axes (operators.py:90-142)."""
    out = []
    for ax, k in enumerate(ks):
        if shape[ax] % 2 == 0:
            k = k.copy()
            idx = [0] * k.ndim
            idx[ax] = shape[ax] // 2
            k[tuple(idx)] = 0.0
        out.append((1j * k * kappa).astype(cdtype))
    return out


# --------------------------------------------------------------------------
# core/pml.py
# --------------------------------------------------------------------------


def sponge_profile_1d(n: int, width: int, edge: float, dtype) -> np.ndarray:
    """exp(-edge ((w - r)/w)^2) ramps at both ends (core/pml.py:210-230)."""
    if 2 * width > n:
        raise ValueError(f"sponge width {width} does not fit twice into length {n}")
    s = np.ones(n, dtype=dtype)
    if width > 0:
        r = np.arange(width, dtype=dtype)
        ramp = np.exp(-edge * ((width - r) / width) ** 2)
        s[:width] = ramp
        s[-width:] = ramp[::-1]
    return s


def sponge_volume(shape, width: int, edge: float, dtype) -> np.ndarray:
    """Separable product ((1*s_0)*s_1)*s_2 (operators.py:145-157)."""
    out = np.ones(shape, dtype=dtype)
    for ax, n in enumerate(shape):
        prof = sponge_profile_1d(n, width, edge, dtype)
        sh = [1] * len(shape)
        sh[ax] = n
        out = out * prof.reshape(sh)
    return out


def pml_vox(thickness: float, dx: float) -> int:
    """PMLSpec.thickness_vox (core/pml.py:203-207)."""
    return int(round(thickness / dx))


# --------------------------------------------------------------------------
# engine.py / sources.py / base.py helpers
# --------------------------------------------------------------------------


def cw_discretization(dx, c_max, f0, cfl=0.48, cfl_hard_max=0.50, harmonics=(1,)):
    """Exact-period (spp, dt) under the CFL limit (engine.py:86-113)."""
    period = 1.0 / f0
    dt_cfl = cfl * dx / c_max
    spp = max(2, int(floor(period / dt_cfl)))
    dt = period / spp
    while dt * c_max / dx > cfl_hard_max + 1e-12 and spp < 1024:
        spp += 1
        dt = period / spp
    h_max = max(harmonics)
    if 2 * h_max >= spp:
        raise ValueError(f"harmonic {h_max} is at/above the temporal Nyquist for spp={spp}")
    return spp, dt


def cw_tof_periods(shape, dx, c_min, f0, src_idx, reference_point=None) -> int:
    """Periods of flight to the farthest corner or the reference (engine.py:116-134)."""
    period = 1.0 / f0
    src_pos = np.asarray(src_idx).astype(np.float64) * dx
    if reference_point is not None:
        refs = np.asarray(reference_point, np.float64)[None, :] * dx
    else:
        refs = np.array(list(product(*((0, n - 1) for n in shape))), np.float64) * dx
    dmax = max(float(np.sqrt(((src_pos - r) ** 2).sum(axis=1)).max()) for r in refs)
    return max(1, int(ceil(dmax / c_min / period)))


def ramp_envelope(t: float, period: float, ramp_periods: float) -> float:
    """Cosine taper 0 -> 1 (sources.py:98-102)."""
    t_ramp = ramp_periods * period
    x = min(t / t_ramp, 1.0)
    return 0.5 * (1.0 - np.cos(np.pi * x))


def interior_slices(shape, margin: int):
    """solvers/base.py:123-129."""
    if any(n <= 2 * margin for n in shape):
        raise ValueError(f"margin {margin} leaves no interior for shape {shape}")
    return tuple(slice(margin, n - margin) for n in shape)


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


def medium_maps(alpha, rho, c, beta, padded, dt, nonlinear, dtype):
    """Per-voxel update coefficients (engine.py:239-249).

    The reference computes these with host NumPy on float32 volumes, so
    ``dt/rho``, ``exp(-alpha c dt)`` and ``2 beta dt`` carry float32
    rounding in every backend; ``rho c^2 dt`` is formed in float64.
    """
    alpha = np.asarray(alpha, np.float32)
    rho = np.asarray(rho, np.float32)
    c = np.asarray(c, np.float32)
    beta = np.asarray(beta, np.float32)
    dt_over_rho = np.asarray(dt / pad_volume(rho, padded), dtype=dtype)
    rhoc2_dt = np.asarray(pad_volume(rho * c.astype(np.float64) ** 2, padded) * dt, dtype=dtype)
    absorb = np.asarray(np.exp(-pad_volume(alpha * c, padded) * dt), dtype=dtype)
    beta2_dt = None
    if nonlinear and not bool((beta == 0).all()):
        beta2_dt = np.asarray(pad_volume(beta, padded) * (2.0 * dt), dtype=dtype)
    return dt_over_rho, rhoc2_dt, absorb, beta2_dt


# --------------------------------------------------------------------------
# the solve: engine.py:167-586 (checkpoint and progress hooks omitted)
# --------------------------------------------------------------------------


def run_cw(
    *,
    shape,
    dx,
    pml_vox_n,
    pml_edge=2.0,
    alpha,
    rho,
    c,
    beta,
    src_idx,
    src_phase,
    amplitude,
    f0,
    ramp_periods=3.0,
    cfl=0.48,
    cfl_hard_max=0.50,
    min_settle_periods=8,
    max_settle_periods=96,
    convergence_tol=0.01,
    n_record_periods=2,
    t_end_min_us=None,
    nonlinear=False,
    harmonics=(1,),
    record_region=None,
    reference_point=None,
    dtype=np.float64,
    workers=1,
    solver_name="oracle",
):
    """One steady-state CW solve; returns a dict shaped like ``SolverResult``.

    Follows ``run_cw_kspace_pstd`` (engine.py:167-586): discretisation
    (234), padded maps (236-249), k-space operators (251-254), sponge (263),
    source scale (268-278), time of flight and settle bounds (281-290),
    convergence region (293-296), the step (458-482), the settle loop
    (484-510), the t_end floor (513-520) and the record window (535-556).
    """
    dtype = np.dtype(dtype).type
    cdtype = np.complex128 if dtype == np.float64 else np.complex64
    shape = tuple(int(s) for s in shape)
    nd = len(shape)
    harmonics = tuple(dict.fromkeys(int(h) for h in harmonics))
    if not harmonics or harmonics[0] != 1 or any(h < 1 for h in harmonics):
        raise ValueError(f"harmonics must start with 1 (fundamental), got {harmonics}")
    alpha = np.asarray(alpha, np.float32)
    rho = np.asarray(rho, np.float32)
    c = np.asarray(c, np.float32)
    beta = np.asarray(beta, np.float32)
    src_idx = np.asarray(src_idx, np.int64)
    src_phase = np.asarray(src_phase, np.float32)
    c_max = float(c.max())
    c_min = float(c.min())
    period = 1.0 / f0
    omega = 2.0 * np.pi * f0

    spp, dt = cw_discretization(dx, c_max, f0, cfl, cfl_hard_max, harmonics)
    active = tuple(slice(0, n) for n in shape)
    padded = pad_shape(shape)
    dt_over_rho, rhoc2_dt, absorb, beta2_dt = medium_maps(
        alpha, rho, c, beta, padded, dt, nonlinear, dtype
    )
    ks = k_vectors(padded, dx, dtype)
    kappa = kappa_sinc(ks, c_max, dt, dtype)
    deriv = spectral_derivative_factors(ks, kappa, padded, cdtype)
    del ks, kappa
    sponge = sponge_volume(padded, pml_vox_n, pml_edge, dtype)

    p = np.zeros(padded, dtype=dtype)
    u = [np.zeros(padded, dtype=dtype) for _ in range(nd)]
    sidx = tuple(src_idx[:, d] for d in range(nd))
    src_ph = np.asarray(src_phase, dtype=dtype)
    c_src = c[sidx]
    src_scale = np.asarray(2.0 * c_src.astype(np.float64) * dt / dx, dtype=dtype)

    tof = cw_tof_periods(shape, dx, c_min, f0, src_idx, reference_point)
    eff_min = tof + max(min_settle_periods, int(ceil(ramp_periods)) + 1)
    eff_max = max(tof + max_settle_periods, eff_min)
    margin = pml_vox_n + 2
    if any(n <= 2 * margin for n in shape):
        margin = 0
    conv = interior_slices(shape, margin)
    rec = normalize_record_region(record_region, shape) if record_region is not None else active

    axes = tuple(range(nd))

    def rfftn(a):
        return spfft.rfftn(a, axes=axes, workers=workers)

    def irfftn(a):
        return spfft.irfftn(a, s=padded, axes=axes, workers=workers)

    def step(n: int) -> None:
        pk = rfftn(p)
        for i in range(nd):
            grad_i = irfftn(deriv[i] * pk)
            u[i] -= dt_over_rho * grad_i
            u[i] *= absorb
            u[i] *= sponge
        acc = None
        for i in range(nd):
            term = deriv[i] * rfftn(u[i])
            acc = term if acc is None else acc + term
        divu = irfftn(acc)
        if beta2_dt is None:
            p[...] -= rhoc2_dt * divu
        else:
            p[...] -= (rhoc2_dt + beta2_dt * p) * divu
        p[...] *= absorb
        p[...] *= sponge
        t = n * dt
        env = ramp_envelope(t, period, ramp_periods)
        p[sidx] += (dtype(amp * env) * src_scale) * np.sin(dtype(omega * t) - src_ph)

    amp = float(amplitude)
    n = 0
    prev_peak = None
    converged = False
    converged_period = eff_max
    history = []
    periods_done = 0
    period_peaks = []
    period_idx = 0
    while not converged and period_idx < eff_max:
        period_idx += 1
        period_peak = dtype(0.0)
        for _ in range(spp):
            step(n)
            n += 1
            period_peak = np.maximum(period_peak, np.abs(p[conv]).max())
        peak = float(period_peak)
        period_peaks.append(peak)
        if not isfinite(peak):
            raise OracleDiverged(f"solver '{solver_name}' diverged in settling period {period_idx}")
        periods_done = period_idx
        rel = abs(peak - prev_peak) / max(prev_peak, 1e-9) if prev_peak is not None else None
        if period_idx >= tof:
            history.append((period_idx, peak, float("nan") if rel is None else rel))
        if period_idx >= eff_min and rel is not None:
            if peak > 0.0 and rel < convergence_tol:
                converged_period = period_idx
                converged = True
        if not converged:
            prev_peak = peak

    if t_end_min_us is not None:
        need = ceil(t_end_min_us * 1e-6 / period) - n_record_periods
        while periods_done < need:
            for _ in range(spp):
                step(n)
                n += 1
            periods_done += 1

    rec_steps = n_record_periods * spp
    buffers = {h: np.zeros(p[rec].shape, dtype=cdtype) for h in harmonics}
    pmax = np.zeros(p[rec].shape, dtype=dtype)
    for _ in range(rec_steps):
        step(n)
        t = n * dt
        pa = p[rec]
        for h in harmonics:
            buffers[h] += pa * np.exp(cdtype(+1j * h * omega * t))
        np.maximum(pmax, np.abs(pa), out=pmax)
        n += 1
    for h in harmonics:
        buffers[h] *= cdtype(2.0 / rec_steps)
    if not isfinite(float(pmax.max())):
        raise OracleDiverged(f"solver '{solver_name}' diverged in the record window")
    return {
        "phasor": buffers[1],
        "phasors": buffers,
        "p_max": pmax,
        "region": rec,
        "dt": dt,
        "spp": spp,
        "steps_total": n,
        "t_end_s": n * dt,
        "tof_periods": tof,
        "converged_period": converged_period,
        "settle_capped": not converged,
        "convergence_history": history,
        "period_peaks": period_peaks,
        "eff_min": eff_min,
        "eff_max": eff_max,
        "p": p,
        "u": u,
    }


def step_fields(*, p, u, dt_over_rho, rhoc2_dt, absorb, beta2_dt, sponge, deriv, padded):
    """One bare step of the scheme (engine.py:458-477) without the source.

    Used by the single-step parity tests: it advances ``p`` and ``u`` in
    place exactly as the engine's ``step`` does before source injection.
    """
    nd = len(padded)
    axes = tuple(range(nd))
    pk = spfft.rfftn(p, axes=axes)
    for i in range(nd):
        grad_i = spfft.irfftn(deriv[i] * pk, s=padded, axes=axes)
        u[i] -= dt_over_rho * grad_i
        u[i] *= absorb
        u[i] *= sponge
    acc = None
    for i in range(nd):
        term = deriv[i] * spfft.rfftn(u[i], axes=axes)
        acc = term if acc is None else acc + term
    divu = spfft.irfftn(acc, s=padded, axes=axes)
    if beta2_dt is None:
        p -= rhoc2_dt * divu
    else:
        p -= (rhoc2_dt + beta2_dt * p) * divu
    p *= absorb
    p *= sponge
    return p, u

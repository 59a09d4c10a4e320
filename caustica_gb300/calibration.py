"""Planner calibration for the GB300 backend (planner/calibration.py:151-584).

caustica's planner predicts a solve's step time from per-device samples
``(P, t_step)`` (P = padded cell count) kept in ``~/.caustica/calibration.json``
under the device's product name; :func:`calibrate` measures those samples with
this backend's own step (the size-specialised passes, one CUDA graph per
period, CUDA events on the solver stream) and writes an entry in the
reference's schema, so ``caustica.planner.estimate(..., gpu=<this device>)``
plans GB300 solves from GB300 numbers. The entry keeps the reference's fields
(``a``/``b`` of ``t = a P log2 P + b P`` fitted by nonnegative least squares,
the samples, the probe shapes, warm-up and peak-memory figures).

Only the measurement needs a GPU; the probe sizing, the fit and the file
update are plain host code.
"""

from __future__ import annotations

import ctypes as C
import json
import time
from datetime import datetime
from pathlib import Path

import numpy as np

# cubic probe sides with a size-specialised pencil split (every axis on the
# fast passes), smallest first
PROBE_SIDES = (96, 128, 160, 192, 256, 320, 400, 512, 640)
# fractions of free device memory the probes are sized to occupy
PROBE_MEMORY_FRACTIONS = (0.01, 0.04, 0.10)
# below this many cells a probe times launch latency, not throughput
MIN_PROBE_CELLS = 2_000_000
# above this the global (a, b) law misses its own samples (the entry then
# anchors on the largest, most throughput-bound sample)
FIT_RESIDUAL_LIMIT = 0.10


def default_calibration_path() -> Path:
    return Path.home() / ".caustica" / "calibration.json"


def device_name() -> str:
    """Product name of the executing GPU (the key of its calibration entry)."""
    import torch

    return torch.cuda.get_device_name(torch.cuda.current_device())


def probe_footprint_bytes(n: int, nonlinear: bool = False) -> int:
    """Device bytes of an n^3 probe handle (state, spectra, label map, tables)."""
    cells = n ** 3
    spec = n * n * (n // 2 + 1)
    return 4 * cells + 12 * cells + 3 * 8 * spec + cells + (64 << 20)


def probe_shapes_for_budget(free_bytes: int, nonlinear: bool = False) -> tuple[tuple[int, int, int], ...]:
    """Cubic probes sized to PROBE_MEMORY_FRACTIONS of ``free_bytes``; at
    least two, the largest at least MIN_PROBE_CELLS (else 128^3 and 192^3)."""
    chosen: list[int] = []
    for frac in PROBE_MEMORY_FRACTIONS:
        fit = [n for n in PROBE_SIDES if probe_footprint_bytes(n, nonlinear) <= free_bytes * frac]
        if fit and fit[-1] not in chosen:
            chosen.append(fit[-1])
    if len(chosen) < 2 or chosen[-1] ** 3 < MIN_PROBE_CELLS:
        chosen = [128, 192]
    return tuple((n, n, n) for n in chosen)


def fit_time_model(samples) -> tuple[float, float]:
    """Nonnegative least squares for ``t = a P log2(P) + b P``
    (planner/calibration.py:291-310): the unconstrained two-term fit, or the
    best one-term fit when a coefficient comes out negative."""
    p = np.array([s[0] for s in samples], np.float64)
    t = np.array([s[1] for s in samples], np.float64)
    cols = np.stack([p * np.log2(p), p], axis=1)
    a, b = np.linalg.lstsq(cols, t, rcond=None)[0]
    if a < 0.0:
        a, b = 0.0, float(np.linalg.lstsq(cols[:, 1:], t, rcond=None)[0][0])
    elif b < 0.0:
        a, b = float(np.linalg.lstsq(cols[:, :1], t, rcond=None)[0][0]), 0.0
    return max(float(a), 0.0), max(float(b), 0.0)


def max_rel_residual(samples, a: float, b: float) -> float:
    """Worst relative miss of the (a, b) law on the samples it was fitted to."""
    worst = 0.0
    for p, t in samples:
        if t > 0.0:
            worst = max(worst, abs(a * p * np.log2(p) + b * p - t) / t)
    return float(worst)


def loo_rel_error(samples) -> float | None:
    """Leave-one-out relative error of log-log interpolation between the
    remaining samples (interior samples only; None with fewer than three)."""
    s = sorted((int(p), float(t)) for p, t in samples)
    if len(s) < 3:
        return None
    worst = 0.0
    for i in range(1, len(s) - 1):
        (p0, t0), (p1, t1) = s[i - 1], s[i + 1]
        w = (np.log(s[i][0]) - np.log(p0)) / (np.log(p1) - np.log(p0))
        pred = float(np.exp(np.log(t0) + w * (np.log(t1) - np.log(t0))))
        worst = max(worst, abs(pred - s[i][1]) / s[i][1])
    return float(worst)


def measure_step_time(shape, nonlinear: bool = False, n_steps: int = 20, warmup: int = 3) -> dict:
    """Per-step device time of this backend's step on a homogeneous water
    probe of ``shape`` (same keys as planner/calibration.py:151-258).

    ``warmup_s`` is the one-time cost before the per-step clock is
    meaningful (plan, handle creation with its autotuning, the first
    periods), less what those periods cost at the steady rate.
    """
    from . import _lib
    from . import engine as eng
    from .contract import CWRunSpec, CWSource, Grid, Medium, PMLSpec

    t_cold0 = time.perf_counter()
    shape = tuple(int(n) for n in shape)
    dx = 0.25e-3
    grid = Grid(shape, dx, PMLSpec(10 * dx))
    med = Medium.homogeneous(shape, alpha_np_m=0.5, c=1500.0, rho=1000.0, beta=3.5 if nonlinear else 0.0)
    idx = np.array([[n // 2 for n in shape[:-1]] + [12]], np.int64)
    src = CWSource(indices=idx, phases=np.zeros(1, np.float32), amplitude=1e5, f0=1e6)
    plan = eng.make_plan("calibration", grid, med, src, CWRunSpec(cfl=0.3), nonlinear=nonlinear)
    periods = max(1, -(-int(n_steps) // plan.spp))
    free0 = _free_bytes()
    with eng.DeviceSolver(plan) as dev:
        dev.extend_drive((warmup + periods + 1) * plan.spp)
        ms = C.c_float(0.0)
        _lib.call("cg_solver_timed_run", dev.h, warmup * plan.spp, 0, 1, C.byref(ms))
        dev.synchronize()
        t_cold = time.perf_counter() - t_cold0
        _lib.call("cg_solver_timed_run", dev.h, periods * plan.spp, 0, 1, C.byref(ms))
        dev.synchronize()
        free1 = _free_bytes()
        footprint = dev.footprint_bytes()
    t_step = float(ms.value) * 1e-3 / (periods * plan.spp)
    peak = (free0 - free1) if (free0 is not None and free1 is not None and free0 > free1) else footprint
    return {"device": device_name(), "backend": "gb300", "shape": shape, "p_elems": int(plan.ncell),
            "t_step_s": t_step, "warmup_s": max(0.0, t_cold - warmup * plan.spp * t_step),
            "vram_peak_bytes": int(peak)}


def _free_bytes() -> int | None:
    try:
        import torch

        return int(torch.cuda.mem_get_info()[0])
    except Exception:  # noqa: BLE001 - no torch CUDA context: the footprint estimate stands in
        return None


def make_entry(runs: list[dict], n_steps: int, nonlinear: bool) -> dict:
    """The calibration entry for measured ``runs`` (planner/calibration.py:520-574)."""
    samples = [(int(r["p_elems"]), float(r["t_step_s"])) for r in runs]
    a, b = fit_time_model(samples)
    residual = max_rel_residual(samples, a, b)
    mode = "nnls"
    if residual > FIT_RESIDUAL_LIMIT:
        p_big, t_big = max(samples)
        a, b, mode = 0.0, t_big / p_big, "throughput-anchored"
        residual = max_rel_residual(samples, a, b)
    later = runs[1:]
    per_elem = min(float(r["warmup_s"]) / max(int(r["p_elems"]), 1) for r in later) if later else 0.0
    context = max(0.0, float(runs[0]["warmup_s"]) - per_elem * int(runs[0]["p_elems"]))
    return {
        "a": a, "b": b, "fit_mode": "interpolated", "global_fit_mode": mode,
        "fit_max_rel_residual": residual, "interp_loo_rel_err": loo_rel_error(samples),
        "p_max_probe": max(p for p, _ in samples), "warmup_context_s": context, "warmup_per_elem_s": per_elem,
        "warmup_s": max(float(r["warmup_s"]) for r in runs), "warmup_source": "probe",
        "backend": "gb300", "n_steps": int(n_steps), "nonlinear": bool(nonlinear),
        "samples": [[p, t] for p, t in samples],
        "shapes": ["x".join(map(str, r["shape"])) for r in runs],
        "vram_peak_bytes_by_shape": {"x".join(map(str, r["shape"])): r["vram_peak_bytes"] for r in runs},
        "calibrated_at": datetime.now().astimezone().isoformat(timespec="seconds"),
    }


def write_entry(device: str, entry: dict, path: str | Path | None = None) -> Path:
    """Store ``entry`` under ``device`` in the calibration file (other devices kept)."""
    target = Path(path) if path is not None else default_calibration_path()
    target.parent.mkdir(parents=True, exist_ok=True)
    data = json.loads(target.read_text()) if target.exists() else {"version": 1, "devices": {}}
    data.setdefault("devices", {})[device] = entry
    target.write_text(json.dumps(data, indent=2))
    return target


def calibrate(shapes=None, *, nonlinear: bool = False, n_steps: int = 20, path: str | Path | None = None) -> dict:
    """Measure ``shapes`` (default: sized to this device's free memory) and
    persist the entry under this device's name; returns the entry."""
    if shapes is None:
        free = _free_bytes()
        shapes = probe_shapes_for_budget(free) if free else ((128,) * 3, (192,) * 3)
    if len(shapes) < 2:
        raise ValueError("calibration needs >= 2 grid sizes to fit a*P*log2(P) + b*P")
    runs = [measure_step_time(s, nonlinear=nonlinear, n_steps=n_steps) for s in shapes]
    entry = make_entry(runs, n_steps, nonlinear)
    write_entry(runs[0]["device"], entry, path)
    return entry


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--nonlinear", action="store_true")
    ap.add_argument("--n-steps", type=int, default=20)
    ap.add_argument("--path", default=None)
    args = ap.parse_args()
    print(json.dumps(calibrate(nonlinear=args.nonlinear, n_steps=args.n_steps, path=args.path), indent=2))

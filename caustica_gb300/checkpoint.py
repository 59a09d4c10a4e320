"""Checkpoint / resume of the device state at period boundaries.

Same container and policy as the reference (io/checkpoint.py:40-226,
engine.py:303-371, 436-451, 522-534): an uncompressed ``.npz`` holding
``meta_json`` (format ``caustica-checkpoint/1``), ``history`` and the
``field_*`` volumes, written atomically every ``every_periods`` periods, a
pre-record snapshot, resume when the fingerprint matches, refusal when it
does not, and a graceful stop through ``stop_when``. The scheme tag is
``cw-kspace-gb300/1``: a GB300 trajectory is float32 on a different FFT and
is not bit-identical to the reference's, so the two never splice.
"""

from __future__ import annotations

import hashlib
import json
import os
import tempfile
import time
from dataclasses import dataclass, field
from pathlib import Path
from typing import Any, Callable

import numpy as np

from .engine import DeviceSolver, Plan, _emit, _guard_finite, _results

CHECKPOINT_FORMAT = "caustica-checkpoint/1"
SCHEME = "cw-kspace-gb300/1"


class RunInterrupted(RuntimeError):
    """Graceful stop on ``stop_when`` (io/checkpoint.py:51-67)."""

    def __init__(self, checkpoint_path, stage: str, periods_done: int, steps_done: int):
        super().__init__(f"run interrupted on request at period {periods_done} (stage '{stage}', {steps_done} "
                         f"steps); state saved to {checkpoint_path} — rerun the same call to resume.")
        self.checkpoint_path = Path(checkpoint_path)
        self.stage = stage
        self.periods_done = periods_done
        self.steps_done = steps_done


class CheckpointMismatch(RuntimeError):
    """The checkpoint on disk belongs to a different run (io/checkpoint.py:70-71)."""


@dataclass
class CheckpointSpec:
    """Checkpoint policy (io/checkpoint.py:74-109)."""

    path: Path
    every_periods: int = 8
    stop_when: Callable[[], bool] | None = field(default=None, compare=False)
    keep_on_success: bool = False

    def __post_init__(self) -> None:
        self.path = Path(self.path)
        if self.every_periods < 1:
            raise ValueError(f"every_periods must be >= 1, got {self.every_periods}")


def arrays_sha1(*arrays) -> str:
    h = hashlib.sha1()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(str(a.dtype).encode())
        h.update(str(a.shape).encode())
        h.update(a.tobytes())
    return h.hexdigest()


def _fp_json(fp: dict) -> str:
    return json.dumps(fp, sort_keys=True, separators=(",", ":"))


def fingerprint(plan: Plan, grid, medium, source) -> dict[str, Any]:
    """Everything that shapes the trajectory (engine.py:306-334)."""
    spec = plan.spec
    dump = spec.model_dump() if hasattr(spec, "model_dump") else dict(spec.__dict__)
    return {
        "scheme": SCHEME, "solver": plan.name, "backend": "gb300", "grid_shape": list(plan.shape),
        "dx": plan.dx, "pml_vox": int(plan.pml3[2]), "pml_edge": plan.pml_edge, "spp": plan.spp, "f0": plan.f0,
        "amplitude": plan.amplitude, "ramp_periods": plan.ramp_periods, "harmonics": list(plan.harmonics),
        "nonlinear": plan.nonlinear_active, "record_region": [[s.start, s.stop] for s in plan.rec],
        "reference_point": plan.meta.get("reference_point"),
        "spec": {k: v for k, v in dump.items()},
        "source_sha1": arrays_sha1(source.indices, source.phases),
        "medium_sha1": arrays_sha1(medium.c, medium.rho, medium.alpha, medium.beta),
    }


def write(path: Path, *, stage, n, periods_done, prev_peak, converged, converged_period, history, fields, fp):
    meta = {"format": CHECKPOINT_FORMAT, "stage": stage, "n": int(n), "periods_done": int(periods_done),
            "prev_peak": None if prev_peak is None else float(prev_peak), "converged": bool(converged),
            "converged_period": int(converged_period), "fingerprint": fp}
    hist = np.asarray(history, dtype=np.float64).reshape(len(history), 3)
    payload = {"meta_json": np.asarray(json.dumps(meta)), "history": hist,
               **{f"field_{k}": np.ascontiguousarray(v) for k, v in fields.items()}}
    path = Path(path)
    fd, tmp = tempfile.mkstemp(dir=path.parent, prefix=path.name + ".", suffix=".tmp")
    try:
        with os.fdopen(fd, "wb") as fh:
            np.savez(fh, **payload)
        os.replace(tmp, path)
    finally:
        if os.path.exists(tmp):
            os.unlink(tmp)
    return path


def load(path: Path, fp: dict) -> dict | None:
    path = Path(path)
    if not path.exists():
        return None
    with np.load(path, allow_pickle=False) as npz:
        meta = json.loads(str(npz["meta_json"]))
        if meta.get("format") != CHECKPOINT_FORMAT:
            raise CheckpointMismatch(f"{path.name}: format {meta.get('format')!r} != {CHECKPOINT_FORMAT!r}")
        if _fp_json(meta["fingerprint"]) != _fp_json(fp):
            keys = sorted(set(meta["fingerprint"]) | set(fp))
            diff = [f"  {k}: checkpoint={meta['fingerprint'].get(k)!r} vs run={fp.get(k)!r}" for k in keys
                    if meta["fingerprint"].get(k) != fp.get(k)]
            raise CheckpointMismatch(f"{path.name} was written by a DIFFERENT run — refusing to splice "
                                     f"trajectories. Differing keys:\n" + "\n".join(diff))
        fields = {k[len("field_"):]: npz[k] for k in npz.files if k.startswith("field_")}
        hist = npz["history"]
    return {"stage": meta["stage"], "n": meta["n"], "periods_done": meta["periods_done"],
            "prev_peak": meta["prev_peak"], "converged": meta["converged"],
            "converged_period": meta["converged_period"],
            "history": [(int(p), float(pk), float(r)) for p, pk, r in hist], "fields": fields}


def _fields(dev: DeviceSolver, plan: Plan) -> dict:
    p, u = dev.get_state()
    out = {"p": p[0].reshape(plan.padded)}
    comps = list(range(3 - plan.nd, 3))
    for i, ci in enumerate(comps):
        out[f"u{i}"] = u[ci, 0].reshape(plan.padded)
    return out


def _restore(dev: DeviceSolver, plan: Plan, fields: dict, n: int) -> None:
    ncell = plan.ncell
    p = np.ascontiguousarray(fields["p"], np.float32).reshape(1, ncell)
    u = np.zeros((3, 1, ncell), np.float32)
    for i, ci in enumerate(range(3 - plan.nd, 3)):
        u[ci, 0] = np.asarray(fields[f"u{i}"], np.float32).reshape(ncell)
    dev.set_state(p, u, n)


def run_with_checkpoint(plan: Plan, checkpoint, *, progress=None, result_cls, grid, medium, source):
    """Period-by-period solve with checkpoint cadence, resume and graceful stop.

    The settle loop, the period-boundary order (progress, then the cadence
    write, then the stop poll), the t_end floor and the pre-record snapshot
    follow engine.py:436-451, 484-534. A checkpoint that belongs to another
    run is refused before any device memory is taken.
    """
    t0 = time.monotonic()
    spec = plan.spec
    fp = fingerprint(plan, grid, medium, source)
    every = int(getattr(checkpoint, "every_periods", 8))
    stop_when = getattr(checkpoint, "stop_when", None)
    path = Path(checkpoint.path)
    state = load(path, fp)
    with DeviceSolver(plan) as dev:
        n = 0
        prev_peak = None
        converged = False
        converged_period = plan.eff_max
        history: list = []
        periods_done = 0
        stage = "settle"
        if state is not None:
            _restore(dev, plan, state["fields"], state["n"])
            n, periods_done = state["n"], state["periods_done"]
            prev_peak, converged = state["prev_peak"], state["converged"]
            converged_period, history, stage = state["converged_period"], state["history"], state["stage"]

        def save(stage_now):
            write(path, stage=stage_now, n=n, periods_done=periods_done, prev_peak=prev_peak, converged=converged,
                  converged_period=converged_period, history=history, fields=_fields(dev, plan), fp=fp)

        def boundary(peak, rel):
            if progress is not None:
                _emit(progress, plan, dev, "settle", periods_done, peak, rel, t0)
            stop = stop_when is not None and stop_when()
            if stop or periods_done % every == 0:
                save("settle")
            if stop:
                raise RunInterrupted(path, "settle", periods_done, n)

        period_idx = periods_done
        while stage == "settle" and not converged and period_idx < plan.eff_max:
            period_idx += 1
            dev.run_periods(1)
            n += plan.spp
            peak = float(dev.read_peaks(period_idx - 1, 1)[0, 0])
            _guard_finite(peak, f"settling period {period_idx} (step {n})", plan.name)
            periods_done = period_idx
            rel = abs(peak - prev_peak) / max(prev_peak, 1e-9) if prev_peak is not None else None
            if period_idx >= plan.tof:
                history.append((period_idx, peak, float("nan") if rel is None else rel))
            if period_idx >= plan.eff_min and rel is not None and peak > 0.0 and rel < spec.convergence_tol:
                converged_period = period_idx
                converged = True
            if not converged:
                prev_peak = peak
            boundary(peak, rel)
        if spec.t_end_min_us is not None and stage == "settle":
            need = int(np.ceil(spec.t_end_min_us * 1e-6 / plan.period)) - spec.n_record_periods
            while periods_done < need:
                dev.run_periods(1)
                n += plan.spp
                periods_done += 1
                boundary(None, None)
        if stage == "settle":
            stage = "record"
            if progress is not None:
                _emit(progress, plan, dev, "record", periods_done, None, None, t0)
            save("record")
            if stop_when is not None and stop_when():
                raise RunInterrupted(path, "record", periods_done, n)
        rec_steps = spec.n_record_periods * plan.spp
        dev.begin_record()
        dev.run_periods(spec.n_record_periods, record=True)
        ph, pm = dev.finalize(rec_steps)
        n += rec_steps
        _guard_finite(float(pm[0].max()), f"the record window (step {n})", plan.name)
        if not getattr(checkpoint, "keep_on_success", False):
            path.unlink(missing_ok=True)
        common = dict(dt=plan.dt, spp=plan.spp, steps_total=n, t_end_s=n * plan.dt, tof_periods=plan.tof,
                      converged_period=converged_period, settle_capped=not converged, convergence_history=history,
                      meta={"solver": plan.name, "backend": "gb300", "padded_shape": plan.padded,
                            "c_ref": plan.c_max, "nonlinear_active": plan.nonlinear_active, "source": plan.label,
                            "checkpoint_scheme": SCHEME})
        return _results(plan, dev, ph, pm, common, 0, result_cls)

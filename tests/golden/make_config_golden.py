"""Generate the full-size parity fixtures of the benchmark workloads.

Runs the UNCHANGED reference (ebx0/caustica) in FP64 -- through the
``numpy64`` backend plugin of ``make_golden.py``, registered in the
reference's own backend registry -- on the four benchmark workloads at their
own sizes, with the inputs this package's ``workloads`` module builds:

* ``cfg1_linear_96x96x128``: linear bowl, 1,320 steps, fundamental;
* ``cfg2_westervelt_192x192x256``: Westervelt over layered tissue, 880 steps,
  harmonics 1-3;
* ``cfg3_pennes_96x96x128`` / ``cfg3_pennes_stress_96x96x128``: Q = 2 alpha I
  from cfg1's FP64 fundamental (``HeatingSource.from_phasors``), 400 heating
  + 1,200 chained cooling steps of 0.05 s with CEM43 dose; the stress variant
  multiplies Q by 2000 so the temperature rise reaches ~10 K;
* ``cfg4_steer_160x160x192``: four of the 64 steering positions of the
  256-element spiral over the ellipsoid medium, each solved alone.

The whole fields are too large to commit, so each fixture holds the inputs
that are not reproducible from a seed alone (label maps, source voxels,
phases), the run bookkeeping, the reference's ``focus_metrics`` dictionary,
and the fields on (a) a full-resolution box around the focus and (b) a
regular lattice over the whole record region (every s-th voxel per axis).

Usage (hours of FP64 CPU time for all four; the fixtures are committed, so
the tests never need the reference)::

    python tests/golden/make_config_golden.py /path/to/caustica/src [cfg1 cfg2 cfg3 cfg4]
"""

from __future__ import annotations

import json
import os
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent

FOCAL_BOX = (16, 16, 32)
LATTICE_TARGET = 45000  # lattice voxels per fixture field


def lattice_stride(shape) -> int:
    n = int(np.prod(shape))
    return max(1, int(round((n / LATTICE_TARGET) ** (1.0 / len(shape)))))


def lattice(a: np.ndarray, s: int) -> np.ndarray:
    """Every s-th voxel per axis, starting at s // 2."""
    return np.ascontiguousarray(a[tuple(slice(s // 2, None, s) for _ in range(a.ndim))])


def focal_box(shape, centre, box=FOCAL_BOX):
    """Half-open box of size ``box`` around ``centre``, shifted to fit ``shape``."""
    lo = [min(max(0, c - b // 2), n - b) for c, b, n in zip(centre, box, shape)]
    return [[int(a), int(a + b)] for a, b in zip(lo, box)]


def _box(a: np.ndarray, box) -> np.ndarray:
    return np.ascontiguousarray(a[tuple(slice(lo, hi) for lo, hi in box)])


def _ref_objects(w):
    from caustica import Grid, Medium, PMLSpec
    from caustica.solvers import CWRunSpec
    from caustica.sources import CWSource

    g, m, s, sp = w["grid"], w["medium"], w["source"], w["spec"]
    grid = Grid(g.shape, g.dx, PMLSpec(g.pml.thickness, g.pml.edge))
    med = Medium(alpha=m.alpha, rho=m.rho, c=m.c, beta=m.beta)
    src = CWSource(indices=s.indices, phases=s.phases, amplitude=s.amplitude, f0=s.f0, ramp_periods=s.ramp_periods)
    spec = CWRunSpec(**sp.model_dump())
    return grid, med, src, spec


def _labels_of(medium):
    """(uint8 labels, float32 table rows alpha, rho, c, beta) of a label-built medium."""
    ids = np.asarray(medium.id_map if medium.id_map is not None else np.zeros(medium.shape, np.int32))
    present = np.unique(ids)
    table = np.zeros((int(present.max()) + 1, 4), np.float32)
    for i in present:
        at = tuple(int(v[0]) for v in np.nonzero(ids == i))
        table[i] = [medium.alpha[at], medium.rho[at], medium.c[at], medium.beta[at]]
    return ids.astype(np.uint8), table


def run_acoustic(w, solver: str, source=None):
    import caustica.solvers as solvers

    grid, med, src, spec = _ref_objects(w)
    if source is not None:
        src = source
    t0 = time.time()
    res = solvers.get(solver)().run(grid, med, src, spec, backend="numpy64", harmonics=w["harmonics"],
                                    reference_point=w["reference_point"])
    return res, time.time() - t0


def _metrics(res, w, apex, focus):
    from caustica.report.metrics import FieldFrame, focus_metrics

    g = w["grid"]
    frame = FieldFrame(dx=g.dx, grid_shape=g.shape, pml_vox=g.pml_vox, apex_vox=apex, focus_vox=focus)
    return focus_metrics(res, frame, source_amplitude=w["source"].amplitude, medium=w["medium"])


def acoustic_fixture(name, w, res, seconds, *, apex, focus, extra=None):
    amp = np.abs(res.phasor)
    s = lattice_stride(amp.shape)
    met = _metrics(res, w, apex, focus)
    peak = tuple(int(v) for v in met["peak"]["voxel_grid"])
    box = focal_box(amp.shape, peak)
    labels, table = _labels_of(w["medium"])
    spec = w["spec"].model_dump()
    out = {
        "shape": np.array(w["grid"].shape), "dx": w["grid"].dx, "pml_thickness": w["grid"].pml.thickness,
        "labels": labels, "table": table,
        "src_idx": w["source"].indices.astype(np.int16), "src_phase": w["source"].phases,
        "amplitude": w["source"].amplitude, "f0": w["source"].f0, "spec": json.dumps(spec),
        "harmonics": np.array(w["harmonics"]), "nonlinear": bool(w["nonlinear"]),
        "reference_point": json.dumps(None if w["reference_point"] is None else list(w["reference_point"])),
        "apex": np.array(apex), "focus": np.array(focus),
        "spp": res.spp, "dt": res.dt, "steps_total": res.steps_total, "tof_periods": res.tof_periods,
        "converged_period": res.converged_period,
        "stride": s, "box": np.array(box), "metrics": json.dumps(met), "fp64_seconds": seconds,
        "p_max_lattice": lattice(np.asarray(res.p_max, np.float32), s),
    }
    for h in w["harmonics"]:
        ph = np.asarray(res.phasors[h])
        out[f"h{h}_lattice"] = lattice(ph, s).astype(np.complex64)
        out[f"h{h}_box"] = _box(ph, box).astype(np.complex64)
        out[f"h{h}_norm2"] = float(np.vdot(ph, ph).real)  # whole-region squared L2 norm, FP64
    if extra:
        out.update(extra)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: spp={res.spp} steps={res.steps_total} peak {met['peak']['p_pa']} Pa at {peak} "
          f"({seconds:.0f} s FP64)", flush=True)


def cfg1(cache: dict):
    from caustica_gb300 import workloads as wl

    w = wl.config1()
    res, sec = run_acoustic(w, "linear")
    cache["cfg1"] = (w, res)
    acoustic_fixture("cfg1_linear_96x96x128", w, res, sec, apex=(48, 48, 10), focus=(48, 48, 110))


def cfg2(cache: dict):
    from caustica_gb300 import workloads as wl

    w = wl.config2()
    res, sec = run_acoustic(w, "westervelt")
    acoustic_fixture("cfg2_westervelt_192x192x256", w, res, sec, apex=(96, 96, 10), focus=w["reference_point"])


def cfg3(cache: dict):
    from caustica.sensors import HeatingSource
    from caustica.thermal import PennesSolver, ThermalMedium

    if "cfg1" not in cache:
        cfg1(cache)
    w, res = cache["cfg1"]
    g = w["grid"]
    hs = HeatingSource.from_phasors({1: res.phasors[1]}, alpha=float(w["medium"].alpha.flat[0]), rho=1000.0,
                                    c=1500.0, dx=g.dx)
    q0 = np.asarray(hs.q, np.float32)
    full = np.ones(g.shape, np.float32)
    tmed = ThermalMedium(k=full * 0.5, rho=full * 1000.0, specific_heat=full * 3600.0,
                         perfusion=full * np.float32(0.5 / 1050.0), dx=g.dx)
    for name, scale in (("cfg3_pennes_96x96x128", 1.0), ("cfg3_pennes_stress_96x96x128", 2000.0)):
        q = q0 * np.float32(scale)
        solver = PennesSolver("numpy64")
        t0 = time.time()
        hot = solver.solve(np.full(g.shape, 37.0, np.float32), q, tmed, dt=0.05, n_steps=400, dose=True)
        cool = solver.solve(hot.temperature, None, tmed, dt=0.05, n_steps=1200, dose=True, dose0=hot.dose_cem43)
        sec = time.time() - t0
        peak = np.unravel_index(int(np.argmax(cool.temperature_max)), g.shape)
        box = focal_box(g.shape, peak)
        s = lattice_stride(g.shape)
        out = {"shape": np.array(g.shape), "dx": g.dx, "q_scale": scale, "dt": 0.05, "n_heat": 400, "n_cool": 1200,
               "k": 0.5, "rho": 1000.0, "cp": 3600.0, "perfusion": np.float32(0.5 / 1050.0),
               "alpha": float(w["medium"].alpha.flat[0]), "stride": s, "box": np.array(box),
               "q_max": float(q.max()), "q_sum": float(q.astype(np.float64).sum()), "fp64_seconds": sec}
        for tag, r in (("heat", hot), ("cool", cool)):
            for key, arr in (("T", r.temperature), ("Tmax", r.temperature_max), ("dose", r.dose_cem43)):
                a = np.asarray(arr, np.float32)
                out[f"{tag}_{key}_lattice"] = lattice(a, s)
                out[f"{tag}_{key}_box"] = _box(a, box)
                out[f"{tag}_{key}_max"] = float(a.max())
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(f"{name}: dT max {float(cool.temperature_max.max()) - 37.0:.4g} K, dose max "
              f"{float(cool.dose_cem43.max()):.4g} min ({sec:.0f} s FP64)", flush=True)


CFG4_MEMBERS = (0, 21, 42, 63)


def cfg4(cache: dict):
    from caustica.sources import CWSource

    from caustica_gb300 import workloads as wl

    w = wl.config4()
    phases = w["phases"]
    apex = (80, 80, 12)
    extra = {"members": np.array(CFG4_MEMBERS), "targets": w["targets"][list(CFG4_MEMBERS)]}
    fields = {}
    total = 0.0
    first = None
    for b in CFG4_MEMBERS:
        src = CWSource(indices=w["source"].indices, phases=phases[b], amplitude=w["source"].amplitude,
                       f0=w["source"].f0)
        res, sec = run_acoustic(w, "linear", source=src)
        total += sec
        if first is None:
            first = res
        amp = np.abs(res.phasor)
        s = lattice_stride(amp.shape)
        met = _metrics(res, w, apex, w["reference_point"])
        peak = tuple(int(v) for v in met["peak"]["voxel_grid"])
        box = focal_box(amp.shape, peak)
        fields[f"m{b}_h1_lattice"] = lattice(np.asarray(res.phasors[1]), s).astype(np.complex64)
        fields[f"m{b}_h1_box"] = _box(np.asarray(res.phasors[1]), box).astype(np.complex64)
        fields[f"m{b}_h1_norm2"] = float(np.vdot(res.phasors[1], res.phasors[1]).real)
        fields[f"m{b}_box"] = np.array(box)
        fields[f"m{b}_metrics"] = json.dumps(met)
        fields[f"m{b}_phases"] = phases[b]
        print(f"cfg4 member {b}: peak {met['peak']['p_pa']} Pa at {peak} ({sec:.0f} s FP64)", flush=True)
    labels, table = _labels_of(w["medium"])
    out = {"shape": np.array(w["grid"].shape), "dx": w["grid"].dx, "pml_thickness": w["grid"].pml.thickness,
           "labels": labels, "table": table, "src_idx": w["source"].indices.astype(np.int16),
           "amplitude": w["source"].amplitude, "f0": w["source"].f0, "spec": json.dumps(w["spec"].model_dump()),
           "reference_point": json.dumps(list(w["reference_point"])), "apex": np.array(apex),
           "spp": first.spp, "dt": first.dt, "steps_total": first.steps_total, "tof_periods": first.tof_periods,
           "stride": lattice_stride(w["grid"].shape), "fp64_seconds": total, **extra, **fields}
    np.savez_compressed(HERE / "cfg4_steer_160x160x192.npz", **out)


def main(src_path: str, which) -> None:
    sys.path.insert(0, src_path)
    sys.path.insert(0, str(ROOT))
    import caustica
    import caustica.core.backend as cb

    from make_golden import _install_numpy64

    _install_numpy64(cb)
    if hasattr(caustica, "set_cpu_fft_workers"):
        caustica.set_cpu_fft_workers(os.cpu_count())
    cache: dict = {}
    for name in which:
        {"cfg1": cfg1, "cfg2": cfg2, "cfg3": cfg3, "cfg4": cfg4}[name](cache)


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CAUSTICA_REFERENCE_SRC")
    if not src:
        sys.exit("usage: make_config_golden.py /path/to/caustica/src [cfg1 cfg2 cfg3 cfg4]")
    sys.path.insert(0, str(HERE))
    main(src, sys.argv[2:] or ["cfg1", "cfg2", "cfg3", "cfg4"])

"""Generate the golden fixtures that pin the oracle to the reference.

Runs the UNCHANGED reference (ebx0/caustica, pure Python) from a source
checkout on small cases and writes inputs and outputs to ``*.npz`` files
beside this script. FP64 runs use a backend plugin ``numpy64`` whose array
module reads ``float32``/``complex64`` as ``float64``/``complex128`` and is
otherwise NumPy, registered through the reference's own backend registry
(core/backend.py:44); the engine and the Pennes solver run unmodified.

Usage (needs the reference checkout; the fixtures are committed, so the
tests themselves never need it)::

    python tests/golden/make_golden.py /path/to/caustica/src
"""

from __future__ import annotations

import json
import sys
import types
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _install_numpy64(caustica_backend):
    class _NumPy64(types.ModuleType):
        def __getattr__(self, name):
            if name == "float32":
                return np.float64
            if name == "complex64":
                return np.complex128
            return getattr(np, name)

    proxy = _NumPy64("numpy64")
    Backend = caustica_backend.Backend

    def _factory():
        return Backend("numpy64", proxy)

    _factory.__module__ = __name__
    _factory.__qualname__ = "numpy64_factory"
    if "numpy64" not in caustica_backend.backends.available():
        caustica_backend.backends.register("numpy64")(_factory)


def _medium_random(shape, seed, *, beta=0.0):
    rng = np.random.default_rng(seed)
    c = rng.uniform(1450.0, 1650.0, shape).astype(np.float32)
    rho = rng.uniform(900.0, 1100.0, shape).astype(np.float32)
    alpha = rng.uniform(0.0, 30.0, shape).astype(np.float32)
    b = np.full(shape, beta, np.float32) if beta else np.zeros(shape, np.float32)
    return alpha, rho, c, b


def _random_source(shape, n, seed, margin):
    rng = np.random.default_rng(seed)
    pts = set()
    while len(pts) < n:
        pts.add(tuple(int(rng.integers(margin, s - margin)) for s in shape))
    idx = np.array(sorted(pts), np.int64)
    ph = rng.uniform(-np.pi, np.pi, len(idx)).astype(np.float32)
    return idx, ph


def kspace_case(name, *, shape, dx, pml_vox, seed, n_src, solver, amplitude, f0, spec_kw,
                harmonics=(1,), record_region=None, reference_point=None, beta=0.0,
                backend="numpy64", homogeneous=False):
    from caustica import Grid, Medium, PMLSpec
    from caustica.solvers import CWRunSpec
    import caustica.solvers as solvers
    from caustica.sources import CWSource

    grid = Grid(shape, dx, PMLSpec(pml_vox * dx))
    if homogeneous:
        alpha = np.full(shape, 0.5, np.float32)
        rho = np.full(shape, 1000.0, np.float32)
        c = np.full(shape, 1500.0, np.float32)
        b = np.full(shape, beta, np.float32)
    else:
        alpha, rho, c, b = _medium_random(shape, seed, beta=beta)
    med = Medium(alpha=alpha, rho=rho, c=c, beta=b)
    idx, ph = _random_source(shape, n_src, seed + 1, pml_vox)
    src = CWSource(indices=idx, phases=ph, amplitude=amplitude, f0=f0)
    spec = CWRunSpec(**spec_kw)
    res = solvers.get(solver)().run(
        grid, med, src, spec, backend=backend, harmonics=harmonics,
        record_region=record_region, reference_point=reference_point,
    )
    out = {
        "shape": np.array(shape), "dx": dx, "pml_vox": grid.pml_vox, "pml_edge": 2.0,
        "alpha": alpha, "rho": rho, "c": c, "beta": b,
        "src_idx": idx, "src_phase": ph, "amplitude": amplitude, "f0": f0, "ramp_periods": 3.0,
        "nonlinear": solver == "westervelt", "harmonics": np.array(harmonics),
        "spec": json.dumps(spec_kw),
        "record_region": json.dumps(None if record_region is None else [[s.start, s.stop] for s in record_region]),
        "reference_point": json.dumps(None if reference_point is None else list(reference_point)),
        "spp": res.spp, "dt": res.dt, "steps_total": res.steps_total, "tof_periods": res.tof_periods,
        "converged_period": res.converged_period, "settle_capped": res.settle_capped,
        "history": np.array(res.convergence_history, np.float64).reshape(-1, 3),
        "p_max": res.p_max,
        "region": np.array([[s.start, s.stop] for s in res.region]),
    }
    for h in harmonics:
        out[f"phasor_h{h}"] = res.phasors[h]
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: spp={res.spp} steps={res.steps_total} |P|max={np.abs(res.phasor).max():.4g}")


def pennes_case(name, *, shape, dx, seed, dt, n_steps, boundary="insulated", on_unstable="refuse",
                q_scale=2e6, perfused=True, chain_steps=0, reference_temperature_c=None):
    from caustica.thermal import PennesSolver, ThermalMedium

    rng = np.random.default_rng(seed)
    k = rng.uniform(0.3, 0.6, shape).astype(np.float32)
    rho = rng.uniform(950.0, 1100.0, shape).astype(np.float32)
    cp = rng.uniform(3000.0, 4000.0, shape).astype(np.float32)
    w = (rng.uniform(0.0, 0.02, shape) if perfused else np.zeros(shape)).astype(np.float32)
    tmed = ThermalMedium(k=k, rho=rho, specific_heat=cp, perfusion=w, dx=dx)
    q = (rng.random(shape) ** 4 * q_scale).astype(np.float32)
    t0 = (37.0 + rng.uniform(0.0, 2.0, shape)).astype(np.float32)
    solver = PennesSolver("numpy64", boundary=boundary, on_unstable=on_unstable,
                          reference_temperature_c=reference_temperature_c)
    hot = solver.solve(t0, q, tmed, dt=dt, n_steps=n_steps, dose=True, record_every=max(1, n_steps // 3))
    out = {
        "shape": np.array(shape), "dx": dx, "dt": dt, "n_steps": n_steps, "k": k, "rho": rho, "cp": cp,
        "w": w, "q": q, "t0": t0, "boundary": boundary, "on_unstable": on_unstable,
        "reference_temperature_c": json.dumps(reference_temperature_c),
        "T": hot.temperature, "Tmax": hot.temperature_max, "dose": hot.dose_cem43,
        "substeps": hot.substeps, "dt_stable": hot.meta["dt_stable_s"],
        "samples": np.array(hot.samples), "times": np.array(hot.times),
    }
    if chain_steps:
        cool = solver.solve(hot.temperature, None, tmed, dt=dt, n_steps=chain_steps, dose=True,
                            dose0=hot.dose_cem43)
        out.update({"chain_steps": chain_steps, "T2": cool.temperature, "Tmax2": cool.temperature_max,
                    "dose2": cool.dose_cem43})
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: substeps={hot.substeps} Tmax={hot.peak_temperature_c:.4f} dose={hot.peak_dose_cem43:.4g}")


def bowl_source_case():
    """The 500 kHz bowl of the 96x96x128 workload, as the reference voxelises it."""
    from caustica import Grid, PMLSpec
    from caustica.sources import bowl_cw_source

    grid = Grid((96, 96, 128), 0.3e-3, PMLSpec(3.0e-3))
    src = bowl_cw_source(grid, f0=5e5, amplitude=1e5, aperture_radius=12e-3, roc=30e-3, apex_vox=(48, 48, 10))
    np.savez_compressed(HERE / "bowl_96x96x128.npz", indices=src.indices.astype(np.int16))
    print(f"bowl: {src.n_points} voxels")


def _focal_field(shape, centre, widths, peak, seed, noise):
    rng = np.random.default_rng(seed)
    ax = np.meshgrid(*[np.arange(n, dtype=np.float64) for n in shape], indexing="ij")
    r2 = sum(((a - c0) / w) ** 2 for a, c0, w in zip(ax, centre, widths))
    ph = rng.uniform(-np.pi, np.pi)
    f = peak * np.exp(-0.5 * r2) * np.exp(1j * (ph + 0.3 * ax[2]))
    f = f + noise * (rng.standard_normal(shape) + 1j * rng.standard_normal(shape))
    return f.astype(np.complex64)


def focus_case(name, *, grid_shape, pml_vox, region, centre, widths, apex, focus, harmonic2, dx, seed,
               spike=None, a2_edge=None, medium=True):
    """``report.metrics.focus_metrics`` on a synthetic focal field (metrics.py:192-313)."""
    from caustica.report.metrics import FieldFrame, focus_metrics
    from caustica.solvers.base import SolverResult

    shape = tuple(len(range(*sl.indices(n))) for sl, n in zip(region, grid_shape))
    org = tuple(sl.indices(n)[0] for sl, n in zip(region, grid_shape))
    ctr = tuple(c0 - o for c0, o in zip(centre, org))
    p1 = _focal_field(shape, ctr, widths, 1.2e6, seed, 2e3)
    if spike is not None:  # a larger value inside the PML margin: must not win the argmax
        p1[spike] = np.complex64(4e6)
    phasors = {1: p1}
    if harmonic2:
        p2 = (0.08 * np.abs(p1).astype(np.float64) ** 2 / 1.2e6).astype(np.complex64) * np.complex64(1j)
        if a2_edge is not None:  # a residue against the absorber
            p2[a2_edge] = np.complex64(2.5e5)
        phasors[2] = p2
    rng = np.random.default_rng(seed + 1)
    pmax = (np.abs(p1) * rng.uniform(1.0, 1.2, shape)).astype(np.float32)
    res = SolverResult(phasor=p1, p_max=pmax, region=tuple(slice(o, o + n) for o, n in zip(org, shape)),
                       dt=2.5e-8, spp=40, steps_total=1200, t_end_s=3.0e-5, tof_periods=12,
                       converged_period=26, settle_capped=False, convergence_history=[],
                       phasors=phasors, meta={"solver": "westervelt"})
    frame = FieldFrame(dx=dx, grid_shape=grid_shape, pml_vox=pml_vox, apex_vox=apex, focus_vox=focus)
    med = None
    if medium:
        mrng = np.random.default_rng(seed + 2)
        lab = mrng.integers(0, 3, grid_shape)
        med = types.SimpleNamespace(rho=np.array([1000.0, 1050.0, 1090.0], np.float32)[lab],
                                    c=np.array([1500.0, 1560.0, 1610.0], np.float32)[lab])
    m = focus_metrics(res, frame, source_amplitude=1e5, medium=med)
    out = {"p1": p1, "pmax": pmax, "origin": np.array(org), "grid_shape": np.array(grid_shape),
           "pml_vox": np.int64(pml_vox), "apex": np.array(apex), "dx": np.float64(dx),
           "focus": np.array(focus if focus is not None else (-1, -1, -1)),
           "metrics": np.array(json.dumps(m))}
    if harmonic2:
        out["p2"] = phasors[2]
    if med is not None:
        out["rho"], out["c"] = med.rho, med.c
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: peak {m['peak']['p_pa']} at {m['peak']['voxel_grid']}, warnings {len(m['warnings'])}")


def heating_case(name, *, shape, seed, harmonics, y):
    """``HeatingSource.from_phasors`` on label-valued maps (sensors.py:193-295)."""
    from caustica.sensors import HeatingSource

    rng = np.random.default_rng(seed)
    labels = rng.integers(0, 4, shape).astype(np.uint8)
    table = np.array([[0.0, 1000.0, 1500.0], [4.3, 1050.0, 1560.0], [12.5, 1090.0, 1610.0],
                      [55.0, 1900.0, 2800.0]], np.float32)  # alpha_f0 [Np/m], rho, c
    alpha, rho, c = (table[labels, i] for i in range(3))
    phasors = {n: (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(np.complex64)
               * np.complex64(1e6 / n) for n in harmonics}
    hs = HeatingSource.from_phasors(phasors, alpha=alpha, rho=rho, c=c, dx=0.3e-3,
                                    harmonics=harmonics, alpha_power_law_y=y)
    out = {"labels": labels, "table": table, "harmonics": np.array(harmonics), "y": np.float64(y),
           "q": hs.q}
    for n, p in phasors.items():
        out[f"p{n}"] = p
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(f"{name}: q max {float(hs.q.max()):.4g}")


def main(src_path: str) -> None:
    sys.path.insert(0, src_path)
    import caustica.core.backend as cb

    _install_numpy64(cb)
    common = dict(f0=1.0e6)
    kspace_case("ks3d_linear_hetero", shape=(12, 10, 16), dx=0.3e-3, pml_vox=2, seed=11, n_src=14,
                solver="linear", amplitude=1e5,
                spec_kw=dict(convergence_tol=0.0, min_settle_periods=2, max_settle_periods=4,
                             n_record_periods=2), **common)
    kspace_case("ks3d_westervelt_padded", shape=(7, 11, 13), dx=0.3e-3, pml_vox=1, seed=21, n_src=9,
                solver="westervelt", amplitude=2e6, beta=4.5, harmonics=(1, 2, 3),
                record_region=(slice(1, 6), slice(2, None), slice(-9, -1)), reference_point=(3, 5, 10),
                spec_kw=dict(cfl=0.3, convergence_tol=0.0, min_settle_periods=3, max_settle_periods=3,
                             n_record_periods=1), **common)
    kspace_case("ks1d_plane_converge", shape=(96,), dx=0.375e-3, pml_vox=12, seed=31, n_src=1,
                solver="linear", amplitude=1e5, homogeneous=True,
                spec_kw=dict(min_settle_periods=6, max_settle_periods=60, convergence_tol=0.01,
                             n_record_periods=2), **common)
    kspace_case("ks2d_westervelt", shape=(20, 24), dx=0.2e-3, pml_vox=3, seed=41, n_src=10,
                solver="westervelt", amplitude=1.5e6, beta=3.5, harmonics=(1, 2),
                spec_kw=dict(cfl=0.4, convergence_tol=0.0, min_settle_periods=2, max_settle_periods=3,
                             n_record_periods=2, t_end_min_us=9.0), **common)
    kspace_case("ks3d_fp32_reference", shape=(10, 9, 12), dx=0.3e-3, pml_vox=2, seed=51, n_src=8,
                solver="linear", amplitude=1e5, backend="numpy",
                spec_kw=dict(convergence_tol=0.0, min_settle_periods=2, max_settle_periods=2,
                             n_record_periods=1), **common)
    pennes_case("pennes3d_insulated", shape=(8, 9, 10), dx=0.3e-3, seed=61, dt=0.01, n_steps=40,
                chain_steps=30)
    pennes_case("pennes2d_dirichlet_substep", shape=(12, 10), dx=0.25e-3, seed=71, dt=0.2, n_steps=12,
                boundary="dirichlet", on_unstable="substep", reference_temperature_c=36.0)
    bowl_source_case()
    focus_case("focus_h2_target", grid_shape=(40, 36, 48), pml_vox=4,
               region=(slice(2, 38), slice(1, 35), slice(3, 46)), centre=(21, 17, 28), widths=(2.5, 3.0, 7.0),
               apex=(20, 18, 5), focus=(22, 17, 27), harmonic2=True, dx=0.25e-3, seed=81,
               spike=(1, 10, 20), a2_edge=(31, 12, 30))
    focus_case("focus_truncated", grid_shape=(32, 30, 40), pml_vox=3,
               region=(slice(0, 32), slice(0, 30), slice(0, 40)), centre=(15, 14, 20), widths=(2.0, 40.0, 5.0),
               apex=(16, 15, 0), focus=None, harmonic2=False, dx=0.3e-3, seed=91, medium=False)
    heating_case("heating_q_h12", shape=(14, 12, 18), seed=101, harmonics=(1, 2), y=1.1)


if __name__ == "__main__":
    import os

    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CAUSTICA_REFERENCE_SRC")
    if not src:
        sys.exit("usage: make_golden.py /path/to/caustica/src  (or set CAUSTICA_REFERENCE_SRC)")
    main(src)

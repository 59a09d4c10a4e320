"""The benchmark workloads at their own sizes against the reference in FP64 (GPU).

Fixtures (``tests/golden/cfg*.npz``, made by ``make_config_golden.py``) hold
the unchanged reference's FP64 results of each workload: the whole-region
fields sampled on a regular lattice (every s-th voxel per axis), the fields
on a full-resolution box around the focus, and its ``focus_metrics``
dictionary. Each test solves the same inputs through the public GB300 front
and checks the stated tolerances:

* complex phasor relative L2 <= 1e-4 per harmonic (lattice and focal box);
* focal peak pressure within 0.1 %, at the same voxel;
* -6 dB extents (axial and both lateral edges) within one voxel;
* temperature max-abs <= 1e-3 K and CEM43 relative error <= 1e-3.

The FP32-vs-FP64 error measured on each result is printed (``-s``) so the
error of every benchmark result against the FP64 oracle is on record.
"""

from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, load_golden, rel_l2
import caustica_gb300 as cg

pytestmark = pytest.mark.gpu

PHASOR_TOL = 1e-4
PEAK_TOL = 1e-3
T_TOL_K = 1e-3
DOSE_TOL = 1e-3


def _have(name):
    return (GOLDEN / f"{name}.npz").exists()


def _lattice(a, s):
    return a[tuple(slice(s // 2, None, s) for _ in range(a.ndim))]


def _box(a, box):
    return a[tuple(slice(int(lo), int(hi)) for lo, hi in box)]


def _json(v):
    return json.loads(v) if isinstance(v, str) else v


def _inputs(g, phases=None):
    shape = tuple(int(v) for v in g["shape"])
    dx = float(g["dx"])
    grid = cg.Grid(shape, dx, cg.PMLSpec(float(g["pml_thickness"])))
    table = {i: tuple(float(v) for v in row) for i, row in enumerate(g["table"])}
    med = cg.Medium.from_labels(g["labels"].astype(np.int32), table)
    ph = g["src_phase"] if phases is None else phases
    src = cg.CWSource(indices=g["src_idx"].astype(np.int64), phases=ph, amplitude=float(g["amplitude"]),
                      f0=float(g["f0"]))
    spec = cg.CWRunSpec(**_json(g["spec"]))
    rp = _json(g["reference_point"])
    return grid, med, src, spec, None if rp is None else tuple(rp)


def _check_extent(mine: dict, ref: dict, dx_mm: float, what: str):
    assert mine["truncated"] == ref["truncated"], what
    if ref["truncated"]:
        return
    for k in ("left_mm", "right_mm"):
        assert abs(mine[k] - ref[k]) <= dx_mm, f"{what} {k}: {mine[k]} vs {ref[k]} mm (one voxel = {dx_mm} mm)"


def _check_metrics(res, g, med, frame_apex, frame_focus, label):
    ref = _json(g["metrics"])
    shape = tuple(int(v) for v in g["shape"])
    frame = cg.FieldFrame(dx=float(g["dx"]), grid_shape=shape, pml_vox=int(round(float(g["pml_thickness"]) /
                                                                                  float(g["dx"]))),
                          apex_vox=tuple(int(v) for v in frame_apex),
                          focus_vox=None if frame_focus is None else tuple(int(v) for v in frame_focus))
    mine = cg.focus_metrics(res, frame, source_amplitude=float(g["amplitude"]), medium=med)
    assert mine["peak"]["voxel_grid"] == ref["peak"]["voxel_grid"], label
    rel = abs(mine["peak"]["p_pa"] - ref["peak"]["p_pa"]) / ref["peak"]["p_pa"]
    assert rel < PEAK_TOL, f"{label}: peak {mine['peak']['p_pa']} vs {ref['peak']['p_pa']} Pa"
    dx_mm = float(g["dx"]) * 1e3
    for key in ("axial_6db", "lateral_x_6db", "lateral_y_6db"):
        _check_extent(mine["focal_spot"][key], ref["focal_spot"][key], dx_mm, f"{label} {key}")
    print(f"{label}: peak {mine['peak']['p_pa']:.1f} Pa (FP64 {ref['peak']['p_pa']:.1f}, rel {rel:.2e}); "
          f"-6 dB widths {[mine['focal_spot'][k]['width_mm'] for k in ('axial_6db', 'lateral_x_6db')]} vs "
          f"{[ref['focal_spot'][k]['width_mm'] for k in ('axial_6db', 'lateral_x_6db')]} mm")
    return mine, ref


def _check_fields(res, g, label, prefix=""):
    s = int(g["stride"])
    errs = {}
    for h in np.atleast_1d(g["harmonics"]) if "harmonics" in g else (1,):
        h = int(h)
        lat = rel_l2(_lattice(res.phasors[h], s), g[f"{prefix}h{h}_lattice"])
        box = rel_l2(_box(res.phasors[h], g[f"{prefix}box" if prefix else "box"]), g[f"{prefix}h{h}_box"])
        errs[h] = (lat, box)
        assert lat < PHASOR_TOL, f"{label} harmonic {h}: lattice rel L2 {lat:.3e}"
        assert box < PHASOR_TOL, f"{label} harmonic {h}: focal-box rel L2 {box:.3e}"
    print(f"{label}: phasor rel L2 vs FP64 (lattice, focal box) " +
          ", ".join(f"h{h} {a:.2e} {b:.2e}" for h, (a, b) in errs.items()))
    return errs


def _acoustic(name):
    g = load_golden(name)
    grid, med, src, spec, rp = _inputs(g)
    solver = cg.WesterveltKSpaceGB300() if bool(g["nonlinear"]) else cg.LinearKSpaceGB300()
    harm = tuple(int(h) for h in np.atleast_1d(g["harmonics"]))
    res = solver.run(grid, med, src, spec, harmonics=harm, reference_point=rp)
    assert res.spp == g["spp"] and res.steps_total == g["steps_total"] and res.tof_periods == g["tof_periods"]
    assert res.converged_period == g["converged_period"]
    return g, med, res


@pytest.mark.skipif(not _have("cfg1_linear_96x96x128"), reason="fixture not generated")
def test_cfg1_linear_bowl_96x96x128_against_fp64():
    g, med, res = _acoustic("cfg1_linear_96x96x128")
    _check_fields(res, g, "cfg1")
    pm = _lattice(res.p_max, int(g["stride"]))
    assert np.abs(pm - g["p_max_lattice"]).max() / np.abs(g["p_max_lattice"]).max() < PHASOR_TOL
    mine, ref = _check_metrics(res, g, med, g["apex"], g["focus"], "cfg1")
    assert mine["peak"]["voxel_grid"] == [48, 48, 90]


@pytest.mark.skipif(not _have("cfg2_westervelt_192x192x256"), reason="fixture not generated")
def test_cfg2_westervelt_layered_192x192x256_against_fp64():
    g, med, res = _acoustic("cfg2_westervelt_192x192x256")
    _check_fields(res, g, "cfg2")
    pm = _lattice(res.p_max, int(g["stride"]))
    assert np.abs(pm - g["p_max_lattice"]).max() / np.abs(g["p_max_lattice"]).max() < PHASOR_TOL
    _check_metrics(res, g, med, g["apex"], g["focus"], "cfg2")


def _thermal_chain(g1, res1, med1, scale):
    """The served chain: device Q from the acoustic result, 400 heating +
    1,200 chained cooling steps with CEM43 dose."""
    shape = tuple(int(v) for v in g1["shape"])
    dx = float(g1["dx"])
    hs = cg.HeatingSource.from_result(res1, med1, dx)
    q = hs.embed(shape) * np.float32(scale)
    tm = cg.ThermalMedium.homogeneous(shape, k=0.5, rho=1000.0, specific_heat=3600.0,
                                      perfusion=float(np.float32(0.5 / 1050.0)), dx=dx)
    solver = cg.PennesSolverGB300()
    hot = solver.solve(np.full(shape, 37.0, np.float32), q, tm, dt=0.05, n_steps=400, dose=True)
    cool = solver.solve(hot.temperature, None, tm, dt=0.05, n_steps=1200, dose=True, dose0=hot.dose_cem43)
    return q, hot, cool


@pytest.mark.skipif(not (_have("cfg3_pennes_96x96x128") and _have("cfg1_linear_96x96x128")),
                    reason="fixture not generated")
@pytest.mark.parametrize("name", ["cfg3_pennes_96x96x128", "cfg3_pennes_stress_96x96x128"])
def test_cfg3_pennes_cem43_chain_against_fp64(name):
    if not _have(name):
        pytest.skip("fixture not generated")
    g1, med1, res1 = _acoustic("cfg1_linear_96x96x128")
    g = load_golden(name)
    q, hot, cool = _thermal_chain(g1, res1, med1, float(g["q_scale"]))
    assert abs(float(q.max()) - float(g["q_max"])) / float(g["q_max"]) < 1e-4
    s = int(g["stride"])
    worst_t = 0.0
    worst_d = 0.0
    for tag, r in (("heat", hot), ("cool", cool)):
        for key, arr in (("T", r.temperature), ("Tmax", r.temperature_max)):
            for part, sel in (("lattice", _lattice(arr, s)), ("box", _box(arr, g["box"]))):
                err = float(np.abs(sel - g[f"{tag}_{key}_{part}"]).max())
                worst_t = max(worst_t, err)
                assert err <= T_TOL_K, f"{name} {tag} {key} {part}: max-abs {err:.3e} K"
        dmax = float(g[f"{tag}_dose_max"])
        for part, sel in (("lattice", _lattice(r.dose_cem43, s)), ("box", _box(r.dose_cem43, g["box"]))):
            ref = g[f"{tag}_dose_{part}"].astype(np.float64)
            # relative error where the dose is significant (>= 1e-3 of its maximum), and
            # no voxel off by more than 1e-3 of the maximum anywhere
            sig = ref >= 1e-3 * dmax
            rel = np.abs(sel[sig] - ref[sig]) / ref[sig]
            worst = float(rel.max()) if rel.size else 0.0
            worst_d = max(worst_d, worst)
            assert worst <= DOSE_TOL, f"{name} {tag} dose {part}: rel {worst:.3e}"
            assert float(np.abs(sel - ref).max()) <= DOSE_TOL * dmax
        assert abs(float(r.dose_cem43.max()) - dmax) <= DOSE_TOL * dmax
    print(f"{name}: T max-abs {worst_t:.2e} K, CEM43 rel {worst_d:.2e} "
          f"(dT max {float(cool.temperature_max.max()) - 37.0:.4g} K, dose max {float(cool.dose_cem43.max()):.4g} min)")


@pytest.mark.skipif(not _have("cfg4_steer_160x160x192"), reason="fixture not generated")
def test_cfg4_steering_members_in_one_batched_launch_against_fp64():
    """All 64 steers in one batched solve; four of them against FP64 solo runs."""
    from caustica_gb300 import workloads
    from caustica_gb300.batch import solve_steering

    g = load_golden("cfg4_steer_160x160x192")
    members = [int(m) for m in g["members"]]
    w = workloads.config4()
    phases = w["phases"]
    for b in members:
        np.testing.assert_array_equal(phases[b], g[f"m{b}_phases"])  # same drive as the FP64 runs
    grid, med, src, spec, rp = _inputs(g, phases=phases[0])
    res = solve_steering(grid, med, src.indices, phases, f0=float(g["f0"]), amplitude=float(g["amplitude"]),
                         spec=spec, reference_point=rp)
    assert len(res) == phases.shape[0]
    for b in members:
        r = res[b]
        assert r.steps_total == g["steps_total"] and r.spp == g["spp"]
        s = int(g["stride"])
        lat = rel_l2(_lattice(r.phasors[1], s), g[f"m{b}_h1_lattice"])
        box = rel_l2(_box(r.phasors[1], g[f"m{b}_box"]), g[f"m{b}_h1_box"])
        print(f"cfg4 member {b}: phasor rel L2 vs FP64 lattice {lat:.2e}, focal box {box:.2e}")
        assert lat < PHASOR_TOL and box < PHASOR_TOL, (b, lat, box)
        ref = _json(g[f"m{b}_metrics"])
        frame = cg.FieldFrame(dx=float(g["dx"]), grid_shape=tuple(int(v) for v in g["shape"]), pml_vox=10,
                              apex_vox=tuple(int(v) for v in g["apex"]), focus_vox=rp)
        mine = cg.focus_metrics(r, frame, source_amplitude=float(g["amplitude"]), medium=med)
        assert mine["peak"]["voxel_grid"] == ref["peak"]["voxel_grid"], b
        assert abs(mine["peak"]["p_pa"] - ref["peak"]["p_pa"]) / ref["peak"]["p_pa"] < PEAK_TOL, b

"""Whole CW solves through the solver front against the reference's FP64 goldens (GPU)."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import KSPACE_GOLDEN, golden_kspace_kwargs, load_golden, rel_l2
import caustica_gb300 as cg
from oracle import kspace as ok

pytestmark = pytest.mark.gpu

PHASOR_TOL = 1e-4  # complex phasor relative L2 per harmonic


def _run(g, **over):
    kw = golden_kspace_kwargs(g)
    grid = cg.Grid(kw["shape"], kw["dx"], cg.PMLSpec(kw["pml_vox_n"] * kw["dx"]))
    med = cg.Medium(kw["alpha"], kw["rho"], kw["c"], kw["beta"])
    src = cg.CWSource(indices=kw["src_idx"], phases=kw["src_phase"], amplitude=kw["amplitude"], f0=kw["f0"])
    spec = cg.CWRunSpec(cfl=kw["cfl"], cfl_hard_max=kw["cfl_hard_max"], min_settle_periods=kw["min_settle_periods"],
                        max_settle_periods=kw["max_settle_periods"], convergence_tol=kw["convergence_tol"],
                        n_record_periods=kw["n_record_periods"], t_end_min_us=kw["t_end_min_us"])
    solver = cg.WesterveltKSpaceGB300() if kw["nonlinear"] else cg.LinearKSpaceGB300()
    return solver.run(grid, med, src, spec, record_region=kw["record_region"], reference_point=kw["reference_point"],
                      harmonics=kw["harmonics"], **over)


@pytest.mark.parametrize("name", KSPACE_GOLDEN)
def test_solve_matches_reference_fp64(name):
    g = load_golden(name)
    res = _run(g)
    assert res.spp == g["spp"]
    assert res.steps_total == g["steps_total"]
    assert res.tof_periods == g["tof_periods"]
    assert res.converged_period == g["converged_period"]
    assert res.settle_capped == bool(g["settle_capped"])
    assert [[s.start, s.stop] for s in res.region] == g["region"].tolist()
    for h in np.atleast_1d(g["harmonics"]):
        err = rel_l2(res.phasors[int(h)], g[f"phasor_h{int(h)}"])
        assert err < PHASOR_TOL, f"harmonic {h}: rel L2 {err:.3e}"
    pm = g["p_max"]
    assert np.abs(res.p_max - pm).max() / np.abs(pm).max() < 1e-4
    hist = np.array(res.convergence_history, np.float64).reshape(-1, 3)
    np.testing.assert_allclose(hist[:, 1], g["history"][:, 1], rtol=1e-4)


def test_westervelt_with_zero_beta_equals_linear_exactly():
    g = load_golden("ks3d_linear_hetero")
    kw = golden_kspace_kwargs(g)
    grid = cg.Grid(kw["shape"], kw["dx"], cg.PMLSpec(kw["pml_vox_n"] * kw["dx"]))
    med = cg.Medium(kw["alpha"], kw["rho"], kw["c"], np.zeros_like(kw["beta"]))
    src = cg.CWSource(indices=kw["src_idx"], phases=kw["src_phase"], amplitude=kw["amplitude"], f0=kw["f0"])
    spec = cg.CWRunSpec(convergence_tol=0.0, min_settle_periods=2, max_settle_periods=3, n_record_periods=1)
    a = cg.LinearKSpaceGB300().run(grid, med, src, spec)
    b = cg.WesterveltKSpaceGB300().run(grid, med, src, spec)
    np.testing.assert_array_equal(a.phasor, b.phasor)
    np.testing.assert_array_equal(a.p_max, b.p_max)
    assert b.meta["nonlinear_active"] is False


def test_progress_is_called_once_per_period_and_a_raising_callback_only_warns():
    g = load_golden("ks3d_linear_hetero")
    seen = []
    snaps = []

    def cb(payload):
        seen.append(payload)
        if len(seen) == 1:
            snaps.append(payload["snapshot"]())  # lazy: one device->host copy, only when asked
        raise RuntimeError("widget broke")

    with pytest.warns(UserWarning, match="progress callback raised"):
        res = _run(g, progress=cb)
    settle = [p for p in seen if p["stage"] == "settle"]
    assert len(settle) == res.steps_total // res.spp - 2
    assert seen[-1]["stage"] == "record"
    assert snaps[0].shape == (12, 16)


def test_bowl_focus_against_the_oracle_midsize():
    """A focused bowl on 32x32x48 through the default solver path vs the FP64 oracle."""
    shape = (32, 32, 48)
    dx = 0.3e-3
    grid = cg.Grid(shape, dx, cg.PMLSpec(4 * dx))
    med = cg.Medium.homogeneous(shape, alpha_np_m=0.5, c=1500.0, rho=1000.0)
    pts = []
    for i in range(-6, 7):
        for j in range(-6, 7):
            r2 = (i * dx) ** 2 + (j * dx) ** 2
            if r2 <= (6 * dx) ** 2:
                z = 10e-3 - np.sqrt(10e-3 ** 2 - r2)
                pts.append((16 + i, 16 + j, 6 + int(round(z / dx))))
    idx = np.unique(np.array(pts, np.int64), axis=0)
    src = cg.CWSource(indices=idx, phases=np.zeros(len(idx), np.float32), amplitude=1e5, f0=1e6)
    spec = cg.CWRunSpec(convergence_tol=0.0, min_settle_periods=4, max_settle_periods=4, n_record_periods=2)
    res = cg.LinearKSpaceGB300().run(grid, med, src, spec)
    ref = ok.run_cw(shape=shape, dx=dx, pml_vox_n=4, alpha=med.alpha, rho=med.rho, c=med.c, beta=med.beta,
                    src_idx=idx, src_phase=np.zeros(len(idx), np.float32), amplitude=1e5, f0=1e6,
                    convergence_tol=0.0, min_settle_periods=4, max_settle_periods=4, n_record_periods=2)
    assert rel_l2(res.phasor, ref["phasor"]) < PHASOR_TOL
    a, b = np.abs(res.phasor), np.abs(ref["phasor"])
    assert np.unravel_index(a.argmax(), a.shape) == np.unravel_index(b.argmax(), b.shape)
    assert abs(a.max() - b.max()) / b.max() < 1e-3
    # focal metrics (device) against the same metrics of the FP64 field: peak within 0.1 %,
    # -6 dB extents within one voxel
    from oracle import metrics as om

    frame = cg.FieldFrame(dx=dx, grid_shape=shape, pml_vox=4, apex_vox=(16, 16, 6))
    m = cg.focus_metrics(res, frame)
    m_ref = om.focus_metrics(ref["phasor"], origin=(0, 0, 0), grid_shape=shape, pml_vox=4, apex=(16, 16, 6),
                             dx=dx, p_max=ref["p_max"], amp=np.abs(ref["phasor"]).astype(np.float32))
    assert m["peak"]["voxel_grid"] == m_ref["peak"]["voxel_grid"]
    assert abs(m["peak"]["p_pa"] - m_ref["peak"]["p_pa"]) / m_ref["peak"]["p_pa"] < 1e-3
    for k in ("axial_6db", "lateral_x_6db", "lateral_y_6db"):
        assert m["focal_spot"][k]["truncated"] == m_ref["focal_spot"][k]["truncated"]
        if not m_ref["focal_spot"][k]["truncated"]:
            assert abs(m["focal_spot"][k]["width_mm"] - m_ref["focal_spot"][k]["width_mm"]) <= dx * 1e3

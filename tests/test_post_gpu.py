"""Device focal metrics and heating Q (GPU): against the reference's own
output on the committed fixtures, against the oracle on the same phasors,
and the acoustic -> thermal hand-over without a host copy of the field."""

from __future__ import annotations

import json

import numpy as np
import pytest

import caustica_gb300 as cg
from caustica_gb300 import _lib
from caustica_gb300.engine import DeviceSolver, make_plan, solve
from conftest import FOCUS_GOLDEN, focus_case, load_golden
from oracle import metrics as om
from oracle import sensors as osen

pytestmark = pytest.mark.gpu


def _oracle(res, frame_kw, med, run=None, source_amplitude=1e5):
    p1, p2 = res.phasors[1], res.phasors.get(2)
    m = om.focus_metrics(
        p1, origin=tuple(s.start for s in res.region), grid_shape=frame_kw["grid_shape"],
        pml_vox=frame_kw["pml_vox"], apex=frame_kw["apex_vox"], dx=frame_kw["dx"], focus=frame_kw["focus_vox"],
        p2=p2, p_max=res.p_max, rho=None if med is None else med.rho, c=None if med is None else med.c,
        source_amplitude=source_amplitude, run=run, amp=om.exact_amp(p1), amp2=None if p2 is None else om.exact_amp(p2))
    return json.loads(json.dumps(m))


@pytest.mark.parametrize("name", FOCUS_GOLDEN)
def test_device_metrics_on_the_reference_fixtures(name):
    res, frame_kw, med, golden = focus_case(name)
    m = json.loads(json.dumps(cg.focus_metrics(res, cg.FieldFrame(**frame_kw), source_amplitude=1e5, medium=med)))
    assert m == _oracle(res, frame_kw, med, run=golden["run"])
    # the reference's numbers (NumPy complex abs) agree to their rounding
    assert m["peak"]["voxel_grid"] == golden["peak"]["voxel_grid"]
    assert m["peak"]["p_pa"] == pytest.approx(golden["peak"]["p_pa"], abs=0.3)
    assert m["focal_spot"]["volume_above_6db_mm3"] == pytest.approx(
        golden["focal_spot"]["volume_above_6db_mm3"], abs=2 * frame_kw["dx"] ** 3 * 1e9)
    for k in ("axial_6db", "lateral_x_6db", "lateral_y_6db"):
        assert m["focal_spot"][k]["truncated"] == golden["focal_spot"][k]["truncated"]
        if not golden["focal_spot"][k]["truncated"]:
            assert m["focal_spot"][k]["width_mm"] == pytest.approx(golden["focal_spot"][k]["width_mm"], abs=2e-3)
    assert m["warnings"] == golden["warnings"]
    assert m.get("harmonics", {}).get("a2_peak_voxel_grid") == golden.get("harmonics", {}).get("a2_peak_voxel_grid")


def test_ties_resolve_to_the_first_voxel_in_c_order():
    shape = (12, 10, 14)
    p = np.zeros(shape, np.complex64)
    p[5, 4, 6] = p[6, 3, 4] = p[5, 4, 9] = 1e6 + 0j  # equal maxima; (5,4,6) comes first in C order
    p[7, 5, 7] = 0 + 1e6j
    res = cg.SolverResult(phasor=p, p_max=np.abs(p).astype(np.float32), region=tuple(slice(0, n) for n in shape),
                          dt=1e-8, spp=10, steps_total=10, t_end_s=1e-7, tof_periods=1, converged_period=1,
                          settle_capped=False, convergence_history=[], phasors={1: p}, meta={})
    frame = cg.FieldFrame(dx=1e-3, grid_shape=shape, pml_vox=1, apex_vox=(0, 0, 0))
    m = cg.focus_metrics(res, frame)
    assert m["peak"]["voxel_grid"] == [5, 4, 6]
    assert m["focal_spot"]["volume_above_6db_mm3"] == pytest.approx(4.0)
    assert m["focal_spot"]["axial_6db"]["truncated"] is False
    want = om.focus_metrics(p, origin=(0, 0, 0), grid_shape=shape, pml_vox=1, apex=(0, 0, 0), dx=1e-3,
                            p_max=res.p_max, run=m["run"])
    assert json.loads(json.dumps(m)) == json.loads(json.dumps(want))


def _label_case(shape=(28, 24, 32), nonlinear=True):
    ids = np.zeros(shape, np.int32)
    x, y, z = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    ids[((x - 14) / 8.0) ** 2 + ((y - 12) / 7.0) ** 2 + ((z - 18) / 6.0) ** 2 <= 1.0] = 1
    ids[z >= 26] = 2
    med = cg.Medium.from_labels(ids, {0: (0.5, 1000.0, 1500.0, 3.5), 1: (8.0, 1050.0, 1580.0, 4.5),
                                      2: (30.0, 1900.0, 2800.0, 0.0)})
    grid = cg.Grid(shape, 0.25e-3, cg.PMLSpec(3 * 0.25e-3))
    src_idx = np.array([[i, j, 5] for i in range(9, 20) for j in range(7, 18)], np.int64)
    src = cg.CWSource(indices=src_idx, phases=np.zeros(len(src_idx), np.float32), amplitude=4e5, f0=1.0e6)
    spec = cg.CWRunSpec(convergence_tol=0.0, min_settle_periods=2, max_settle_periods=3, n_record_periods=1)
    plan = make_plan("westervelt_gb300", grid, med, src, spec, nonlinear=nonlinear, harmonics=(1, 2))
    return grid, med, src, plan


def test_metrics_and_heating_from_a_live_solver_equal_the_uploaded_path():
    grid, med, src, plan = _label_case()
    assert plan.labels is not None
    with DeviceSolver(plan) as dev:
        res = solve(plan, dev=dev)[0]
        frame = cg.FieldFrame(dx=grid.dx, grid_shape=grid.shape, pml_vox=grid.pml_vox, apex_vox=(14, 12, 5),
                              focus_vox=(14, 12, 18))
        md = cg.device_focus_metrics(dev, 0, res, frame, source_amplitude=src.amplitude, medium=med)
        hs = cg.HeatingSource.from_solver(dev, 0, res, med, grid.dx, harmonics=(1, 2), alpha_power_law_y=1.1,
                                          scale=2.0)
    mh = cg.focus_metrics(res, frame, source_amplitude=src.amplitude, medium=med)
    assert json.loads(json.dumps(md)) == json.loads(json.dumps(mh))
    fk = dict(dx=grid.dx, grid_shape=grid.shape, pml_vox=grid.pml_vox, apex_vox=(14, 12, 5), focus_vox=(14, 12, 18))
    want = _oracle(res, fk, med, run=json.loads(json.dumps(mh["run"])), source_amplitude=src.amplitude)
    assert json.loads(json.dumps(md)) == want
    assert "harmonics" in md and md["harmonics"]["a2_at_fundamental_peak_pa"] > 0.0

    # heating: live solver (solver label map) == uploaded phasors == oracle on exact amplitudes
    region = res.region
    q_osc = osen.heating_q(res.phasors, alpha=med.alpha[region], rho=med.rho[region], c=med.c[region],
                           harmonics=(1, 2), alpha_power_law_y=1.1, exact_amp=True)
    q_osc = q_osc * np.float32(2.0)
    full = hs.embed(grid.shape)
    np.testing.assert_array_equal(full[region], q_osc)
    hu = cg.HeatingSource.from_result(res, med, grid.dx, harmonics=(1, 2), alpha_power_law_y=1.1, scale=2.0)
    np.testing.assert_array_equal(hu.q, q_osc)
    assert hs.meta["alpha_model"] == "power_law" and hs.harmonics == (1, 2)
    for n in (1, 2):
        assert hs.meta["mean_q_by_harmonic_w_m3"][n] == pytest.approx(hu.meta["mean_q_by_harmonic_w_m3"][n],
                                                                      rel=1e-12)
        lo, hi = hs.meta["alpha_np_m_range"][n]
        assert (lo, hi) == pytest.approx(hu.meta["alpha_np_m_range"][n], rel=0)

    # the device Q drives the Pennes step exactly as the same Q from the host does
    tm = cg.ThermalMedium.homogeneous(grid.shape, k=0.5, rho=1050.0, specific_heat=3600.0, perfusion=0.0,
                                      dx=grid.dx)
    t0 = np.full(grid.shape, 37.0, np.float32)
    s = cg.PennesSolverGB300(on_unstable="substep")
    a = s.solve(t0, hs, tm, dt=0.05, n_steps=20, dose=True)
    b = s.solve(t0, full, tm, dt=0.05, n_steps=20, dose=True)
    np.testing.assert_array_equal(a.temperature, b.temperature)
    np.testing.assert_array_equal(a.dose_cem43, b.dose_cem43)
    assert "device" in a.meta["q"]
    hs.close()
    hu.close()


def test_heating_on_the_reference_fixture_label_and_dense_paths():
    g = load_golden("heating_q_h12")
    tab, lab = g["table"], g["labels"]
    harm = tuple(int(n) for n in g["harmonics"])
    phasors = {n: g[f"p{n}"] for n in harm}
    alpha, rho, c = tab[lab, 0], tab[lab, 1], tab[lab, 2]
    exact = osen.heating_q(phasors, alpha=alpha, rho=rho, c=c, harmonics=harm, alpha_power_law_y=g["y"],
                           exact_amp=True)
    hs = cg.HeatingSource.from_phasors(phasors, alpha=alpha, rho=rho, c=c, dx=0.3e-3, harmonics=harm,
                                       alpha_power_law_y=g["y"])
    np.testing.assert_array_equal(hs.q, exact)
    np.testing.assert_allclose(hs.q, g["q"], rtol=1e-6, atol=0)  # the reference (NumPy abs)
    # > 256 distinct materials: dense float32 maps on the device
    rng = np.random.default_rng(5)
    alpha_d = rng.uniform(0.0, 40.0, lab.shape).astype(np.float32)
    rho_d = rng.uniform(900.0, 1200.0, lab.shape).astype(np.float32)
    c_d = rng.uniform(1400.0, 1700.0, lab.shape).astype(np.float32)
    hd = cg.HeatingSource.from_phasors(phasors, alpha=alpha_d, rho=rho_d, c=c_d, dx=0.3e-3, harmonics=harm,
                                       alpha_power_law_y=g["y"])
    want = osen.heating_q(phasors, alpha=alpha_d, rho=rho_d, c=c_d, harmonics=harm, alpha_power_law_y=g["y"],
                          exact_amp=True)
    np.testing.assert_array_equal(hd.q, want)
    # placed on a larger grid, zero outside the region
    region = (slice(2, 16), slice(1, 13), slice(3, 21))
    hg = cg.HeatingSource.from_phasors(phasors, alpha=alpha, rho=rho, c=c, dx=0.3e-3, harmonics=harm,
                                       alpha_power_law_y=g["y"], region=region, grid_shape=(20, 16, 24))
    full = hg.embed((20, 16, 24))
    np.testing.assert_array_equal(full[region], exact)
    outside = full.copy()
    outside[region] = 0.0
    assert not outside.any()
    for h in (hs, hd, hg):
        h.close()


def test_heating_refuses_what_the_reference_refuses_before_touching_the_device():
    p = {1: np.ones((4, 5, 6), np.complex64), 2: np.ones((4, 5, 6), np.complex64)}
    with pytest.raises(ValueError, match="above the fundamental"):
        cg.HeatingSource.from_phasors(p, alpha=1.0, rho=1000.0, c=1500.0, dx=1e-3)
    bad = {1: np.full((4, 5, 6), np.nan, np.complex64)}
    with pytest.raises(ValueError, match="non-finite"):
        cg.HeatingSource.from_phasors(bad, alpha=1.0, rho=1000.0, c=1500.0, dx=1e-3)


def test_device_buffers_round_trip():
    a = np.arange(1000, dtype=np.float32).reshape(10, 100)
    d = _lib.DeviceArray.from_host(a)
    np.testing.assert_array_equal(d.to_host(), a)
    d.close()

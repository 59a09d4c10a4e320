"""Host-side set-up against the oracle: discretisation, maps, labels, drive (CPU only)."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import KSPACE_GOLDEN, golden_kspace_kwargs, load_golden
from caustica_gb300 import contract as ct
from caustica_gb300 import engine as eng
from caustica_gb300 import thermal as th
from oracle import kspace as ok
from oracle import pennes as op


def _setup(g):
    kw = golden_kspace_kwargs(g)
    grid = ct.Grid(kw["shape"], kw["dx"], ct.PMLSpec(kw["pml_vox_n"] * kw["dx"]))
    med = ct.Medium(kw["alpha"], kw["rho"], kw["c"], kw["beta"])
    src = ct.CWSource(indices=kw["src_idx"], phases=kw["src_phase"], amplitude=kw["amplitude"], f0=kw["f0"])
    spec = ct.CWRunSpec(cfl=kw["cfl"], cfl_hard_max=kw["cfl_hard_max"], min_settle_periods=kw["min_settle_periods"],
                        max_settle_periods=kw["max_settle_periods"], convergence_tol=kw["convergence_tol"],
                        n_record_periods=kw["n_record_periods"], t_end_min_us=kw["t_end_min_us"])
    return kw, grid, med, src, spec


@pytest.mark.parametrize("name", KSPACE_GOLDEN)
def test_plan_matches_the_reference_discretisation(name):
    g = load_golden(name)
    kw, grid, med, src, spec = _setup(g)
    plan = eng.make_plan("t", grid, med, src, spec, record_region=kw["record_region"],
                         reference_point=kw["reference_point"], nonlinear=kw["nonlinear"], harmonics=kw["harmonics"])
    assert plan.spp == g["spp"]
    assert plan.dt == pytest.approx(g["dt"], rel=1e-15)
    assert plan.tof == g["tof_periods"]
    assert [[s.start, s.stop] for s in plan.rec] == g["region"].tolist()
    assert plan.padded == ok.pad_shape(kw["shape"])


@pytest.mark.parametrize("name", KSPACE_GOLDEN)
def test_device_coefficients_equal_the_reference_float32_maps(name):
    g = load_golden(name)
    kw, grid, med, src, spec = _setup(g)
    plan = eng.make_plan("t", grid, med, src, spec, nonlinear=kw["nonlinear"], harmonics=kw["harmonics"],
                         record_region=kw["record_region"], reference_point=kw["reference_point"])
    want = ok.medium_maps(kw["alpha"], kw["rho"], kw["c"], kw["beta"], plan.padded, plan.dt, kw["nonlinear"],
                          np.float32)
    if plan.labels is not None:
        got = [plan.label_table[plan.labels.reshape(plan.padded), i] for i in range(4)]
    else:
        got = [m.reshape(plan.padded) for m in plan.dense]
    for i in range(3):
        np.testing.assert_array_equal(got[i], want[i])
    if want[3] is not None:
        np.testing.assert_array_equal(got[3], want[3])


def test_label_decomposition_is_exact_and_uses_the_id_map():
    rng = np.random.default_rng(3)
    ids = rng.integers(0, 5, size=(9, 10, 11))
    table = {i: (0.1 * i, 1000.0 + i, 1500.0 + 10 * i, 0.0) for i in range(5)}
    med = ct.Medium.from_labels(ids, table)
    lab, props = eng.label_medium(med)
    for j, key in enumerate(("alpha", "rho", "c", "beta")):
        np.testing.assert_array_equal(props[lab, j], getattr(med, key))
    med.id_map = None
    lab2, props2 = eng.label_medium(med)
    for j, key in enumerate(("alpha", "rho", "c", "beta")):
        np.testing.assert_array_equal(props2[lab2, j], getattr(med, key))


def test_heterogeneous_medium_falls_back_to_dense_maps():
    rng = np.random.default_rng(4)
    shape = (8, 8, 8)
    med = ct.Medium(rng.random(shape), 1000 + rng.random(shape), 1500 + rng.random(shape), np.zeros(shape))
    assert eng.label_medium(med) is None


def test_drive_table_is_the_reference_ramp_and_phase():
    g = load_golden("ks3d_linear_hetero")
    kw, grid, med, src, spec = _setup(g)
    plan = eng.make_plan("t", grid, med, src, spec)
    d = plan.drive_table()
    period = 1.0 / kw["f0"]
    for n in (0, 1, 7, plan.spp * 3 + 2, len(d) - 1):
        t = n * plan.dt
        assert d[n, 0] == np.float32(kw["amplitude"] * ok.ramp_envelope(t, period, 3.0))
        assert d[n, 1] == pytest.approx(np.sin(2 * np.pi * kw["f0"] * t), abs=1e-7)
    ac, as_ = plan.source_amplitudes()
    scale = np.sqrt(ac.astype(np.float64) ** 2 + as_.astype(np.float64) ** 2)
    c_src = kw["c"][tuple(kw["src_idx"].T)]
    np.testing.assert_allclose(scale[0], 2.0 * c_src * plan.dt / kw["dx"], rtol=1e-6)


def test_unknown_run_options_raise_type_error_before_any_device_call():
    from caustica_gb300.solvers import LinearKSpaceGB300

    with pytest.raises(TypeError):
        LinearKSpaceGB300().run(None, None, None, bogus=1)


def test_linear_solver_refuses_a_nonlinear_medium():
    from caustica_gb300.solvers import LinearKSpaceGB300

    grid = ct.Grid((8, 8, 8), 1e-3, ct.PMLSpec(1e-3))
    med = ct.Medium.homogeneous((8, 8, 8), beta=3.5)
    src = ct.CWSource(indices=np.array([[4, 4, 4]]), phases=np.zeros(1), amplitude=1.0, f0=1e5)
    with pytest.raises(ct.SolverCapabilityError):
        LinearKSpaceGB300().run(grid, med, src)


def test_source_entirely_inside_the_pml_is_refused():
    grid = ct.Grid((16, 16, 16), 1e-3, ct.PMLSpec(3e-3))
    med = ct.Medium.homogeneous((16, 16, 16))
    src = ct.CWSource(indices=np.array([[1, 1, 1]]), phases=np.zeros(1), amplitude=1.0, f0=1e5)
    with pytest.raises(ct.SolverCapabilityError):
        ct.validate_setup("x", ct.SolverCaps(frozenset({3}), False, frozenset({"cw"}), frozenset()), grid, med, src)


def test_thermal_coefficients_and_stable_dt_match_the_oracle():
    g = load_golden("pennes3d_insulated")
    tm = th.ThermalMedium(g["k"], g["rho"], g["cp"], g["w"], g["dx"])
    s = th.PennesSolverGB300()
    faces = s._faces(np.asarray(tm.k, np.float32), tm.dx)
    want = op.face_conductances(np.asarray(tm.k, np.float32), tm.dx, np.float32)
    for a, b in zip(faces, want):
        np.testing.assert_array_equal(a, b)
    assert s.stable_dt(tm) == pytest.approx(g["dt_stable"], rel=1e-6)


def test_unstable_thermal_step_is_refused_with_the_bound():
    tm = th.ThermalMedium.homogeneous((6, 6, 6), k=0.5, rho=1000.0, specific_heat=3600.0, perfusion=0.0, dx=1e-4)
    with pytest.raises(th.ThermalStabilityError, match="stability bound"):
        th.PennesSolverGB300().solve(np.full((6, 6, 6), 37.0, np.float32), None, tm, dt=10.0, n_steps=1)


def test_thermal_result_chain_refuses_an_unchained_dose():
    a = th.ThermalResult(np.zeros(3), np.zeros(3), np.ones(3), [], [], 1.0, 1, 1.0, 1)
    b = th.ThermalResult(np.zeros(3), np.zeros(3), np.zeros(3), [], [], 1.0, 1, 1.0, 1)
    with pytest.raises(ValueError, match="not chained"):
        th.ThermalResult.chain([a, b])


def test_stable_step_of_a_single_material_from_the_small_grid_equals_the_full_grid():
    for boundary in ("insulated", "dirichlet"):
        s = th.PennesSolverGB300(boundary=boundary)
        for shape in ((9, 8, 7), (2, 5, 6), (12, 4)):
            tm = th.ThermalMedium.homogeneous(shape, k=0.52, rho=1045.0, specific_heat=3580.0, perfusion=3e-3,
                                              dx=0.25e-3)
            k = np.asarray(tm.k, np.float32)
            walls = s._walls(k, tm.dx) if boundary == "dirichlet" else None
            full = s._stable(tm, s._faces(k, tm.dx), walls, s._perf(tm), s._inv_rho_c(tm))
            assert s.stable_dt(tm) == full


def test_thermal_label_decomposition_is_exact():
    g = load_golden("pennes3d_insulated")
    ids = np.random.default_rng(2).integers(0, 3, g["k"].shape)
    vals = {0: (0.5, 1000.0, 3600.0, 0.0), 1: (0.4, 950.0, 3400.0, 2e-3), 2: (0.55, 1050.0, 3700.0, 5e-3)}
    vols = [np.vectorize(lambda i, j=j: vals[int(i)][j])(ids).astype(np.float32) for j in range(4)]
    tm = th.ThermalMedium(*vols, dx=1e-3)
    lab, props = th.thermal_labels(tm)
    for j, v in enumerate(vols):
        np.testing.assert_array_equal(props[lab, j], v)


@pytest.mark.parametrize("n_mat", [3, 40])
def test_label_decomposition_without_an_id_map_is_exact_for_rare_materials(n_mat):
    """Few materials take the comparison-scan path (a material the 4096-cell
    sample misses is appended), many take the sorting path; both are exact."""
    rng = np.random.default_rng(n_mat)
    shape = (40, 50, 64)
    ids = rng.integers(0, n_mat, shape)
    vals = np.array([[0.5 + 0.01 * i, 1000.0 + i, 3600.0 - i, 1e-4 * i] for i in range(n_mat)], np.float32)
    vols = [vals[ids, j] for j in range(4)]
    vols[1][7, 8, 9] = np.float32(999.25)  # one cell of a material no sample row has
    vols[3][1, 2, 3] = np.float32(-0.0)    # differs from +0.0 only in its bit pattern
    lab, props = eng.label_volumes(vols)
    for j in range(4):
        np.testing.assert_array_equal(props[lab, j].view(np.uint32), vols[j].view(np.uint32))


def test_label_built_media_carry_their_decomposition_and_lose_it_when_a_map_changes():
    from caustica_gb300.engine import label_medium, label_volumes

    rng = np.random.default_rng(12)
    ids = rng.integers(3, 7, (10, 12, 14)).astype(np.int32)  # ids 3..6, lo = 3
    ids[ids == 5] = 6  # id 5 absent inside the range
    table = {i: (0.5 * i, 900.0 + i, 1450.0 + 10 * i, 0.0) for i in range(3, 7)}
    med = ct.Medium.from_labels(ids, table)
    vols = [med.alpha, med.rho, med.c, med.beta]
    want = label_volumes(vols, med.id_map)
    got = label_medium(med)
    np.testing.assert_array_equal(got[0], want[0])
    np.testing.assert_array_equal(got[1], want[1])
    assert not med.c.flags.writeable  # the decomposition stays true
    # replacing a map drops the shortcut: the new maps are decomposed and verified
    med.c = med.c.copy()
    med.c[0, 0, 0] = 1999.0
    lab, props = label_medium(med)
    np.testing.assert_array_equal(props[lab][..., 2], med.c)

"""Pennes + CEM43 on the GPU against the reference's goldens and its float32 path (GPU)."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import PENNES_GOLDEN, load_golden
import caustica_gb300 as cg
from oracle import pennes as op

pytestmark = pytest.mark.gpu

T_TOL = 1e-3  # K, max-abs
DOSE_TOL = 1e-3  # relative


def _solve(g, **kw):
    tm = cg.ThermalMedium(g["k"], g["rho"], g["cp"], g["w"], g["dx"])
    s = cg.PennesSolverGB300(boundary=g["boundary"], on_unstable=g["on_unstable"],
                             reference_temperature_c=g["reference_temperature_c"])
    return s, tm, s.solve(g["t0"], g["q"], tm, dt=g["dt"], n_steps=g["n_steps"], dose=True,
                          record_every=max(1, g["n_steps"] // 3), **kw)


@pytest.mark.parametrize("name", PENNES_GOLDEN)
def test_pennes_matches_reference_fp64(name):
    g = load_golden(name)
    s, tm, res = _solve(g)
    assert res.substeps == g["substeps"]
    assert np.abs(res.temperature - g["T"]).max() < T_TOL
    assert np.abs(res.temperature_max - g["Tmax"]).max() < T_TOL
    rel = np.abs(res.dose_cem43 - g["dose"]) / np.maximum(np.abs(g["dose"]), 1e-30)
    assert rel.max() < DOSE_TOL
    assert len(res.samples) == len(g["samples"])
    if "chain_steps" in g:
        cool = s.solve(res.temperature, None, tm, dt=g["dt"], n_steps=g["chain_steps"], dose=True,
                       dose0=res.dose_cem43)
        assert np.abs(cool.temperature - g["T2"]).max() < T_TOL
        rel2 = np.abs(cool.dose_cem43 - g["dose2"]) / np.abs(g["dose2"])
        assert rel2.max() < DOSE_TOL
        chained = cg.ThermalResult.chain([res, cool])
        assert chained.n_steps == g["n_steps"] + g["chain_steps"]


@pytest.mark.parametrize("name", PENNES_GOLDEN)
def test_temperature_equals_the_reference_float32_path_bit_for_bit(name):
    g = load_golden(name)
    _, _, res = _solve(g)
    ref = op.solve(g["t0"], g["q"], k=g["k"], rho=g["rho"], specific_heat=g["cp"], perfusion=g["w"], dx=g["dx"],
                   dt=g["dt"], n_steps=g["n_steps"], dose=True, boundary=g["boundary"],
                   on_unstable=g["on_unstable"], reference_temperature_c=g["reference_temperature_c"],
                   dtype=np.float32)
    np.testing.assert_array_equal(res.temperature, ref["temperature"])
    np.testing.assert_array_equal(res.temperature_max, ref["temperature_max"])


def test_cem43_unit_definitions_on_the_device():
    """43 C held for 60 s accrues exactly 1 CEM43 minute; 44 C, 2; 42 C, 0.25."""
    shape = (2, 2, 2)
    tm = cg.ThermalMedium.homogeneous(shape, k=1e-12, rho=1000.0, specific_heat=4000.0, perfusion=0.0, dx=1e-3)
    for temp, want in ((43.0, 1.0), (44.0, 2.0), (42.0, 0.25)):
        res = cg.PennesSolverGB300().solve(np.full(shape, temp, np.float32), None, tm, dt=1.0, n_steps=60, dose=True)
        np.testing.assert_allclose(res.dose_cem43, want, rtol=1e-6)


def test_a_non_finite_initial_temperature_is_refused():
    """pennes.py:531-536, checked on the device after the upload."""
    shape = (6, 7, 8)
    tm = cg.ThermalMedium.homogeneous(shape, k=0.5, rho=1050.0, specific_heat=3600.0, perfusion=0.0, dx=1e-3)
    t0 = np.full(shape, 37.0, np.float32)
    t0[3, 4, 5] = np.nan
    with pytest.raises(ValueError, match="temperature0 contains non-finite values"):
        cg.PennesSolverGB300().solve(t0, None, tm, 0.01, 2)


def test_a_state_that_stops_being_finite_raises_instead_of_returning_nan():
    """A near-insulator with a heat source float32 cannot carry (the reference's own recipe)."""
    shape = (8, 8, 8)
    tm = cg.ThermalMedium.homogeneous(shape, k=1e-6, rho=1050.0, specific_heat=3600.0, perfusion=0.0, dx=1e-3)
    s = cg.PennesSolverGB300()
    with pytest.raises(cg.thermal.ThermalDivergedError) as exc:
        s.solve(np.full(shape, 37.0, np.float32), 1e37, tm, s.stable_dt(tm), 300)
    msg = str(exc.value)
    assert "stopped being finite" in msg and "outer step" in msg and "stable_dt" in msg


def test_an_overflowing_dose_is_caught_by_the_same_guard():
    shape = (4, 4, 4)
    tm = cg.ThermalMedium.homogeneous(shape, k=0.5, rho=1050.0, specific_heat=3600.0, perfusion=0.0, dx=1e-3)
    with pytest.raises(cg.thermal.ThermalDivergedError, match="CEM43 dose"):
        cg.PennesSolverGB300().solve(np.full(shape, 37.0, np.float32), 2.0e6, tm, 1.0, 400, dose=True)


# The larger shapes span several tiles of the streaming label kernels (even
# nz: z-pairs; odd nz: single cells); 40 materials exceed the 32-material
# face table.
@pytest.mark.parametrize("shape,boundary,tref,n_ids", [((10, 9, 12), "insulated", None, 3),
                                                       ((9, 11, 8), "dirichlet", 36.0, 3),
                                                       ((14, 12), "dirichlet", None, 3),
                                                       ((12, 10), "insulated", 38.0, 3),
                                                       ((70, 19, 40), "insulated", None, 3),
                                                       ((40, 17, 70), "dirichlet", 36.0, 5),
                                                       ((33, 20, 36), "dirichlet", None, 40),
                                                       ((21, 18, 37), "dirichlet", 37.0, 4),
                                                       ((6, 5, 2), "insulated", None, 3)])
def test_label_coefficients_equal_the_reference_float32_path(shape, boundary, tref, n_ids):
    rng = np.random.default_rng(sum(shape))
    ids = rng.integers(0, n_ids, shape)
    vals = {0: (0.5, 1000.0, 3600.0, 0.0), 1: (0.4, 950.0, 3400.0, 2e-3), 2: (0.55, 1050.0, 3700.0, 5e-3)}
    for i in range(3, n_ids):
        vals[i] = (0.3 + 0.01 * i, 900.0 + 5.0 * i, 3300.0 + 10.0 * i, 1e-4 * i)
    vols = [np.vectorize(lambda i, j=j: vals[int(i)][j])(ids).astype(np.float32) for j in range(4)]
    tm = cg.ThermalMedium(*vols, dx=0.3e-3)
    q = (rng.random(shape) ** 3 * 4e6).astype(np.float32)
    t0 = (37.0 + rng.uniform(0, 3, shape)).astype(np.float32)
    s = cg.PennesSolverGB300(boundary=boundary, reference_temperature_c=tref, on_unstable="substep")
    res = s.solve(t0, q, tm, dt=0.05, n_steps=30, dose=True)
    assert res.meta["coefficients"] == "labels"
    kw = dict(k=vols[0], rho=vols[1], specific_heat=vols[2], perfusion=vols[3], dx=tm.dx, dt=0.05, n_steps=30,
              dose=True, boundary=boundary, reference_temperature_c=tref, on_unstable="substep")
    ref32 = op.solve(t0, q, dtype=np.float32, **kw)
    np.testing.assert_array_equal(res.temperature, ref32["temperature"])
    ref64 = op.solve(t0, q, dtype=np.float64, **kw)
    assert np.abs(res.temperature - ref64["temperature"]).max() < T_TOL
    rel = np.abs(res.dose_cem43 - ref64["dose_cem43"]) / np.maximum(np.abs(ref64["dose_cem43"]), 1e-30)
    assert rel.max() < DOSE_TOL

"""Pin the oracle to the reference: every committed fixture, CPU only.

The fixtures were produced by the unchanged reference (FP64 backend plugin,
plus one stock FP32 run); see ``tests/golden/make_golden.py``.
"""

from __future__ import annotations

import numpy as np
import pytest

from conftest import KSPACE_GOLDEN, PENNES_GOLDEN, golden_kspace_kwargs, load_golden, rel_l2
from oracle import kspace as ok
from oracle import pennes as op


@pytest.mark.parametrize("name", KSPACE_GOLDEN)
def test_oracle_matches_reference_fp64(name):
    g = load_golden(name)
    res = ok.run_cw(**golden_kspace_kwargs(g), dtype=np.float64)
    assert res["spp"] == g["spp"]
    assert res["dt"] == pytest.approx(g["dt"], rel=1e-15)
    assert res["steps_total"] == g["steps_total"]
    assert res["tof_periods"] == g["tof_periods"]
    assert res["converged_period"] == g["converged_period"]
    assert res["settle_capped"] == bool(g["settle_capped"])
    hist = np.array(res["convergence_history"], np.float64).reshape(-1, 3)
    np.testing.assert_allclose(hist, g["history"], rtol=1e-10, equal_nan=True)
    assert np.array([[s.start, s.stop] for s in res["region"]]).tolist() == g["region"].tolist()
    for h in np.atleast_1d(g["harmonics"]):
        assert rel_l2(res["phasors"][int(h)], g[f"phasor_h{int(h)}"]) < 1e-11
    np.testing.assert_allclose(res["p_max"], g["p_max"], rtol=1e-11, atol=1e-6)


def test_oracle_fp32_mode_matches_reference_stock_path():
    g = load_golden("ks3d_fp32_reference")
    res = ok.run_cw(**golden_kspace_kwargs(g), dtype=np.float32)
    assert res["phasor"].dtype == np.complex64
    # Same arithmetic in the same order with the same library: bit-identical.
    np.testing.assert_array_equal(res["phasor"], g["phasor_h1"])
    np.testing.assert_array_equal(res["p_max"], g["p_max"])


def test_plane_wave_case_converged_before_its_cap():
    g = load_golden("ks1d_plane_converge")
    assert not g["settle_capped"]
    assert g["converged_period"] < g["tof_periods"] + 60


@pytest.mark.parametrize("name", PENNES_GOLDEN)
def test_pennes_oracle_matches_reference_fp64(name):
    g = load_golden(name)
    res = op.solve(
        g["t0"], g["q"], k=g["k"], rho=g["rho"], specific_heat=g["cp"], perfusion=g["w"], dx=g["dx"],
        dt=g["dt"], n_steps=g["n_steps"], dose=True, boundary=g["boundary"], on_unstable=g["on_unstable"],
        reference_temperature_c=g["reference_temperature_c"], record_every=max(1, g["n_steps"] // 3),
        dtype=np.float64,
    )
    assert res["substeps"] == g["substeps"]
    assert res["dt_stable_s"] == pytest.approx(g["dt_stable"], rel=1e-12)
    np.testing.assert_array_equal(res["temperature"], g["T"])
    np.testing.assert_array_equal(res["temperature_max"], g["Tmax"])
    np.testing.assert_allclose(res["dose_cem43"], g["dose"], rtol=1e-6)
    np.testing.assert_array_equal(np.array(res["samples"]), g["samples"])
    if "chain_steps" in g:
        cool = op.solve(res["temperature"], None, k=g["k"], rho=g["rho"], specific_heat=g["cp"],
                        perfusion=g["w"], dx=g["dx"], dt=g["dt"], n_steps=g["chain_steps"], dose=True,
                        dose0=res["dose_cem43"], dtype=np.float64)
        np.testing.assert_array_equal(cool["temperature"], g["T2"])
        np.testing.assert_allclose(cool["dose_cem43"], g["dose2"], rtol=1e-6)


def test_cem43_unit_definitions():
    """43 C for 60 s is 1 minute, 44 C is 2, 42 C is 0.25 (dose.py:92-102)."""
    r = op.cem43_rate(np.array([43.0, 44.0, 42.0]))
    np.testing.assert_allclose(r, [1.0, 2.0, 0.25], rtol=1e-15)

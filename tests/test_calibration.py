"""Planner calibration entries for the GB300 backend (planner/calibration.py:151-584)."""

from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

from caustica_gb300 import calibration as cal
from conftest import reference_src

# the fields of the reference's calibration entry (planner/calibration.py:536-570)
REFERENCE_ENTRY_KEYS = {"a", "b", "fit_mode", "global_fit_mode", "fit_max_rel_residual", "interp_loo_rel_err",
                        "p_max_probe", "warmup_context_s", "warmup_per_elem_s", "warmup_s", "warmup_source",
                        "backend", "n_steps", "nonlinear", "samples", "shapes", "vram_peak_bytes_by_shape",
                        "calibrated_at"}


def _runs(ps, a=2e-12, b=3e-10):
    return [{"device": "NVIDIA GB300", "backend": "gb300", "shape": (round(p ** (1 / 3)),) * 3, "p_elems": p,
             "t_step_s": a * p * np.log2(p) + b * p, "warmup_s": 0.5 + 1e-8 * p, "vram_peak_bytes": 40 * p}
            for p in ps]


def test_fit_recovers_the_time_law():
    ps = [128 ** 3, 256 ** 3, 512 ** 3]
    a, b = cal.fit_time_model([(r["p_elems"], r["t_step_s"]) for r in _runs(ps)])
    assert a == pytest.approx(2e-12, rel=1e-6) and b == pytest.approx(3e-10, rel=1e-6)


def test_fit_clips_a_negative_coefficient():
    samples = [(1_000_000, 1e-3), (8_000_000, 4e-3)]  # sub-linear: the P log P term would go negative
    a, b = cal.fit_time_model(samples)
    assert a == 0.0 and b > 0.0


def test_probes_fill_the_memory_fractions_of_a_large_device():
    shapes = cal.probe_shapes_for_budget(270 << 30)
    sides = [s[0] for s in shapes]
    assert len(shapes) >= 2 and sides == sorted(sides) and sides[-1] ** 3 >= cal.MIN_PROBE_CELLS
    for (n, _, _), frac in zip(shapes, cal.PROBE_MEMORY_FRACTIONS):
        assert cal.probe_footprint_bytes(n) <= (270 << 30) * frac


def test_a_small_budget_falls_back_to_two_throughput_sized_probes():
    assert cal.probe_shapes_for_budget(1 << 28) == ((128, 128, 128), (192, 192, 192))


def test_entry_has_the_reference_schema_and_merges_into_the_file(tmp_path):
    path = tmp_path / "calibration.json"
    path.write_text(json.dumps({"version": 1, "devices": {"NVIDIA A100-SXM4-40GB": {"a": 1.0}}}))
    entry = cal.make_entry(_runs([96 ** 3, 160 ** 3, 256 ** 3]), 20, False)
    assert set(entry) == REFERENCE_ENTRY_KEYS
    assert entry["global_fit_mode"] == "nnls" and entry["fit_max_rel_residual"] < 1e-9
    assert entry["warmup_per_elem_s"] == pytest.approx(0.5 / 256 ** 3 + 1e-8, rel=1e-9)  # the smallest later ratio
    cal.write_entry("NVIDIA GB300", entry, path)
    data = json.loads(path.read_text())
    assert set(data["devices"]) == {"NVIDIA A100-SXM4-40GB", "NVIDIA GB300"}
    assert data["devices"]["NVIDIA GB300"]["samples"][0] == [96 ** 3, entry["samples"][0][1]]


def test_the_reference_planner_reads_the_entry():
    src = reference_src()
    if src is None or not (src / "caustica" / "planner" / "calibration.py").exists():
        pytest.skip("reference sources not present (set CAUSTICA_REFERENCE_SRC)")
    sys.path.insert(0, str(src))
    try:
        ref = pytest.importorskip("caustica.planner.calibration")
    finally:
        sys.path.remove(str(src))
    entry = cal.make_entry(_runs([96 ** 3, 160 ** 3, 256 ** 3]), 20, False)
    for p, t in entry["samples"]:
        assert ref.predict_step_time(entry, p) == pytest.approx(t, rel=1e-6)
    mid = ref.predict_step_time(entry, 200 ** 3)
    assert entry["samples"][1][1] < mid < entry["samples"][2][1]
    # the same fit and residual as the reference's on the same samples
    rng = np.random.default_rng(11)
    for _ in range(5):
        samples = [(int(p), float(t)) for p, t in zip(sorted(rng.integers(10 ** 6, 10 ** 9, 3)),
                                                      sorted(rng.uniform(1e-4, 1e-1, 3)))]
        a, b = cal.fit_time_model(samples)
        ra, rb = ref.fit_time_model(samples)
        assert a == pytest.approx(ra, rel=1e-9, abs=1e-30) and b == pytest.approx(rb, rel=1e-9, abs=1e-30)
        assert cal.max_rel_residual(samples, a, b) == pytest.approx(ref.fit_max_rel_residual(samples, ra, rb),
                                                                     rel=1e-9)


@pytest.mark.gpu
def test_calibrate_measures_this_device(tmp_path):
    entry = cal.calibrate(((64, 64, 64), (128, 128, 128)), n_steps=8, path=tmp_path / "c.json")
    (p0, t0), (p1, t1) = entry["samples"]
    assert p0 == 64 ** 3 and p1 == 128 ** 3 and 0.0 < t0 < t1
    data = json.loads((tmp_path / "c.json").read_text())
    (name,) = data["devices"]
    assert name and data["devices"][name]["backend"] == "gb300"

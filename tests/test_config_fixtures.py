"""The full-size fixtures hold the inputs the workload builders make (no GPU).

``make_config_golden.py`` ran the reference on the inputs of
``caustica_gb300.workloads``; the parity tests rebuild those inputs from the
fixture itself (label map, material table, source voxels, phases). This
checks that the two agree, so the bench times the workloads the fixtures
pin, and that every fixture carries the tolerance-relevant pieces.
"""

from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
from caustica_gb300 import workloads


def _have(name):
    return (GOLDEN / f"{name}.npz").exists()


def _labels_of(medium):
    ids = np.asarray(medium.id_map if medium.id_map is not None else np.zeros(medium.shape, np.int32))
    return ids.astype(np.uint8)


@pytest.mark.parametrize("name,builder", [("cfg1_linear_96x96x128", workloads.config1),
                                          ("cfg2_westervelt_192x192x256", workloads.config2)])
def test_acoustic_fixture_inputs_equal_the_workload(name, builder):
    if not _have(name):
        pytest.skip("fixture not generated")
    g = load_golden(name)
    w = builder()
    assert tuple(g["shape"]) == w["grid"].shape and g["dx"] == w["grid"].dx
    np.testing.assert_array_equal(g["labels"], _labels_of(w["medium"]))
    np.testing.assert_array_equal(g["src_idx"].astype(np.int64), w["source"].indices)
    np.testing.assert_array_equal(g["src_phase"], w["source"].phases)
    assert g["amplitude"] == w["source"].amplitude and g["f0"] == w["source"].f0
    spec = g["spec"] if isinstance(g["spec"], dict) else json.loads(g["spec"])
    assert spec == w["spec"].model_dump()
    for h in w["harmonics"]:
        assert f"h{h}_lattice" in g and f"h{h}_box" in g
    assert json.loads(g["metrics"])["peak"]["p_pa"] > 0


def test_cfg1_fixture_is_the_surveyed_fp64_solve():
    if not _have("cfg1_linear_96x96x128"):
        pytest.skip("fixture not generated")
    g = load_golden("cfg1_linear_96x96x128")
    m = json.loads(g["metrics"])
    assert g["spp"] == 33 and g["steps_total"] == 1320
    assert m["peak"]["voxel_grid"] == [48, 48, 90]
    assert abs(m["peak"]["p_pa"] - 702.1e3) < 100.0


def test_cfg4_fixture_inputs_equal_the_workload():
    if not _have("cfg4_steer_160x160x192"):
        pytest.skip("fixture not generated")
    g = load_golden("cfg4_steer_160x160x192")
    w = workloads.config4()
    np.testing.assert_array_equal(g["labels"], _labels_of(w["medium"]))
    np.testing.assert_array_equal(g["src_idx"].astype(np.int64), w["source"].indices)
    for b in g["members"]:
        np.testing.assert_array_equal(g[f"m{int(b)}_phases"], w["phases"][int(b)])

"""Focal metrics and heating Q: the oracle against the reference's own output,
and the host half of the device post-processing (CPU only).

The device half (``cg_focus_metrics`` / ``cg_heating_q``) is simulated here by
a report built with NumPy from the same correctly rounded amplitudes the
kernels use, so the dictionary assembly, the crossing arithmetic and the
refusals are checked without a GPU.
"""

from __future__ import annotations

import json

import numpy as np
import pytest

from conftest import FOCUS_GOLDEN, focus_case, load_golden
from oracle import metrics as om
from oracle import sensors as osen


def _oracle_dict(res, frame, med, *, exact):
    p1 = res.phasors[1]
    p2 = res.phasors.get(2)
    return om.focus_metrics(
        p1, origin=tuple(s.start for s in res.region), grid_shape=frame["grid_shape"], pml_vox=frame["pml_vox"],
        apex=frame["apex_vox"], dx=frame["dx"], focus=frame["focus_vox"], p2=p2, p_max=res.p_max,
        rho=None if med is None else med.rho, c=None if med is None else med.c, source_amplitude=1e5,
        run=None, amp=om.exact_amp(p1) if exact else None,
        amp2=om.exact_amp(p2) if (exact and p2 is not None) else None)


@pytest.mark.parametrize("name", FOCUS_GOLDEN)
def test_metrics_oracle_matches_reference(name):
    res, frame, med, golden = focus_case(name)
    m = _oracle_dict(res, frame, med, exact=False)
    gold = dict(golden)
    gold.pop("run")
    assert json.loads(json.dumps(m)) == gold


def test_golden_cases_cover_the_metric_branches():
    res, frame, _, g = focus_case("focus_h2_target")
    assert g["warnings"] and "harmonics" in g and "target" in g
    # the spike inside the PML margin is larger than the focus and must lose
    assert float(np.abs(res.phasor).max()) > g["peak"]["p_pa"]
    _, _, med, g2 = focus_case("focus_truncated")
    assert g2["focal_spot"]["lateral_y_6db"]["truncated"] and med is None and "target" not in g2


def test_heating_oracle_matches_reference():
    g = load_golden("heating_q_h12")
    tab = g["table"]
    lab = g["labels"]
    phasors = {int(n): g[f"p{int(n)}"] for n in g["harmonics"]}
    q = osen.heating_q(phasors, alpha=tab[lab, 0], rho=tab[lab, 1], c=tab[lab, 2],
                       harmonics=tuple(int(n) for n in g["harmonics"]), alpha_power_law_y=g["y"])
    np.testing.assert_array_equal(q, g["q"])
    # correctly rounded amplitudes move Q by a few float32 units at most
    qe = osen.heating_q(phasors, alpha=tab[lab, 0], rho=tab[lab, 1], c=tab[lab, 2],
                        harmonics=tuple(int(n) for n in g["harmonics"]), alpha_power_law_y=g["y"], exact_amp=True)
    np.testing.assert_allclose(qe, g["q"], rtol=1e-6, atol=0)


def _simulated_report(p1, p2, pmax, q):
    """What cg_focus_metrics returns, computed with NumPy on exact amplitudes."""
    from caustica_gb300 import _lib

    a1 = om.exact_amp(p1)
    box = tuple(slice(q.lo[i], q.hi[i]) for i in range(3))
    pk = om.argmax_in(a1, box)
    rep = _lib.FocusReport()
    rep.peak = int(np.ravel_multi_index(pk, a1.shape))
    rep.p_peak = float(a1[pk])
    rep.p_max_at_peak = float(pmax[pk])
    rep.n_above_half = int((a1[box] >= 0.5 * a1[pk]).sum())
    probe = tuple(q.probe[i] for i in range(3))
    rep.p_probe = float(a1[probe]) if min(probe) >= 0 else float("nan")
    rep.has_a2 = int(p2 is not None)
    if p2 is not None:
        a2 = om.exact_amp(p2)
        pk2 = om.argmax_in(a2, box)
        rep.a2_at_peak = float(a2[pk])
        rep.a2_peak = float(a2[pk2])
        rep.a2_peak_index = int(np.ravel_multi_index(pk2, a2.shape))
    lines = [a1[:, pk[1], pk[2]], a1[pk[0], :, pk[2]], a1[pk[0], pk[1], :]]
    for d in range(3):
        coord = (np.arange(a1.shape[d]) + q.offset[d]) * q.dx
        level = 0.5 * float(lines[d][pk[d]])
        right = om.crossing(coord, lines[d], pk[d], level)
        left = om.crossing(coord[::-1], lines[d][::-1], a1.shape[d] - 1 - pk[d], level)
        rep.truncated[d] = int(right is None or left is None)
        rep.left[d] = float("nan") if rep.truncated[d] else left
        rep.right[d] = float("nan") if rep.truncated[d] else right
    return rep


@pytest.mark.parametrize("name", FOCUS_GOLDEN)
def test_host_assembly_of_a_device_report(name):
    from caustica_gb300 import metrics as cm

    res, frame_kw, med, golden = focus_case(name)
    frame = cm.FieldFrame(**frame_kw)
    org = cm.region_origin(res)
    q = cm._query(org, res.phasor.shape, frame)
    rep = _simulated_report(res.phasors[1], res.phasors.get(2), res.p_max, q)
    m = cm._assemble(rep, res, frame, org, res.phasor.shape, source_amplitude=1e5, medium=med, solver=None)
    want = _oracle_dict(res, frame_kw, med, exact=True)
    want["run"] = golden["run"]
    assert json.loads(json.dumps(m)) == json.loads(json.dumps(want))
    # and the exact-amplitude answer is the reference's to within its rounding
    assert m["peak"]["voxel_grid"] == golden["peak"]["voxel_grid"]
    assert m["peak"]["p_pa"] == pytest.approx(golden["peak"]["p_pa"], abs=0.3)
    assert m["focal_spot"]["volume_above_6db_mm3"] == pytest.approx(golden["focal_spot"]["volume_above_6db_mm3"],
                                                                     abs=2 * frame.dx ** 3 * 1e9)


def test_interior_box_matches_the_oracle_and_refuses_an_all_sponge_region():
    from caustica_gb300 import metrics as cm

    frame = cm.FieldFrame(dx=1e-3, grid_shape=(40, 36, 48), pml_vox=4, apex_vox=(0, 0, 0))
    for org, shape in [((2, 1, 3), (36, 34, 43)), ((0, 0, 0), (40, 36, 48)), ((10, 10, 10), (5, 6, 7))]:
        assert cm._interior(org, shape, frame) == om.interior(org, shape, frame.grid_shape, frame.pml_vox)
    with pytest.raises(ValueError, match="inside the PML margin"):
        cm._interior((0, 0, 0), (5, 36, 48), frame)
    with pytest.raises(ValueError, match="3-D"):
        cm._query((0, 0), (40, 36), frame)


def test_heating_refusals_mirror_the_reference():
    from caustica_gb300 import sensors as cs

    a = np.ones((2, 3), np.float64)
    with pytest.raises(ValueError, match="above the fundamental"):
        cs._resolve_alpha((1, 2), a, available=(1, 2), alpha_power_law_y=None, alpha_at_harmonics=None)
    with pytest.raises(ValueError, match="physical range"):
        cs._resolve_alpha((1, 2), a, available=(1, 2), alpha_power_law_y=3.5, alpha_at_harmonics=None)
    with pytest.raises(ValueError, match="EITHER"):
        cs._resolve_alpha((1, 2), a, available=(1, 2), alpha_power_law_y=1.0, alpha_at_harmonics={2: 1.0})
    with pytest.raises(ValueError, match="missing harmonic"):
        cs._resolve_alpha((1, 2, 3), a, available=(1, 2, 3), alpha_power_law_y=None, alpha_at_harmonics={2: 1.0})
    with pytest.raises(ValueError, match="not in the result"):
        cs._requested((1,), (1, 2))
    with pytest.raises(ValueError, match="alpha must be >= 0"):
        cs._check_maps(-a, a, a, a.shape)
    with pytest.raises(ValueError, match="rho and c must be > 0"):
        cs._check_maps(a, 0 * a, a, a.shape)
    maps, factors = cs._resolve_alpha((1, 2), a * 3.0, available=(1, 2), alpha_power_law_y=1.1,
                                      alpha_at_harmonics=None)
    np.testing.assert_array_equal(maps[2], a * 3.0 * 2.0 ** 1.1)
    assert factors == {1: 1.0, 2: 2.0 ** 1.1}


def test_float64_labels_are_exact():
    from caustica_gb300 import sensors as cs

    rng = np.random.default_rng(3)
    tab = rng.uniform(0, 1, (7, 3))
    lab = rng.integers(0, 7, (5, 6, 4))
    vols = [tab[lab, i] for i in range(3)]
    labels, props = cs._labels_f64(vols)
    for i in range(3):
        np.testing.assert_array_equal(props[labels, i], vols[i])
    many = [rng.uniform(0, 1, (20, 20)) for _ in range(2)]
    assert cs._labels_f64(many) is None

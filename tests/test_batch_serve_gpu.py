"""Batched steering and the continuous-batching server against solo solves (GPU)."""

from __future__ import annotations

import numpy as np
import pytest

import caustica_gb300 as cg
from caustica_gb300 import serve
from caustica_gb300.batch import solve_steering
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _setup(shape, seed, nonlinear=False, n_src=20):
    rng = np.random.default_rng(seed)
    ids = rng.integers(0, 3, shape)
    table = {0: (0.5, 1000.0, 1500.0, 3.5 if nonlinear else 0.0), 1: (8.0, 1050.0, 1580.0, 4.5 if nonlinear else 0.0),
             2: (3.0, 950.0, 1450.0, 5.0 if nonlinear else 0.0)}
    med = cg.Medium.from_labels(ids, table)
    grid = cg.Grid(shape, 0.25e-3, cg.PMLSpec(2 * 0.25e-3))
    pts = set()
    while len(pts) < n_src:
        pts.add((int(rng.integers(3, shape[0] - 3)), int(rng.integers(3, shape[1] - 3)), int(rng.integers(3, 6))))
    idx = np.array(sorted(pts), np.int64)
    return grid, med, idx, rng


def _same_metrics(a, b, where):
    """Equal structure and integers; floats within the rounding the metrics are reported with."""
    if isinstance(a, dict):
        assert isinstance(b, dict) and a.keys() == b.keys(), where
        for k in a:
            _same_metrics(a[k], b[k], where + (k,))
    elif isinstance(a, list):
        assert isinstance(b, list) and len(a) == len(b), where
        for x, y in zip(a, b):
            _same_metrics(x, y, where)
    elif isinstance(a, float) and isinstance(b, float):
        assert a == pytest.approx(b, rel=1e-5, abs=0.2), where
    else:
        assert a == b, where


def _solo(grid, med, idx, ph, spec, nonlinear, harmonics=(1,)):
    src = cg.CWSource(indices=idx, phases=ph, amplitude=2e5, f0=1e6)
    s = cg.WesterveltKSpaceGB300() if nonlinear else cg.LinearKSpaceGB300()
    return s.run(grid, med, src, spec, harmonics=harmonics)


# the larger z axes run the persistent z-passes on 20- and 32-thread pencils
# with a ragged last y-tile, for every member of the batch
@pytest.mark.parametrize("shape", [(16, 24, 32), (12, 40, 400), (8, 34, 640)])
def test_steering_batch_members_equal_their_solo_solves(shape):
    grid, med, idx, rng = _setup(shape, 1)
    phases = rng.uniform(0, 2 * np.pi, (5, len(idx))).astype(np.float32)
    spec = cg.CWRunSpec(convergence_tol=0.0, min_settle_periods=2, max_settle_periods=3, n_record_periods=2)
    res = solve_steering(grid, med, idx, phases, f0=1e6, amplitude=2e5, spec=spec)
    assert len(res) == 5
    for b in (0, 3, 4):
        solo = _solo(grid, med, idx, phases[b], spec, False)
        assert rel_l2(res[b].phasor, solo.phasor) < 1e-6
        np.testing.assert_allclose(res[b].p_max, solo.p_max, rtol=1e-6, atol=1e-3)
        assert res[b].steps_total == solo.steps_total


def test_converging_batch_replays_each_members_own_decisions():
    grid, med, idx, rng = _setup((16, 16, 24), 2)
    phases = rng.uniform(0, 2 * np.pi, (3, len(idx))).astype(np.float32)
    spec = cg.CWRunSpec(convergence_tol=0.02, min_settle_periods=2, max_settle_periods=12, n_record_periods=1)
    res = solve_steering(grid, med, idx, phases, f0=1e6, amplitude=2e5, spec=spec)
    for b in range(3):
        solo = _solo(grid, med, idx, phases[b], spec, False)
        assert res[b].converged_period == solo.converged_period
        assert rel_l2(res[b].phasor, solo.phasor) < 1e-6


def test_server_results_are_the_same_alone_and_in_the_mix():
    reqs = []
    spec = cg.CWRunSpec(convergence_tol=0.0, min_settle_periods=2, max_settle_periods=3, n_record_periods=2)
    grid_a, med_a, idx_a, rng = _setup((16, 24, 32), 3)
    for k in range(3):  # packable: same grid, medium, voxels, spec
        ph = rng.uniform(0, 2 * np.pi, len(idx_a)).astype(np.float32)
        src = cg.CWSource(indices=idx_a, phases=ph, amplitude=2e5, f0=1e6)
        reqs.append(serve.Request(grid=grid_a, medium=med_a, source=src, spec=spec, tag=("a", k)))
    grid_b, med_b, idx_b, rng_b = _setup((24, 16, 24), 4, nonlinear=True)
    src_b = cg.CWSource(indices=idx_b, phases=np.zeros(len(idx_b), np.float32), amplitude=2e5, f0=1e6)
    frame_b = cg.FieldFrame(dx=grid_b.dx, grid_shape=grid_b.shape, pml_vox=grid_b.pml_vox, apex_vox=(12, 8, 2),
                            focus_vox=(12, 8, 14))
    reqs.append(serve.Request(grid=grid_b, medium=med_b, source=src_b, spec=spec, nonlinear=True, harmonics=(1, 2),
                              frame=frame_b, tag=("b", 0)))
    tm = cg.ThermalMedium.homogeneous(grid_a.shape, k=0.5, rho=1000.0, specific_heat=3600.0, perfusion=5e-4,
                                      dx=grid_a.dx)
    src_t = cg.CWSource(indices=idx_a, phases=np.zeros(len(idx_a), np.float32), amplitude=2e5, f0=1e6)
    reqs.append(serve.Request(grid=grid_a, medium=med_a, source=src_t, spec=spec, tag=("t", 0),
                              thermal={"medium": tm, "dt": 0.05, "n_heat": 20, "n_cool": 10, "q_scale": 1e4},
                              frame=cg.FieldFrame(dx=grid_a.dx, grid_shape=grid_a.shape, pml_vox=grid_a.pml_vox,
                                                  apex_vox=(8, 12, 2))))
    with serve.Server(max_pack=8) as srv:
        futs = [srv.submit(r) for r in reqs]
        outs = [f.result(timeout=300) for f in futs]
        stats = dict(srv.stats)
    assert max(o.group_size for o in outs) > 1, "compatible requests were not packed"
    assert stats["groups"] < len(reqs)
    for r, o in zip(reqs, outs):
        solo = _solo(r.grid, r.medium, r.source.indices, r.source.phases, r.spec, r.nonlinear, r.harmonics)
        for h in r.harmonics:
            assert rel_l2(o.result.phasors[h], solo.phasors[h]) < 1e-6, r.tag
        if r.frame is not None:
            # device metrics of the packed handle == metrics of the solo result
            want_m = cg.focus_metrics(solo, r.frame, source_amplitude=r.source.amplitude, medium=r.medium)
            for k in ("peak", "focal_spot", "harmonics", "target"):
                _same_metrics(o.metrics.get(k), want_m.get(k), (r.tag, k))
        else:
            assert o.metrics is None
        if r.thermal is not None:
            want = serve.run_thermal(r, solo)
            assert np.abs(o.thermal.temperature - want.temperature).max() < 1e-5
            np.testing.assert_allclose(o.thermal.dose_cem43, want.dose_cem43, rtol=1e-5, atol=1e-12)
        assert o.latency_s > 0


def test_server_admits_by_budget_and_still_finishes_everything():
    spec = cg.CWRunSpec(convergence_tol=0.0, min_settle_periods=2, max_settle_periods=2, n_record_periods=1)
    reqs = []
    for k in range(4):
        grid, med, idx, rng = _setup((16, 16, 24), 10 + k)
        src = cg.CWSource(indices=idx, phases=np.zeros(len(idx), np.float32), amplitude=2e5, f0=1e6)
        reqs.append(serve.Request(grid=grid, medium=med, source=src, spec=spec))
    # a budget that holds one request at a time
    with serve.Server(hbm_budget_bytes=1) as srv:
        outs = [f.result(timeout=300) for f in [srv.submit(r) for r in reqs]]
        assert srv.stats["max_active"] == 1
    assert len(outs) == 4


def test_requests_arriving_while_the_gpu_is_busy_pack_across_arrivals():
    """A long request holds the whole budget; three compatible requests that
    arrive one after another while it runs (their media equal in content but
    built separately) wait, are packed into one handle when memory frees,
    and each result equals its solo solve."""
    import time

    spec_long = cg.CWRunSpec(convergence_tol=0.0, min_settle_periods=40, max_settle_periods=40, n_record_periods=2)
    grid_l, med_l, idx_l, _ = _setup((64, 64, 96), 21)
    src_l = cg.CWSource(indices=idx_l, phases=np.zeros(len(idx_l), np.float32), amplitude=2e5, f0=1e6)
    long_req = serve.Request(grid=grid_l, medium=med_l, source=src_l, spec=spec_long, tag="long")
    spec = cg.CWRunSpec(convergence_tol=0.0, min_settle_periods=2, max_settle_periods=3, n_record_periods=2)
    late = []
    for k in range(3):
        grid, med, idx, rng = _setup((16, 24, 32), 22)  # same seed: equal media, distinct objects
        ph = np.random.default_rng(100 + k).uniform(0, 2 * np.pi, len(idx)).astype(np.float32)
        late.append(serve.Request(grid=grid, medium=med, source=cg.CWSource(indices=idx, phases=ph, amplitude=2e5,
                                                                            f0=1e6), spec=spec, tag=("late", k)))
    assert late[0].medium is not late[1].medium
    from caustica_gb300.engine import device_footprint, make_plan

    plan_l = make_plan("x", grid_l, med_l, src_l, spec_long)
    plan_s = make_plan("x", late[0].grid, late[0].medium, late[0].source, spec)
    # room for the long request or the packed three, never for the long one and any other
    budget = max(device_footprint(plan_l, 1), device_footprint(plan_s, 3))
    assert budget < device_footprint(plan_l, 1) + device_footprint(plan_s, 1)
    with serve.Server(hbm_budget_bytes=budget, max_pack=8) as srv:
        futs = [srv.submit(long_req)]
        for r in late:
            time.sleep(0.002)
            futs.append(srv.submit(r))
        outs = [f.result(timeout=300) for f in futs]
        stats = dict(srv.stats)
    assert stats["groups"] == 2, stats
    assert [o.group_size for o in outs[1:]] == [3, 3, 3]
    assert outs[1].t_admit >= outs[0].t_done - 1e-3  # admitted once the long request released its memory
    for r, o in zip(late, outs[1:]):
        solo = _solo(r.grid, r.medium, r.source.indices, r.source.phases, r.spec, False)
        assert rel_l2(o.result.phasor, solo.phasor) < 1e-6, r.tag


def test_served_requests_carry_device_store_fields_of_their_own_result():
    from oracle import quantize as oq

    spec = cg.CWRunSpec(convergence_tol=0.0, min_settle_periods=2, max_settle_periods=2, n_record_periods=1)
    grid, med, idx, rng = _setup((16, 16, 24), 41, nonlinear=True)
    reqs = [serve.Request(grid=grid, medium=med, nonlinear=True, harmonics=(1, 2), spec=spec, store_quantize=1e-3,
                          source=cg.CWSource(indices=idx, phases=rng.uniform(-3, 3, len(idx)).astype(np.float32),
                                             amplitude=2e5, f0=1e6))
            for _ in range(3)]
    reqs.append(serve.Request(grid=grid, medium=med, nonlinear=True, harmonics=(1, 2), spec=spec,
                              source=reqs[0].source))
    with serve.Server() as srv:
        outs = [f.result(timeout=300) for f in [srv.submit(r) for r in reqs]]
    for o in outs[:3]:
        q = o.result.meta["quantized"]
        for name, f in oq.store_order(o.result.phasors, o.result.p_max):
            ref = oq.try_float16(f)
            got = q["fields"][name]
            assert got.dtype_name == ref.dtype_name and got.scale == ref.scale and got.norm_err == ref.norm_err
            assert np.array_equal(np.asarray(got.stored).view(np.uint8), np.asarray(ref.stored).view(np.uint8))
    assert "quantized" not in outs[3].result.meta

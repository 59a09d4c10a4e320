"""Checkpoint / resume and the divergence guard through the real kernels (GPU).

Checkpoints (the reference's tests/test_checkpoint.py:61-140): a run stopped
at a period boundary and resumed from its ``caustica-checkpoint/1`` file
reproduces the uninterrupted GB300 run bit for bit -- the saved state is
float32 through an uncompressed npz and the step is deterministic.

Divergence (tests/test_divergence_guard.py:26-58): a drive float32 cannot
carry overflows the field in the first period and the solve raises
``SolverDivergedError`` naming the settling period; a state that turns
non-finite inside the record window (a pre-record snapshot whose pressure
was corrupted on disk) raises naming the record window. Both failures are
made on the host: the kernels only ever see finite or IEEE-special floats.
"""

from __future__ import annotations

import numpy as np
import pytest

import caustica_gb300 as cg

pytestmark = pytest.mark.gpu

F0, C0 = 1.0e6, 1500.0


def _setup_1d(amplitude=1e5):
    dx = C0 / (F0 * 4.0)
    grid = cg.Grid((96,), dx, cg.PMLSpec(12 * dx))
    med = cg.Medium.homogeneous(grid.shape, alpha_np_m=0.0253, rho=1000.0, c=C0)
    src = cg.CWSource(indices=np.array([[18]]), phases=np.zeros(1, np.float32), amplitude=amplitude, f0=F0)
    spec = cg.CWRunSpec(min_settle_periods=10, max_settle_periods=24)
    return grid, med, src, spec, cg.LinearKSpaceGB300(), (1,)


def _setup_3d_westervelt():
    rng = np.random.default_rng(17)
    shape = (20, 24, 28)
    dx = 0.2e-3
    grid = cg.Grid(shape, dx, cg.PMLSpec(3 * dx))
    labels = rng.integers(0, 3, shape)
    table = {0: (2.5, 1000.0, 1500.0, 3.5), 1: (8.0, 1050.0, 1580.0, 4.7), 2: (20.0, 1090.0, 1610.0, 4.95)}
    med = cg.Medium.from_labels(labels, table)
    idx = np.array([[10, 12, 5], [10, 13, 5], [9, 12, 5], [11, 11, 6], [10, 12, 6]])
    src = cg.CWSource(indices=idx, phases=rng.uniform(-1, 1, len(idx)).astype(np.float32), amplitude=1.2e6, f0=F0)
    spec = cg.CWRunSpec(min_settle_periods=3, max_settle_periods=9, convergence_tol=0.005, n_record_periods=2)
    return grid, med, src, spec, cg.WesterveltKSpaceGB300(), (1, 2)


def _setup_3d_size_specialised():
    """A grid whose every axis runs the size-specialised passes (persistent
    z-passes): the restored spectrum must come from the step's own kernel."""
    rng = np.random.default_rng(23)
    shape = (32, 48, 64)
    dx = 0.2e-3
    grid = cg.Grid(shape, dx, cg.PMLSpec(3 * dx))
    labels = rng.integers(0, 3, shape)
    table = {0: (2.5, 1000.0, 1500.0, 3.5), 1: (8.0, 1050.0, 1580.0, 4.7), 2: (20.0, 1090.0, 1610.0, 4.95)}
    med = cg.Medium.from_labels(labels, table)
    idx = np.array([[16, 24, 5], [16, 25, 5], [15, 24, 5], [17, 23, 6], [16, 24, 6]])
    src = cg.CWSource(indices=idx, phases=rng.uniform(-1, 1, len(idx)).astype(np.float32), amplitude=1.2e6, f0=F0)
    spec = cg.CWRunSpec(min_settle_periods=3, max_settle_periods=9, convergence_tol=0.005, n_record_periods=2)
    return grid, med, src, spec, cg.WesterveltKSpaceGB300(), (1, 2)


SETUPS = {"linear_1d": _setup_1d, "westervelt_3d": _setup_3d_westervelt,
          "westervelt_3d_size_specialised": _setup_3d_size_specialised}


def _stop_after(k: int):
    """A stop_when that fires on the k-th period-boundary poll."""
    calls = {"n": 0}

    def stop() -> bool:
        calls["n"] += 1
        return calls["n"] >= k

    return stop


def _assert_identical(a, b):
    np.testing.assert_array_equal(a.phasor, b.phasor)
    np.testing.assert_array_equal(a.p_max, b.p_max)
    assert sorted(a.phasors) == sorted(b.phasors)
    for h in a.phasors:
        np.testing.assert_array_equal(a.phasors[h], b.phasors[h])
    assert a.steps_total == b.steps_total
    assert a.converged_period == b.converged_period
    assert a.settle_capped == b.settle_capped
    assert a.convergence_history == b.convergence_history


@pytest.mark.parametrize("setup", sorted(SETUPS))
def test_interrupt_then_resume_reproduces_the_uninterrupted_run(setup, tmp_path):
    grid, med, src, spec, solver, harm = SETUPS[setup]()
    baseline = solver.run(grid, med, src, spec, harmonics=harm)
    ck = tmp_path / "run.ckpt.npz"
    with pytest.raises(cg.RunInterrupted) as exc:
        solver.run(grid, med, src, spec, harmonics=harm,
                   checkpoint=cg.CheckpointSpec(path=ck, every_periods=2, stop_when=_stop_after(3)))
    assert exc.value.periods_done == 3 and exc.value.stage == "settle"
    assert exc.value.steps_done == 3 * baseline.spp
    assert ck.exists()
    resumed = solver.run(grid, med, src, spec, harmonics=harm, checkpoint=cg.CheckpointSpec(path=ck))
    _assert_identical(baseline, resumed)
    assert not ck.exists()  # removed on success


def test_a_chain_of_interruptions_still_resumes_bit_exactly(tmp_path):
    grid, med, src, spec, solver, harm = _setup_1d()
    baseline = solver.run(grid, med, src, spec)
    ck = tmp_path / "chain.ckpt.npz"
    for k in (2, 4):  # stopped twice, at different depths
        with pytest.raises(cg.RunInterrupted):
            solver.run(grid, med, src, spec,
                       checkpoint=cg.CheckpointSpec(path=ck, every_periods=3, stop_when=_stop_after(k)))
    resumed = solver.run(grid, med, src, spec, checkpoint=cg.CheckpointSpec(path=ck))
    _assert_identical(baseline, resumed)


@pytest.mark.parametrize("setup", sorted(SETUPS))
def test_resume_from_the_pre_record_snapshot(setup, tmp_path):
    grid, med, src, spec, solver, harm = SETUPS[setup]()
    baseline = solver.run(grid, med, src, spec, harmonics=harm)
    ck = tmp_path / "rec.ckpt.npz"
    # the poll after the last settled period is the pre-record one
    with pytest.raises(cg.RunInterrupted) as exc:
        solver.run(grid, med, src, spec, harmonics=harm,
                   checkpoint=cg.CheckpointSpec(path=ck, every_periods=64,
                                                stop_when=_stop_after(baseline.converged_period + 1)))
    assert exc.value.stage == "record"
    resumed = solver.run(grid, med, src, spec, harmonics=harm,
                         checkpoint=cg.CheckpointSpec(path=ck, keep_on_success=True))
    _assert_identical(baseline, resumed)
    assert ck.exists()  # keep_on_success


def test_a_state_that_turns_non_finite_in_the_record_window_raises(tmp_path):
    grid, med, src, spec, solver, harm = _setup_3d_westervelt()
    ck = tmp_path / "nan.ckpt.npz"
    baseline = solver.run(grid, med, src, spec, harmonics=harm)
    with pytest.raises(cg.RunInterrupted):
        solver.run(grid, med, src, spec, harmonics=harm,
                   checkpoint=cg.CheckpointSpec(path=ck, every_periods=64,
                                                stop_when=_stop_after(baseline.converged_period + 1)))
    # corrupt one pressure voxel of the pre-record snapshot on disk; the
    # fingerprint still matches, so the resume runs the record window on it
    with np.load(ck, allow_pickle=False) as z:
        payload = {k: z[k] for k in z.files}
    payload["field_p"] = payload["field_p"].copy()
    payload["field_p"][10, 12, 14] = np.float32(np.nan)
    with open(ck, "wb") as fh:
        np.savez(fh, **payload)
    with pytest.raises(cg.SolverDivergedError) as exc:
        solver.run(grid, med, src, spec, harmonics=harm, checkpoint=cg.CheckpointSpec(path=ck))
    assert "record window" in str(exc.value)


def _tiny(amplitude, beta=0.0):
    grid = cg.Grid((24, 24, 24), 0.5e-3, None)
    med = cg.Medium.homogeneous(grid.shape, alpha_np_m=0.0253, rho=1000.0, c=C0, beta=beta)
    src = cg.CWSource(indices=np.array([[12, 12, 6]]), phases=np.zeros(1, np.float32), amplitude=amplitude, f0=F0)
    return grid, med, src, cg.CWRunSpec(min_settle_periods=1, max_settle_periods=3)


@pytest.mark.parametrize("solver", [cg.LinearKSpaceGB300, cg.WesterveltKSpaceGB300])
def test_a_drive_float32_cannot_carry_raises_instead_of_returning_nan(solver):
    grid, med, src, spec = _tiny(1e38, beta=3.5 if solver.nonlinear else 0.0)
    with pytest.raises(cg.SolverDivergedError) as exc:
        solver().run(grid, med, src, spec)
    msg = str(exc.value)
    assert "diverged" in msg
    assert "settling period" in msg
    assert "CFL" in msg


@pytest.mark.parametrize("solver", [cg.LinearKSpaceGB300, cg.WesterveltKSpaceGB300])
def test_a_healthy_run_of_the_same_shape_still_returns(solver):
    grid, med, src, spec = _tiny(1e4, beta=3.5 if solver.nonlinear else 0.0)
    res = solver().run(grid, med, src, spec)
    assert np.isfinite(res.phasor).all()
    assert np.isfinite(res.p_max).all()


def test_a_diverging_steering_member_raises():
    """Batched members are guarded too: one member driven past float32 fails the call."""
    from caustica_gb300.batch import solve_steering

    grid, med, src, spec = _tiny(1e38)
    phases = np.zeros((2, 1), np.float32)
    with pytest.raises(cg.SolverDivergedError):
        solve_steering(grid, med, src.indices, phases, f0=F0, amplitude=1e38, spec=spec)

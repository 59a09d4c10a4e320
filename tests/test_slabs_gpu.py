"""Slab mode of the step: bit-identical to the plain eight-launch step (GPU).

In slab mode (``cg_solver_set_slabs``) the plane-local passes run over runs
of x-planes in turn, so each run's spectra and fields stay in L2 between
its y-, z- and y-passes. Every cell is still computed by the same kernel
code from the same inputs, so whole solves -- fields, phasors, p_max, the
per-period peaks -- must be bitwise equal to the plain step's, for any slab
count (including ragged slabs), batch size and medium storage, and a handle
may switch modes between steps.
"""

from __future__ import annotations

import numpy as np
import pytest

import caustica_gb300 as cg
from caustica_gb300.engine import DeviceSolver, make_plan, solve

pytestmark = pytest.mark.gpu


def _case(shape, nonlinear, seed, dense=False):
    rng = np.random.default_rng(seed)
    dx = 0.2e-3
    grid = cg.Grid(shape, dx, cg.PMLSpec(3 * dx))
    if dense:
        c = rng.uniform(1450.0, 1650.0, shape).astype(np.float32)
        rho = rng.uniform(900.0, 1100.0, shape).astype(np.float32)
        alpha = rng.uniform(0.0, 20.0, shape).astype(np.float32)
        beta = np.full(shape, 4.0 if nonlinear else 0.0, np.float32)
        med = cg.Medium(alpha, rho, c, beta)
    else:
        labels = rng.integers(0, 4, shape)
        table = {i: (float(rng.uniform(0, 20)), float(rng.uniform(900, 1100)), float(rng.uniform(1450, 1650)),
                     4.0 if nonlinear else 0.0) for i in range(4)}
        med = cg.Medium.from_labels(labels, table)
    n = 40
    pts = set()
    while len(pts) < n:
        pts.add(tuple(int(rng.integers(4, s - 4)) for s in shape))
    idx = np.array(sorted(pts), np.int64)
    src = cg.CWSource(indices=idx, phases=rng.uniform(-np.pi, np.pi, n).astype(np.float32), amplitude=8e5, f0=1e6)
    spec = cg.CWRunSpec(cfl=0.4, convergence_tol=0.0, min_settle_periods=2, max_settle_periods=3, n_record_periods=1)
    rec = tuple(slice(2, s - 3) for s in shape)
    return make_plan("westervelt_gb300" if nonlinear else "linear_gb300", grid, med, src, spec, record_region=rec,
                     nonlinear=nonlinear, harmonics=(1, 2) if nonlinear else (1,))


def _solve(plan, slabs, phases=None):
    batch = 1 if phases is None else phases.shape[0]
    with DeviceSolver(plan, batch=batch, phases=phases, autotune=False) as dev:
        dev.set_slabs(slabs)
        assert dev.config()["slabs"] == slabs
        return solve(plan, dev=dev, phases=phases)


def _same(a, b):
    for h in a.phasors:
        np.testing.assert_array_equal(a.phasors[h], b.phasors[h])
    np.testing.assert_array_equal(a.p_max, b.p_max)
    assert a.convergence_history == b.convergence_history


@pytest.mark.parametrize("shape,nonlinear,dense,slabs", [
    ((32, 48, 64), True, False, 2),
    ((32, 48, 64), True, False, 5),    # ragged runs of 6 and 7 planes
    ((48, 32, 96), False, False, 3),
    ((24, 64, 48), True, True, 4),     # dense float32 maps
    ((64, 64, 64), False, False, 8),
])
def test_slab_step_is_bitwise_the_plain_step(shape, nonlinear, dense, slabs):
    plan = _case(shape, nonlinear, seed=sum(shape) + slabs, dense=dense)
    ref = _solve(plan, 1)[0]
    got = _solve(plan, slabs)[0]
    _same(ref, got)


def test_slab_step_batched_members_are_bitwise_the_plain_step():
    plan = _case((32, 48, 64), False, seed=5)
    rng = np.random.default_rng(9)
    phases = rng.uniform(-np.pi, np.pi, (3, plan.src_xyz.shape[0])).astype(np.float32)
    ref = _solve(plan, 1, phases)
    got = _solve(plan, 3, phases)
    for a, b in zip(ref, got):
        _same(a, b)


def test_switching_modes_between_steps_keeps_the_trajectory():
    plan = _case((32, 48, 64), True, seed=13)
    n = 3 * plan.spp
    with DeviceSolver(plan, autotune=False) as dev:
        dev.run_steps(n)
        p_ref, u_ref = dev.get_state()
        dev.reset()
        dev.run_steps(n // 3)
        dev.set_slabs(4)
        dev.run_steps(n // 3)
        dev.set_slabs(1)
        dev.run_steps(n - 2 * (n // 3))
        p, u = dev.get_state()
    np.testing.assert_array_equal(p, p_ref)
    np.testing.assert_array_equal(u, u_ref)


def test_slab_counts_outside_the_supported_range_are_refused():
    from caustica_gb300 import _lib

    plan = _case((32, 48, 64), False, seed=3)
    with DeviceSolver(plan, autotune=False) as dev:
        for bad in (0, 9, 33):
            with pytest.raises(_lib.CGInvalidArgument, match="slabs"):
                dev.set_slabs(bad)
        assert dev.config()["slabs"] == 1

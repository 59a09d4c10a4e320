"""Tensor-map (TMA) staging of the persistent z-tiles (GPU).

With ``cg_solver_set_zstaging(s, 1)`` the persistent z-passes receive each
tile's half spectra by two tensor-map box copies completed on an mbarrier
and read them through the 128-byte swizzle, instead of per-thread 16-byte
``cp.async`` into padded rows. Every kernel computes from the same staged
values, so whole solves -- phasors, p_max, the per-period peaks -- must be
bitwise equal either way: on 16-, 20- and 32-thread pencils, ragged last
y-tiles, batches, label and dense media. Grids the staging cannot serve are
refused.
"""

from __future__ import annotations

import numpy as np
import pytest

import caustica_gb300 as cg
from caustica_gb300 import _lib
from caustica_gb300.engine import DeviceSolver, solve
from test_slabs_gpu import _case, _same

pytestmark = pytest.mark.gpu


def _solve(plan, tma, phases=None):
    batch = 1 if phases is None else phases.shape[0]
    with DeviceSolver(plan, batch=batch, phases=phases, autotune=False) as dev:
        dev.set_zstaging(tma)
        assert dev.config()["tma_staging"] == tma
        out = solve(plan, dev=dev, phases=phases)
        assert dev.config()["tma_staging"] == tma
        return out


@pytest.mark.parametrize("shape,nonlinear,dense", [
    ((16, 32, 64), True, False),
    ((20, 34, 64), False, False),     # ragged last y-tile (34 = 32 + 2)
    ((12, 48, 256), True, False),     # the 256-point kernels of config 2
    ((10, 40, 320), False, False),    # 20-thread pencils, ragged tile
    ((10, 32, 400), True, False),     # 201 k rows per box
    ((24, 64, 48), True, True),       # dense float32 maps
])
def test_tensor_map_staging_is_bitwise_the_cp_async_staging(shape, nonlinear, dense):
    plan = _case(shape, nonlinear, seed=sum(shape), dense=dense)
    ref = _solve(plan, False)[0]
    got = _solve(plan, True)[0]
    _same(ref, got)


def test_batched_members_are_bitwise_equal_with_either_staging():
    plan = _case((16, 40, 96), False, seed=11)
    n = plan.src_xyz.shape[0]
    phases = np.random.default_rng(3).uniform(-np.pi, np.pi, (3, n)).astype(np.float32)
    for a, b in zip(_solve(plan, False, phases), _solve(plan, True, phases)):
        _same(a, b)


def test_switching_staging_between_periods_keeps_the_run_bitwise():
    plan = _case((16, 32, 128), True, seed=4)
    with DeviceSolver(plan, autotune=False) as a, DeviceSolver(plan, autotune=False) as b:
        a.set_zstaging(False)
        b.set_zstaging(True)
        a.run_periods(2)
        b.run_periods(1)
        b.set_zstaging(False)
        b.run_periods(1)
        np.testing.assert_array_equal(a.get_state()[0], b.get_state()[0])
        np.testing.assert_array_equal(a.read_peaks(0, 2), b.read_peaks(0, 2))


def test_grids_without_the_staging_are_refused():
    odd = _case((16, 27, 64), False, seed=2)        # odd (2/3/5-smooth) ny: no persistent z-passes
    wide = _case((10, 16, 512), False, seed=2)      # 257 k rows: above the 256-row box
    for plan in (odd, wide):
        with DeviceSolver(plan, autotune=False) as dev:
            with pytest.raises(_lib.CGInvalidArgument, match="tensor-map staging"):
                dev.set_zstaging(True)
            assert dev.config()["tma_staging"] is False


def test_the_tuner_reports_its_staging_choice():
    plan = _case((16, 32, 64), False, seed=9)
    with DeviceSolver(plan) as dev:
        assert isinstance(dev.tuning["tma_staging"], bool)
        assert dev.tuning["tma_staging"] == dev.config()["tma_staging"]


def test_handles_created_and_destroyed_from_several_threads_stay_bitwise():
    """Handles of different grids come and go concurrently (as in a serving
    process), so a new handle's staging can follow a freed one's on the same
    device: every tensor-map-staged run must still equal its cp.async run."""
    import threading

    plans = [_case(shape, nl, seed=40 + i) for i, (shape, nl) in
             enumerate([((16, 32, 64), False), ((12, 40, 128), True), ((10, 34, 320), False)])]

    def run(plan, tma):
        with DeviceSolver(plan, autotune=False) as dev:
            dev.set_zstaging(tma)
            dev.run_periods(1)
            return dev.get_state()[0], dev.read_peaks(0, 1)

    want = [run(p, False) for p in plans]
    errors = []

    def worker(k):
        try:
            for r in range(6):
                i = (k + r) % len(plans)
                p, peaks = run(plans[i], True)
                np.testing.assert_array_equal(p, want[i][0])
                np.testing.assert_array_equal(peaks, want[i][1])
        except Exception as exc:  # noqa: BLE001 - reported below
            errors.append(exc)

    threads = [threading.Thread(target=worker, args=(k,)) for k in range(3)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors, errors

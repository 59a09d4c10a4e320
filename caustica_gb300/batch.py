"""Many right-hand sides over one medium in one launch (steering batches).

``solve_steering(grid, medium, indices, phases, ...)`` runs B CW solves that
share the grid, the medium, the drive frequency/amplitude and the source
voxel set, and differ in their per-voxel phases (e.g. the delay-and-sum
phases of a phased array steered to B targets). Every kernel launch of the
step covers all B members (grid dimension y); the medium tables, k-space
tables and twiddles are read once per tile for all of them. Each result is
the one the plain solver returns for that member alone.
"""

from __future__ import annotations

import numpy as np

from .contract import CWRunSpec, CWSource, SolverResult
from .engine import DeviceSolver, make_plan, solve


def solve_steering(grid, medium, indices, phases, *, f0: float, amplitude: float, spec: CWRunSpec | None = None,
                   nonlinear: bool = False, harmonics=(1,), record_region=None, reference_point=None,
                   ramp_periods: float = 3.0, max_batch: int | None = None, name: str = "steering_gb300",
                   result_cls=SolverResult, quantize: float | None = None) -> list:
    """Solve B steering positions; ``phases`` is (B, n_voxels) float32, host
    or device (a device array is read back: the source scale is formed with
    the host's float32 arithmetic either way). ``quantize`` also attaches
    each member's device-quantised store fields (``meta["quantized"]``)."""
    from .device import is_device_array, to_host

    if is_device_array(phases):
        phases = to_host(phases, np.float32)
    phases = np.ascontiguousarray(np.atleast_2d(np.asarray(phases, np.float32)))
    indices = np.asarray(indices, np.int64)
    if phases.shape[1] != indices.shape[0]:
        raise ValueError(f"phases have {phases.shape[1]} voxels, indices {indices.shape[0]}")
    spec = spec or CWRunSpec()
    src0 = CWSource(indices=indices, phases=phases[0], amplitude=amplitude, f0=f0, ramp_periods=ramp_periods)
    plan = make_plan(name, grid, medium, src0, spec, record_region=record_region, reference_point=reference_point,
                     nonlinear=nonlinear, harmonics=harmonics)
    B = phases.shape[0]
    chunk = B if max_batch is None else max(1, int(max_batch))
    out = []
    for lo in range(0, B, chunk):
        part = phases[lo:lo + chunk]
        with DeviceSolver(plan, batch=part.shape[0], phases=part) as dev:
            out.extend(solve(plan, phases=part, dev=dev, result_cls=result_cls, quantize=quantize))
    return out

"""GB300 CW solvers with the reference's solver interface.

``LinearKSpaceGB300`` / ``WesterveltKSpaceGB300`` take exactly the arguments
of the reference fronts (solvers/kspace/linear.py:37-68,
westervelt.py:41-72): ``run(grid, medium, source, spec=None, backend="auto",
record_region=None, reference_point=None, harmonics=(1,), checkpoint=None,
progress=None)`` and return a ``SolverResult``. Unknown keyword arguments
raise ``TypeError`` (linear.py:51-52); setups are validated as
``SolverBase.validate`` does (solvers/base.py:178-201).

When caustica itself is importable, :mod:`caustica_gb300.plugin` registers
subclasses of caustica's own ``SolverBase`` under the names
``linear_gb300`` / ``westervelt_gb300``.
"""

from __future__ import annotations

from typing import Any

from . import contract
from .checkpoint import run_with_checkpoint
from .engine import make_plan, solve


class KSpaceGB300Base:
    """Shared front of the two GB300 CW solvers."""

    name = "kspace_gb300"
    nonlinear = False
    caps = contract.SolverCaps(ndim=frozenset({1, 2, 3}), nonlinear=False, drive=frozenset({"cw"}),
                               backends=frozenset({"gb300"}))
    result_cls = contract.SolverResult
    spec_cls = contract.CWRunSpec
    capability_error = contract.SolverCapabilityError
    # a bound on the relative round-trip error (1e-3 is the store's default):
    # run() then also quantises the stored fields on the device, for
    # caustica_gb300.store.save_result, as result.meta["quantized"]
    store_quantize: float | None = None

    def validate(self, grid, medium, source) -> None:
        contract.validate_setup(self.name, self.caps, grid, medium, source)

    def run(self, grid, medium, source, spec=None, backend: str = "auto", record_region=None,
            reference_point=None, harmonics=(1,), checkpoint=None, progress=None, **kwargs: Any):
        if kwargs:
            raise TypeError(f"unknown run() options: {sorted(kwargs)}")
        spec = spec or self.spec_cls()
        self.validate(grid, medium, source)
        plan = make_plan(self.name, grid, medium, source, spec, record_region=record_region,
                         reference_point=reference_point, nonlinear=self.nonlinear, harmonics=harmonics)
        if checkpoint is not None:
            return run_with_checkpoint(plan, checkpoint, progress=progress, result_cls=self.result_cls,
                                       grid=grid, medium=medium, source=source)
        return solve(plan, progress=progress, result_cls=self.result_cls, quantize=self.store_quantize)[0]


class LinearKSpaceGB300(KSpaceGB300Base):
    """Linear k-space PSTD on GB300 (1/2/3-D, CW steady state)."""

    name = "linear_gb300"
    nonlinear = False
    caps = contract.SolverCaps(ndim=frozenset({1, 2, 3}), nonlinear=False, drive=frozenset({"cw"}),
                               backends=frozenset({"gb300"}))


class WesterveltKSpaceGB300(KSpaceGB300Base):
    """Westervelt (nonlinear) k-space PSTD on GB300 (1/2/3-D, CW steady state)."""

    name = "westervelt_gb300"
    nonlinear = True
    caps = contract.SolverCaps(ndim=frozenset({1, 2, 3}), nonlinear=True, drive=frozenset({"cw"}),
                               backends=frozenset({"gb300"}))


SOLVERS = {cls.name: cls for cls in (LinearKSpaceGB300, WesterveltKSpaceGB300)}


def get(name: str):
    """Solver class by registry name (the shape of ``caustica.solvers.get``)."""
    try:
        return SOLVERS[name]
    except KeyError:
        raise KeyError(f"unknown solver {name!r}; available: {sorted(SOLVERS)}") from None

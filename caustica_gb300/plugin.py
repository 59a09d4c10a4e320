"""Registration of the GB300 solvers into caustica's solver registry.

Loaded by caustica through the ``caustica.solvers`` entry-point group
(registry.py:49, solvers/registry.py:26-52), declared in this project's
``pyproject.toml``::

    [project.entry-points."caustica.solvers"]
    linear_gb300 = "caustica_gb300.plugin:LinearKSpaceGB300"
    westervelt_gb300 = "caustica_gb300.plugin:WesterveltKSpaceGB300"

The classes below subclass caustica's own ``SolverBase`` and return its own
``SolverResult``; the errors a solve can raise are re-raised as caustica's
``SolverDivergedError`` / ``RunInterrupted`` / ``CheckpointMismatch`` so the
runner's handlers (runner.py:1025-1060) see the types they expect.

:func:`install_compat` is the one place this project touches caustica
internals: the runner, the facade and the planner model only the solver
names ``linear``/``westervelt`` (runner.py:111, facade.py:68,504,
planner/__init__.py:307), so a plugin solver would otherwise run unplanned
and without backend, checkpoint and progress options.
"""

from __future__ import annotations

import dataclasses
from typing import Any

from caustica.io.checkpoint import CheckpointMismatch as _CkMismatch
from caustica.io.checkpoint import RunInterrupted as _Interrupted
from caustica.solvers.base import CWRunSpec, SolverBase, SolverCaps, SolverDivergedError, SolverResult

from . import checkpoint as _ck
from . import contract
from .solvers import KSpaceGB300Base

NAMES = ("linear_gb300", "westervelt_gb300")


def _run(front: KSpaceGB300Base, args, kwargs):
    try:
        return KSpaceGB300Base.run(front, *args, **kwargs)
    except contract.SolverDivergedError as exc:
        raise SolverDivergedError(str(exc)) from exc
    except _ck.RunInterrupted as exc:
        raise _Interrupted(exc.checkpoint_path, exc.stage, exc.periods_done, exc.steps_done) from exc
    except _ck.CheckpointMismatch as exc:
        raise _CkMismatch(str(exc)) from exc


class LinearKSpaceGB300(SolverBase):
    """caustica solver ``linear_gb300``: the linear k-space PSTD on GB300."""

    name = "linear_gb300"
    caps = SolverCaps(ndim=frozenset({1, 2, 3}), nonlinear=False, drive=frozenset({"cw"}),
                      backends=frozenset({"gb300"}))
    _front = type("_LinearFront", (KSpaceGB300Base,),
                  {"name": "linear_gb300", "nonlinear": False, "result_cls": SolverResult, "spec_cls": CWRunSpec})

    def run(self, grid, medium, source, spec=None, **kwargs: Any) -> SolverResult:
        front = self._front()
        front.caps = self.caps
        front.validate = self.validate  # caustica's own SolverBase.validate
        front.store_quantize = getattr(self, "store_quantize", None)
        return _run(front, (grid, medium, source, spec), kwargs)


class WesterveltKSpaceGB300(SolverBase):
    """caustica solver ``westervelt_gb300``: the Westervelt k-space PSTD on GB300."""

    name = "westervelt_gb300"
    caps = SolverCaps(ndim=frozenset({1, 2, 3}), nonlinear=True, drive=frozenset({"cw"}),
                      backends=frozenset({"gb300"}))
    _front = type("_WesterveltFront", (KSpaceGB300Base,),
                  {"name": "westervelt_gb300", "nonlinear": True, "result_cls": SolverResult, "spec_cls": CWRunSpec})

    def run(self, grid, medium, source, spec=None, **kwargs: Any) -> SolverResult:
        front = self._front()
        front.caps = self.caps
        front.validate = self.validate
        front.store_quantize = getattr(self, "store_quantize", None)
        return _run(front, (grid, medium, source, spec), kwargs)


def register() -> None:
    """Register both classes in caustica's registry (idempotent)."""
    from caustica.solvers import registry

    for cls in (LinearKSpaceGB300, WesterveltKSpaceGB300):
        if cls.name not in registry.available():
            registry.register(cls)


def install_compat() -> None:
    """Let caustica's runner, facade and planner treat the GB300 names as native.

    * appends ``linear_gb300``/``westervelt_gb300`` to
      ``caustica.runner._NATIVE_SOLVERS`` and ``caustica.facade._NATIVE_SOLVERS``
      (the facade binds the tuple by value at import, facade.py:68);
    * wraps ``caustica.planner.estimate`` so a ``*_gb300`` name is planned
      with the inventory of its reference counterpart.
    Opt-in and idempotent.
    """
    import caustica.facade as facade
    import caustica.planner as planner
    import caustica.runner as runner

    register()
    for mod in (runner, facade):
        names = tuple(getattr(mod, "_NATIVE_SOLVERS", ()))
        setattr(mod, "_NATIVE_SOLVERS", names + tuple(n for n in NAMES if n not in names))
    if not getattr(planner.estimate, "_gb300_wrapped", False):
        original = planner.estimate

        def estimate(*args, solver: str = "westervelt", **kwargs):
            if not solver.endswith("_gb300"):
                return original(*args, solver=solver, **kwargs)
            est = original(*args, solver=solver[: -len("_gb300")], **kwargs)
            # the verdict names the solver that will run
            return dataclasses.replace(est, solver=solver) if dataclasses.is_dataclass(est) else est

        estimate._gb300_wrapped = True  # type: ignore[attr-defined]
        planner.estimate = estimate
        if hasattr(runner, "estimate"):
            runner.estimate = estimate


def result_store(root, *, probe: bool = True):
    """caustica's own ``ResultStore`` (io/store.py:338-398) whose ``save`` quantises on the GPU.

    The directory plumbing -- verified mkdir, write probe, temp-debris sweep,
    the resume scan, ``load`` -- is the reference's; ``save`` writes the same
    ``caustica-result/1`` file through :func:`caustica_gb300.store.save_result`,
    so the float16 fields a GB300 solve attached (or the result's arrays,
    quantised on the device) are stored without a host quantisation pass.
    caustica's store module imports h5py, so this needs it as well.
    """
    from caustica.io import store as ref_store

    from . import store as gb_store

    class ResultStoreGB300(ref_store.ResultStore):
        def save(self, name, result, source, **kwargs):
            ref_store.ensure_dir_verified(self.root)  # re-verified at write time, as the reference's save does
            return gb_store.save_result(self.path(name), result, source, **kwargs)

    return ResultStoreGB300(root, probe=probe)

"""caustica_gb300 -- GB300-native (sm_103a) k-space CW solver and Pennes/CEM43 step.

A drop-in for caustica's ``linear``/``westervelt`` solvers and its
``PennesSolver``: the host code here mirrors the reference interfaces and
calls ``libcaustica_gb300.so`` (C ABI, ``include/caustica_gb300.h``) through
ctypes. Every time step runs in hand-written CUDA kernels; there is no CPU
fallback. The focal metrics (``report/metrics.py``) and the heating source
(``sensors.py``) of a result are reduced on the GPU as well.
"""

from .contract import (
    CWRunSpec,
    CWSource,
    Grid,
    Medium,
    PMLSpec,
    SolverCapabilityError,
    SolverDivergedError,
    SolverResult,
)
from .checkpoint import CheckpointMismatch, CheckpointSpec, RunInterrupted
from .metrics import FieldFrame, device_focus_metrics, focus_metrics
from .sensors import HeatingSource
from .solvers import LinearKSpaceGB300, WesterveltKSpaceGB300, get
from .thermal import PennesSolverGB300, ThermalMedium, ThermalResult

__all__ = [
    "CWRunSpec", "CWSource", "Grid", "Medium", "PMLSpec", "SolverCapabilityError", "SolverDivergedError",
    "SolverResult", "LinearKSpaceGB300", "WesterveltKSpaceGB300", "get", "PennesSolverGB300", "ThermalMedium",
    "ThermalResult", "FieldFrame", "focus_metrics", "device_focus_metrics", "HeatingSource", "CheckpointSpec",
    "CheckpointMismatch", "RunInterrupted",
]
__version__ = "0.1.0"

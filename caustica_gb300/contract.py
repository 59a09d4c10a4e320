"""The reference's solver data contract, restated for hosts without caustica.

The GB300 solvers accept the reference's own objects (``caustica.Grid``,
``Medium``, ``CWSource``, ``CWRunSpec``) by duck typing. Where caustica is not
installed (the GPU hosts), these classes carry the same fields, defaults and
refusals so jobs and tests can be written the same way:

* :class:`PMLSpec`, :class:`Grid`            -- core/pml.py:25-50, core/grid.py:28-150
* :class:`Medium`                            -- medium.py:23-106
* :class:`CWSource`, :func:`ramp_envelope`   -- sources.py:26-102
* :class:`CWRunSpec`, :class:`SolverResult`,
  :class:`SolverCaps`, the errors,
  :func:`check_source_clears_pml`            -- solvers/base.py:30-212
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any

import numpy as np


class SolverCapabilityError(ValueError):
    """A setup asked a solver for something it declares it cannot do (base.py:30-31)."""


class SolverDivergedError(RuntimeError):
    """The field stopped being a number (base.py:34-41)."""


@dataclass(frozen=True)
class PMLSpec:
    """Sponge thickness [m] and Gaussian edge factor (core/pml.py:25-50)."""

    thickness: float
    edge: float = 2.0

    def __post_init__(self) -> None:
        if self.thickness < 0:
            raise ValueError(f"PML thickness must be >= 0, got {self.thickness}")
        if self.edge <= 0:
            raise ValueError(f"PML edge factor must be > 0, got {self.edge}")

    def thickness_vox(self, dx: float) -> int:
        if dx <= 0:
            raise ValueError(f"dx must be > 0, got {dx}")
        return int(round(self.thickness / dx))


class Grid:
    """Isotropic 1/2/3-D grid (core/grid.py:28-150; geometry only)."""

    def __init__(self, shape, dx: float, pml: PMLSpec | None = None):
        shape = tuple(int(s) for s in shape)
        if not 1 <= len(shape) <= 3:
            raise ValueError(f"Grid supports 1..3 dimensions, got shape {shape}")
        if any(s < 4 for s in shape):
            raise ValueError(f"every axis needs >= 4 voxels, got shape {shape}")
        if not (np.isfinite(dx) and dx > 0):
            raise ValueError(f"dx must be a positive finite number in meters, got {dx}")
        self.shape = shape
        self.dx = float(dx)
        self.pml = pml

    @property
    def ndim(self) -> int:
        return len(self.shape)

    @property
    def pml_vox(self) -> int:
        return 0 if self.pml is None else self.pml.thickness_vox(self.dx)

    def __repr__(self) -> str:  # pragma: no cover - cosmetic
        return f"Grid(shape={self.shape}, dx={self.dx * 1e3:.3g} mm, pml={self.pml_vox}vox)"


class Medium:
    """Four float32 property volumes alpha [Np/m], rho, c, beta (medium.py:23-106)."""

    def __init__(self, alpha, rho, c, beta, id_map=None):
        vols = {"alpha": alpha, "rho": rho, "c": c, "beta": beta}
        shapes = {k: np.shape(v) for k, v in vols.items()}
        if len(set(shapes.values())) != 1:
            raise ValueError(f"property volumes disagree in shape: {shapes}")
        for k, v in vols.items():
            setattr(self, k, np.ascontiguousarray(v, dtype=np.float32))
        if id_map is not None and np.shape(id_map) != self.alpha.shape:
            raise ValueError(f"id_map shape {np.shape(id_map)} != property shape {self.alpha.shape}")
        self.id_map = id_map

    @classmethod
    def homogeneous(cls, shape, *, alpha_np_m: float = 0.0, rho: float = 1000.0, c: float = 1500.0,
                    beta: float = 0.0) -> Medium:
        full = np.full(shape, 1.0, dtype=np.float32)
        return cls(alpha=full * alpha_np_m, rho=full * rho, c=full * c, beta=full * beta)

    @classmethod
    def from_labels(cls, id_map, table: dict[int, tuple[float, float, float, float]]) -> Medium:
        """Dense volumes from an integer id map and ``{id: (alpha, rho, c, beta)}``
        (the shape of ``Medium.from_id_map``, medium.py:57-81)."""
        id_map = np.asarray(id_map)
        small = id_map.dtype.kind in "iu" and id_map.size > 0 and 0 <= int(id_map.min()) and int(id_map.max()) < 65536
        if small:  # one gather per property through a lookup table
            present = np.flatnonzero(np.bincount(id_map.reshape(-1)))
        else:
            present = np.unique(id_map)
        unknown = [int(i) for i in present if int(i) not in table]
        if unknown:
            raise ValueError(f"id_map contains ids {unknown} that are missing from the table")
        if small:
            lut = np.zeros((int(present[-1]) + 1, 4), np.float32)
            for i in present:
                lut[int(i)] = np.asarray(table[int(i)], np.float32)
            out = [np.ascontiguousarray(lut[:, k])[id_map] for k in range(4)]
            med = cls(*out, id_map=id_map)
            lo, hi = int(present[0]), int(present[-1])
            if hi - lo < 256:
                # the label decomposition the solver needs, known by construction:
                # labels id - lo and one row per id (absent ids repeat the first
                # present row), kept with read-only maps so it stays true
                rows = lut[lo:hi + 1].copy()
                absent = np.setdiff1d(np.arange(lo, hi + 1), present) - lo
                rows[absent] = rows[0]
                labels = (id_map - lo).astype(np.uint8) if lo else id_map.astype(np.uint8)
                maps = (med.alpha, med.rho, med.c, med.beta)
                for m in (*maps, labels, rows):
                    m.setflags(write=False)
                med._label_cache = (maps, labels, rows)
            return med
        out = [np.zeros(id_map.shape, np.float32) for _ in range(4)]
        for i in present:
            mask = id_map == i
            for arr, val in zip(out, table[int(i)], strict=True):
                arr[mask] = val
        return cls(*out, id_map=id_map)

    @property
    def shape(self):
        return self.alpha.shape

    @property
    def c_min(self) -> float:
        return float(self.c.min())

    @property
    def c_max(self) -> float:
        return float(self.c.max())

    @property
    def is_linear(self) -> bool:
        return bool((self.beta == 0).all())


def ramp_envelope(t: float, period: float, ramp_periods: float) -> float:
    """Cosine taper 0 -> 1 over ``ramp_periods`` periods (sources.py:98-102)."""
    t_ramp = ramp_periods * period
    x = min(t / t_ramp, 1.0)
    return 0.5 * (1.0 - np.cos(np.pi * x))


@dataclass(frozen=True)
class CWSource:
    """CW multi-voxel pressure source (sources.py:26-96)."""

    indices: np.ndarray
    phases: np.ndarray
    amplitude: float
    f0: float
    ramp_periods: float = 3.0
    label: str = field(default="", compare=False)

    def __post_init__(self) -> None:
        idx = np.asarray(self.indices)
        ph = self.phases
        if not isinstance(ph, np.ndarray) and (hasattr(ph, "__cuda_array_interface__") or
                                                hasattr(ph, "__dlpack_device__")):
            from .device import is_device_array, to_host

            if is_device_array(ph):  # device phases: a few KB read back
                ph = to_host(ph, np.float32)
        ph = np.asarray(ph, dtype=np.float32)
        if idx.ndim != 2:
            raise ValueError(f"indices must be (n, ndim), got shape {idx.shape}")
        if not np.issubdtype(idx.dtype, np.integer):
            raise TypeError(f"indices must be integer voxel coords, got {idx.dtype}")
        if ph.shape != (idx.shape[0],):
            raise ValueError(f"phases must be ({idx.shape[0]},), got {ph.shape}")
        if self.amplitude <= 0 or self.f0 <= 0:
            raise ValueError("amplitude and f0 must be > 0")
        if self.ramp_periods <= 0:
            raise ValueError("ramp_periods must be > 0")
        if np.unique(idx, axis=0).shape[0] != idx.shape[0]:
            raise ValueError("source contains duplicate voxel indices; deduplicate (and decide the phase) "
                             "before constructing the CWSource.")
        object.__setattr__(self, "indices", np.ascontiguousarray(idx.astype(np.int64)))
        object.__setattr__(self, "phases", np.ascontiguousarray(ph))

    @property
    def n_points(self) -> int:
        return int(self.indices.shape[0])

    @property
    def ndim(self) -> int:
        return int(self.indices.shape[1])

    def check_inside(self, grid) -> None:
        if self.ndim != grid.ndim:
            raise ValueError(f"source is {self.ndim}-D but grid is {grid.ndim}-D")
        upper = np.asarray(grid.shape)
        if (self.indices < 0).any() or (self.indices >= upper).any():
            bad = np.where((self.indices < 0).any(1) | (self.indices >= upper).any(1))[0]
            raise ValueError(f"{bad.size} source voxel(s) fall outside grid {grid.shape} "
                             f"(first offender: {self.indices[bad[0]].tolist()})")


@dataclass
class CWRunSpec:
    """Steady-state run policy with the reference defaults (base.py:55-82)."""

    cfl: float = 0.48
    cfl_hard_max: float = 0.50
    min_settle_periods: int = 8
    max_settle_periods: int = 96
    convergence_tol: float = 0.01
    n_record_periods: int = 2
    t_end_min_us: float | None = None

    def __post_init__(self) -> None:
        if not (0.0 < self.cfl <= 0.6 and 0.0 < self.cfl_hard_max <= 0.6):
            raise ValueError("cfl and cfl_hard_max must lie in (0, 0.6]")
        if self.min_settle_periods < 0 or self.max_settle_periods < 1 or self.n_record_periods < 1:
            raise ValueError("settle/record period counts out of range")
        if self.convergence_tol < 0:
            raise ValueError("convergence_tol must be >= 0")
        if self.t_end_min_us is not None and self.t_end_min_us <= 0:
            raise ValueError("t_end_min_us must be > 0")
        if self.max_settle_periods < self.min_settle_periods:
            raise ValueError(f"max_settle_periods ({self.max_settle_periods}) < "
                             f"min_settle_periods ({self.min_settle_periods})")
        if self.cfl > self.cfl_hard_max:
            raise ValueError(f"cfl ({self.cfl}) exceeds cfl_hard_max ({self.cfl_hard_max})")

    def model_dump(self) -> dict:
        return dict(self.__dict__)


@dataclass(frozen=True)
class SolverCaps:
    """What a solver supports (base.py:44-52)."""

    ndim: frozenset
    nonlinear: bool
    drive: frozenset
    backends: frozenset
    absorption: frozenset = frozenset({"exponential"})


@dataclass
class SolverResult:
    """Steady-state CW result over ``region`` of the active grid (base.py:85-120)."""

    phasor: np.ndarray
    p_max: np.ndarray
    region: tuple
    dt: float
    spp: int
    steps_total: int
    t_end_s: float
    tof_periods: int
    converged_period: int
    settle_capped: bool
    convergence_history: list
    phasors: dict = field(default_factory=dict)
    meta: dict[str, Any] = field(default_factory=dict)

    @property
    def amp(self) -> np.ndarray:
        return np.abs(self.phasor).astype(np.float32)

    @property
    def phase(self) -> np.ndarray:
        return np.angle(self.phasor).astype(np.float32)

    def harmonic_amp(self, n: int) -> np.ndarray:
        if n not in self.phasors:
            raise KeyError(f"harmonic {n} was not recorded (available: {sorted(self.phasors)}); "
                           f"pass harmonics=(1, {n}) to run().")
        return np.abs(self.phasors[n]).astype(np.float32)


def check_source_clears_pml(grid, source) -> None:
    """Refuse a source lying entirely inside the sponge band (base.py:132-169)."""
    band = grid.pml_vox
    if band <= 0 or any(n <= 2 * band for n in grid.shape):
        return
    idx = source.indices
    upper = np.asarray(grid.shape) - band
    interior = ((idx >= band) & (idx < upper)).all(axis=1)
    if interior.any():
        return
    lo = tuple(int(v) for v in idx.min(axis=0))
    hi = tuple(int(v) for v in idx.max(axis=0))
    raise SolverCapabilityError(
        f"every source voxel (span {lo}..{hi}) lies inside the PML band ({band} voxels on each face of "
        f"{grid.shape}), where it is damped as fast as it is driven. Move the source inward, thin the "
        f"PML, or enlarge the grid."
    )


def validate_setup(name: str, caps: SolverCaps, grid, medium, source) -> None:
    """``SolverBase.validate`` (base.py:178-201)."""
    if grid.ndim not in caps.ndim:
        raise SolverCapabilityError(f"solver '{name}' supports {sorted(caps.ndim)}-D grids, got {grid.ndim}-D.")
    if tuple(medium.shape) != tuple(grid.shape):
        raise ValueError(f"medium shape {medium.shape} != grid shape {grid.shape}")
    if not medium.is_linear and not caps.nonlinear:
        raise SolverCapabilityError(
            f"solver '{name}' is linear-only but the medium has beta != 0. Zero the medium's beta or pick a "
            f"nonlinear solver (e.g. 'westervelt_gb300')."
        )
    if "cw" not in caps.drive:
        raise SolverCapabilityError(f"solver '{name}' does not support CW drive.")
    source.check_inside(grid)
    check_source_clears_pml(grid, source)

"""Shared pytest configuration: the ``gpu`` marker and fixture helpers."""

from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def reference_src() -> Path | None:
    """Source tree of the reference package (the directory holding ``caustica/``).

    Taken from ``CAUSTICA_REFERENCE_SRC``, else a ``reference/src`` checkout
    beside this repository; None when neither exists (tests that need the
    reference then skip; the GPU tests never do).
    """
    cands = [os.environ.get("CAUSTICA_REFERENCE_SRC"), ROOT.parent / "reference" / "src"]
    for cand in cands:
        if cand and (Path(cand) / "caustica" / "__init__.py").exists():
            return Path(cand)
    return None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")


def load_golden(name: str) -> dict:
    """Load one committed fixture as a plain dict (JSON fields decoded)."""
    with np.load(GOLDEN / f"{name}.npz", allow_pickle=False) as z:
        out = {k: z[k] for k in z.files}
    for key in ("spec", "record_region", "reference_point", "reference_temperature_c"):
        if key in out:
            out[key] = json.loads(str(out[key]))
    for key, val in list(out.items()):
        if isinstance(val, np.ndarray) and val.ndim == 0 and val.dtype.kind in "fiub":
            out[key] = val.item()
        elif isinstance(val, np.ndarray) and val.ndim == 0 and val.dtype.kind == "U":
            out[key] = str(val)
    return out


def golden_kspace_kwargs(g: dict) -> dict:
    """Oracle/solver keyword arguments reconstructed from a k-space fixture."""
    rr = g["record_region"]
    spec = dict(g["spec"])
    return dict(
        shape=tuple(int(s) for s in g["shape"]),
        dx=float(g["dx"]),
        pml_vox_n=int(g["pml_vox"]),
        pml_edge=float(g["pml_edge"]),
        alpha=g["alpha"], rho=g["rho"], c=g["c"], beta=g["beta"],
        src_idx=g["src_idx"], src_phase=g["src_phase"],
        amplitude=float(g["amplitude"]), f0=float(g["f0"]), ramp_periods=float(g["ramp_periods"]),
        nonlinear=bool(g["nonlinear"]),
        harmonics=tuple(int(h) for h in np.atleast_1d(g["harmonics"])),
        record_region=None if rr is None else tuple(slice(a, b) for a, b in rr),
        reference_point=None if g["reference_point"] is None else tuple(g["reference_point"]),
        cfl=spec.get("cfl", 0.48),
        cfl_hard_max=spec.get("cfl_hard_max", 0.50),
        min_settle_periods=spec.get("min_settle_periods", 8),
        max_settle_periods=spec.get("max_settle_periods", 96),
        convergence_tol=spec.get("convergence_tol", 0.01),
        n_record_periods=spec.get("n_record_periods", 2),
        t_end_min_us=spec.get("t_end_min_us"),
    )


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.complex128)
    b = np.asarray(b, np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


KSPACE_GOLDEN = [
    "ks3d_linear_hetero",
    "ks3d_westervelt_padded",
    "ks1d_plane_converge",
    "ks2d_westervelt",
]
PENNES_GOLDEN = ["pennes3d_insulated", "pennes2d_dirichlet_substep"]


@pytest.fixture
def golden():
    return load_golden


FOCUS_GOLDEN = ["focus_h2_target", "focus_truncated"]


def focus_case(name: str):
    """A committed focal-metrics fixture as (SolverResult mirror, frame kwargs, medium or None, golden dict)."""
    from types import SimpleNamespace

    from caustica_gb300.contract import SolverResult

    g = load_golden(name)
    org = tuple(int(v) for v in g["origin"])
    p1 = g["p1"]
    phasors = {1: p1}
    if "p2" in g:
        phasors[2] = g["p2"]
    region = tuple(slice(o, o + n) for o, n in zip(org, p1.shape))
    res = SolverResult(phasor=p1, p_max=g["pmax"], region=region, dt=2.5e-8, spp=40, steps_total=1200,
                       t_end_s=3.0e-5, tof_periods=12, converged_period=26, settle_capped=False,
                       convergence_history=[], phasors=phasors, meta={"solver": "westervelt"})
    focus = tuple(int(v) for v in g["focus"])
    frame = dict(dx=float(g["dx"]), grid_shape=tuple(int(v) for v in g["grid_shape"]), pml_vox=int(g["pml_vox"]),
                 apex_vox=tuple(int(v) for v in g["apex"]), focus_vox=None if focus[0] < 0 else focus)
    med = SimpleNamespace(rho=g["rho"], c=g["c"]) if "rho" in g else None
    return res, frame, med, json.loads(g["metrics"])

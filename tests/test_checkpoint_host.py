"""Checkpoint container and refusals on the host (no GPU).

The run fingerprint and the ``caustica-checkpoint/1`` container follow the
reference (io/checkpoint.py:120-226, solvers/kspace/engine.py:303-334). A
checkpoint written by a different run, or in another format, is refused
with ``CheckpointMismatch`` before any device memory is taken, so these
tests run the real solver front without a GPU.
"""

from __future__ import annotations

import json

import numpy as np
import pytest

import caustica_gb300 as cg
from caustica_gb300 import checkpoint as ckpt
from caustica_gb300.engine import make_plan

F0, C0 = 1.0e6, 1500.0


def _setup(amplitude=1e5, reference_point=None):
    dx = C0 / (F0 * 4.0)
    grid = cg.Grid((96,), dx, cg.PMLSpec(12 * dx))
    med = cg.Medium.homogeneous(grid.shape, alpha_np_m=0.0253, rho=1000.0, c=C0)
    src = cg.CWSource(indices=np.array([[18]]), phases=np.zeros(1, np.float32), amplitude=amplitude, f0=F0)
    spec = cg.CWRunSpec(min_settle_periods=10, max_settle_periods=24)
    plan = make_plan("linear_gb300", grid, med, src, spec, reference_point=reference_point)
    return grid, med, src, spec, plan


def _write_for(path, plan, grid, med, src, fmt=None):
    fp = ckpt.fingerprint(plan, grid, med, src)
    fields = {"p": np.zeros(plan.padded, np.float32), "u0": np.zeros(plan.padded, np.float32)}
    ckpt.write(path, stage="settle", n=3 * plan.spp, periods_done=3, prev_peak=1.0, converged=False,
               converged_period=plan.eff_max, history=[(3, 1.0, 0.5)], fields=fields, fp=fp)
    if fmt is not None:
        with np.load(path, allow_pickle=False) as z:
            payload = {k: z[k] for k in z.files}
        meta = json.loads(str(payload["meta_json"]))
        meta["format"] = fmt
        payload["meta_json"] = np.asarray(json.dumps(meta))
        with open(path, "wb") as fh:
            np.savez(fh, **payload)
    return fp


def test_a_checkpoint_of_another_run_is_refused_with_the_differing_keys(tmp_path):
    path = tmp_path / "other.ckpt.npz"
    grid, med, src, spec, plan = _setup(amplitude=1e5)
    _write_for(path, plan, grid, med, src)
    grid2, med2, src2, spec2, _ = _setup(amplitude=2e5)
    with pytest.raises(cg.CheckpointMismatch) as exc:
        cg.LinearKSpaceGB300().run(grid2, med2, src2, spec2, checkpoint=cg.CheckpointSpec(path=path))
    msg = str(exc.value)
    assert "DIFFERENT run" in msg and "amplitude" in msg
    assert path.exists()  # a refused checkpoint is left as it was


def test_a_checkpoint_in_another_format_is_refused(tmp_path):
    path = tmp_path / "fmt.ckpt.npz"
    grid, med, src, spec, plan = _setup()
    _write_for(path, plan, grid, med, src, fmt="caustica-checkpoint/0")
    with pytest.raises(cg.CheckpointMismatch, match="format"):
        cg.LinearKSpaceGB300().run(grid, med, src, spec, checkpoint=cg.CheckpointSpec(path=path))


def test_the_container_round_trips_state_and_bookkeeping(tmp_path):
    path = tmp_path / "rt.ckpt.npz"
    grid, med, src, spec, plan = _setup()
    fp = _write_for(path, plan, grid, med, src)
    state = ckpt.load(path, fp)
    assert state["stage"] == "settle" and state["periods_done"] == 3 and state["n"] == 3 * plan.spp
    assert state["history"] == [(3, 1.0, 0.5)]
    assert set(state["fields"]) == {"p", "u0"}
    with np.load(path, allow_pickle=False) as z:  # the reference's container layout
        meta = json.loads(str(z["meta_json"]))
        assert meta["format"] == "caustica-checkpoint/1"
        assert z["history"].shape == (1, 3) and z["history"].dtype == np.float64
    assert not list(tmp_path.glob("*.tmp"))  # atomic write leaves no temporary behind


def test_the_fingerprint_covers_what_shapes_the_trajectory():
    grid, med, src, spec, plan = _setup()
    base = ckpt.fingerprint(plan, grid, med, src)
    assert base["scheme"] == "cw-kspace-gb300/1"
    for change in (dict(amplitude=3e5), dict(reference_point=(60,))):
        g2, m2, s2, _, p2 = _setup(**change)
        other = ckpt.fingerprint(p2, g2, m2, s2)
        assert other != base, change
    src2 = cg.CWSource(indices=src.indices, phases=np.full(1, 0.5, np.float32), amplitude=src.amplitude, f0=F0)
    assert ckpt.fingerprint(plan, grid, med, src2)["source_sha1"] != base["source_sha1"]


def test_every_periods_must_be_positive(tmp_path):
    with pytest.raises(ValueError):
        cg.CheckpointSpec(path=tmp_path / "x.npz", every_periods=0)

"""The drop-in boundary seen from the reference's side (no GPU).

With the reference package importable, the GB300 solvers must reach
caustica through its own doors:

* the ``caustica.solvers`` entry-point group (registry.py:112-244,
  solvers/registry.py:26-52) resolves ``linear_gb300`` / ``westervelt_gb300``
  to the classes of ``caustica_gb300.plugin``;
* ``install_compat()`` puts both names in the runner's and the facade's
  native-solver whitelists (runner.py:111, facade.py:68) and lets the
  planner's ``estimate`` (planner/__init__.py:307) model them with the
  inventory of their reference counterparts;
* a ``caustica-job/1`` document naming ``westervelt_gb300`` parses and builds
  through ``config.build_job`` and passes the solver's own ``validate``.

Each check runs in a fresh interpreter: the registry scans its entry-point
group once per process, and the package is made visible to
``importlib.metadata`` through a ``.dist-info`` folder holding this
project's entry points (what ``pip install`` would write). h5py, which only
the result store needs, is replaced by an empty module when absent.
"""

from __future__ import annotations

import os
import subprocess
import sys
import textwrap
import tomllib
from pathlib import Path

import pytest

from conftest import ROOT, reference_src

REF = reference_src()
pytestmark = pytest.mark.skipif(REF is None, reason="reference sources not present (set CAUSTICA_REFERENCE_SRC)")


def _dist_info(tmp_path: Path) -> Path:
    meta = tomllib.loads((ROOT / "pyproject.toml").read_text())
    eps = meta["project"]["entry-points"]["caustica.solvers"]
    site = tmp_path / "site"
    d = site / "caustica_gb300-0.1.0.dist-info"
    d.mkdir(parents=True)
    (d / "METADATA").write_text("Metadata-Version: 2.1\nName: caustica-gb300\nVersion: 0.1.0\n")
    lines = ["[caustica.solvers]"] + [f"{k} = {v}" for k, v in eps.items()]
    (d / "entry_points.txt").write_text("\n".join(lines) + "\n")
    return site


PRELUDE = """
import sys, types
try:
    import h5py  # noqa: F401
except ImportError:
    sys.modules["h5py"] = types.ModuleType("h5py")
"""


def _run(tmp_path: Path, body: str) -> str:
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([str(_dist_info(tmp_path)), str(REF), str(ROOT)])
    code = PRELUDE + textwrap.dedent(body)
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, f"stdout:\n{r.stdout}\nstderr:\n{r.stderr}"
    return r.stdout


def test_the_entry_point_group_resolves_both_solvers(tmp_path):
    out = _run(tmp_path, """
        import caustica.solvers as solvers
        from caustica.solvers.base import SolverBase
        import caustica_gb300.plugin as plugin
        assert "linear_gb300" in solvers.available() and "westervelt_gb300" in solvers.available()
        assert solvers.get("linear_gb300") is plugin.LinearKSpaceGB300
        assert solvers.get("westervelt_gb300") is plugin.WesterveltKSpaceGB300
        assert issubclass(solvers.get("westervelt_gb300"), SolverBase)
        assert solvers.get("westervelt_gb300").caps.nonlinear is True
        # the reference's own solvers are untouched
        assert solvers.get("linear").__module__.startswith("caustica.")
        print("ok")
    """)
    assert out.strip().endswith("ok")


def test_install_compat_whitelists_the_names_and_plans_them(tmp_path):
    out = _run(tmp_path, """
        import numpy as np
        import caustica.facade as facade
        import caustica.planner as planner
        import caustica.runner as runner
        from caustica import Grid, Medium, PMLSpec
        from caustica.materials import water
        from caustica.solvers import CWRunSpec
        from caustica.sources import CWSource
        from caustica_gb300.plugin import install_compat

        install_compat()
        install_compat()  # idempotent
        for mod in (runner, facade):
            names = mod._NATIVE_SOLVERS
            assert "linear_gb300" in names and "westervelt_gb300" in names, names
            assert len(names) == len(set(names))
        grid = Grid((64, 64, 80), 0.25e-3, PMLSpec(2.5e-3))
        med = Medium.homogeneous(grid.shape, water(beta=3.5))
        src = CWSource(indices=np.array([[32, 32, 12], [33, 32, 12]]), phases=np.zeros(2, np.float32),
                       amplitude=1e5, f0=1e6)
        spec = CWRunSpec()
        mine = planner.estimate(grid, med, src, spec, solver="westervelt_gb300", harmonics=(1, 2))
        ref = planner.estimate(grid, med, src, spec, solver="westervelt", harmonics=(1, 2))
        assert mine.solver == "westervelt_gb300" and ref.solver == "westervelt"
        assert mine.vram_bytes == ref.vram_bytes and mine.vram_breakdown == ref.vram_breakdown
        assert mine.spp == ref.spp and mine.dt == ref.dt
        assert (mine.steps_expected, mine.steps_worst) == (ref.steps_expected, ref.steps_worst)
        lin = planner.estimate(grid, med, src, spec, solver="linear_gb300")
        ref_lin = planner.estimate(grid, med, src, spec, solver="linear")
        assert lin.solver == "linear_gb300" and lin.vram_bytes == ref_lin.vram_bytes
        # the runner reads the planner through its own module binding
        if hasattr(runner, "estimate"):
            assert runner.estimate is planner.estimate
        print("ok")
    """)
    assert out.strip().endswith("ok")


JOB = {
    "format": "caustica-job/1",
    "kind": "explicit",
    "name": "gb300-job",
    "medium": {"kind": "homogeneous"},
    "grid": {"ndim": 3, "dx_mm": 0.5, "size_mm": [12.0, 12.0, 12.0], "pml": {"thickness_mm": 1.0}},
    "source": {"kind": "array", "array": {"kind": "bowl", "d_outer_mm": 4.0, "roc_mm": 5.0},
               "apex_mm": [6.0, 6.0, 3.0]},
    "drive": {"f0_mhz": 1.0, "amplitude_kpa": 100.0},
    "run": {"spec": {"min_settle_periods": 1, "max_settle_periods": 2, "n_record_periods": 1}},
    "solver": "westervelt_gb300",
    "backend": "auto",
}


def test_a_job_naming_the_gb300_solver_builds_and_validates(tmp_path):
    out = _run(tmp_path, f"""
        import caustica.solvers as solvers
        from caustica.config.job import build_job, parse_job
        import caustica_gb300.plugin as plugin

        job = parse_job({JOB!r})
        assert job.solver == "westervelt_gb300"
        built = build_job(job)
        assert built.solver == "westervelt_gb300"
        cls = solvers.get(built.solver)
        assert cls is plugin.WesterveltKSpaceGB300
        src = getattr(built, "source")
        cls().validate(built.grid, built.medium, src)
        # the run() front refuses unknown options before touching the device
        try:
            cls().run(built.grid, built.medium, src, bogus=1)
        except TypeError as exc:
            assert "bogus" in str(exc)
        else:
            raise AssertionError("unknown run() option accepted")
        print("ok")
    """)
    assert out.strip().endswith("ok")

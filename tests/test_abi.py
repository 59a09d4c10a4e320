"""The C-ABI library builds, loads and exports every symbol the header declares (CPU only)."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

from caustica_gb300 import _lib
from caustica_gb300 import build as builder

HEADER = Path(__file__).resolve().parent.parent / "include" / "caustica_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+char\s*\*|int|void)\s+(cg_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    builder.build()
    return _lib.load()


def test_header_declares_the_solver_fft_and_thermal_entry_points():
    names = declared_functions()
    for must in ("cg_solver_create", "cg_solver_run_periods", "cg_solver_finalize", "cg_fft3d_forward",
                 "cg_pennes_run", "cg_last_error"):
        assert must in names


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"declared in the header but not exported: {missing}"


def test_binding_table_covers_the_header():
    assert set(declared_functions()) <= set(_lib.SIGNATURES)


def test_version_and_error_string_need_no_gpu(lib):
    assert lib.cg_version() == 10000
    assert isinstance(lib.cg_last_error(), bytes)


def test_invalid_config_is_refused_before_touching_the_device(lib):
    cfg = _lib.SolverConfig()
    cfg.nx, cfg.ny, cfg.nz = 7, 8, 8  # 7 is not 2/3/5-smooth
    cfg.batch, cfg.spp, cfg.max_periods, cfg.n_harmonics = 1, 10, 4, 1
    cfg.harmonics[0] = 1
    for i in range(3):
        cfg.rec_hi[i] = 1
    h = ctypes.c_void_p()
    rc = lib.cg_solver_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc == _lib.CG_ERR_INVALID
    assert b"2/3/5-smooth" in lib.cg_last_error()


def test_library_is_built_for_sm_103a_only():
    assert "-gencode=arch=compute_103a,code=sm_103a" in builder.ARCH

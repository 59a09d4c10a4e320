"""Result store, host side (no GPU): the quantisation oracle pinned to the
reference, the ``caustica-result/1`` writer against the reference's own
writer, argument refusals before any device call.

The writer tests pass the quantised fields in (from the oracle), so the file
layout is checked here; the device quantisation itself is a GPU test.
"""

from __future__ import annotations

import ctypes
import importlib
import sys
from pathlib import Path

import numpy as np
import pytest

import h5stub
from caustica_gb300 import _lib, store
from caustica_gb300.contract import CWSource, SolverResult
from conftest import GOLDEN, reference_src
from oracle import quantize as oq

REF = reference_src()


def golden_cases():
    z = np.load(GOLDEN / "quantize_cases.npz")
    for name in z["names"]:
        name = str(name)
        yield name, {k.split("__", 1)[1]: z[k] for k in z.files if k.startswith(name + "__")}


def bits(a: np.ndarray) -> np.ndarray:
    return a.view(np.uint16 if a.dtype == np.float16 else np.uint32)


@pytest.mark.parametrize("name,case", list(golden_cases()), ids=[n for n, _ in golden_cases()])
def test_oracle_equals_the_reference_fixture(name, case):
    with np.errstate(invalid="ignore"):
        q = oq.try_float16(case["x"], float(case["bound"]))
    assert q.dtype_name == str(case["dtype"])
    assert np.array_equal(bits(np.asarray(q.stored)), case["stored_bits"])
    assert q.scale == float(case["scale"])
    assert q.norm_err == float(case["norm_err"])


@pytest.mark.skipif(REF is None, reason="reference sources not present")
def test_oracle_equals_the_reference_on_fresh_fields():
    sys.path.insert(0, str(REF))
    try:
        from caustica.io.quantize import try_float16
    finally:
        sys.path.remove(str(REF))
    rng = np.random.default_rng(7)
    for i in range(40):
        n = int(rng.integers(0, 5000))
        x = (rng.standard_normal(n) * 10.0 ** rng.uniform(-20, 20)).astype(np.float32)
        bound = float(rng.choice([1e-3, 1e-4, 3e-4, 1e-2]))
        a, b = oq.try_float16(x, bound), try_float16(x, bound)
        assert a.dtype_name == b.dtype_name and a.scale == b.scale and a.norm_err == b.norm_err
        assert np.array_equal(bits(np.asarray(a.stored)), bits(np.asarray(b.stored)))


def _result(harmonics=(1, 2, 3), shape=(5, 4, 6), seed=3) -> SolverResult:
    rng = np.random.default_rng(seed)
    phasors = {h: (rng.normal(0, 1e5 / h, shape) + 1j * rng.normal(0, 1e5 / h, shape)).astype(np.complex64)
               for h in harmonics}
    p_max = np.abs(rng.normal(0, 2e5, shape)).astype(np.float32)
    region = (slice(2, 2 + shape[0]), slice(1, 1 + shape[1]), slice(3, 3 + shape[2]))
    return SolverResult(phasor=phasors[harmonics[0]], p_max=p_max, region=region, dt=2.5e-8, spp=40,
                        steps_total=880, t_end_s=2.2e-5, tof_periods=12, converged_period=18,
                        settle_capped=False, convergence_history=[(8, 1.0e5, 0.5), (9, 1.1e5, 0.09)],
                        phasors=phasors, meta={"solver": "westervelt_gb300", "backend": "gb300"})


def _source() -> CWSource:
    return CWSource(indices=np.array([[1, 2, 3], [1, 2, 4]]), f0=1e6, amplitude=1e6,
                    phases=np.array([0.0, 0.5]), ramp_periods=2.0, label="bowl")


def _oracle_fields(res: SolverResult, bound=1e-3) -> dict:
    return {name: store.Quantized(*oq.try_float16(f, bound)) for name, f in oq.store_order(res.phasors, res.p_max)}


def test_field_names_follow_the_store_order():
    assert store.field_names([3, 1, 2]) == ["p_real_h1", "p_imag_h1", "p_real_h2", "p_imag_h2", "p_real_h3",
                                           "p_imag_h3", "p_max"]
    res = _result()
    assert [n for n, _ in oq.store_order(res.phasors, res.p_max)] == store.field_names(res.phasors)


def _write(tmp_path, monkeypatch, res, q) -> h5stub.File:
    h5stub.install(monkeypatch)
    path = store.save_result(tmp_path / "r.h5", res, _source(), dx=1.5e-4, grid_shape=(192, 192, 256),
                             pml_vox=10, quantized=q, extra_attrs={"job_name": "cfg2"})
    assert path.exists() and not list(tmp_path.glob("*.tmp"))
    return h5stub.tree(path)


def test_writer_layout(tmp_path, monkeypatch):
    res = _result()
    q = _oracle_fields(res)
    f = _write(tmp_path, monkeypatch, res, q)
    assert f.attrs["format"] == "caustica-result/1"
    assert f.attrs["harmonics"] == [1, 2, 3]
    assert f.attrs["region_start"] == [2, 1, 3] and f.attrs["region_stop"] == [7, 5, 9]
    assert f.attrs["job_name"] == "cfg2" and f.attrs["pml_vox"] == 10
    assert sorted(f["output"].children) == sorted(store.field_names(res.phasors))
    for name, qq in q.items():
        ds = f[f"output/{name}"]
        assert ds.dtype == qq.stored.dtype and np.array_equal(bits(ds.data), bits(qq.stored))
        assert ds.attrs["scale"] == qq.scale and ds.attrs["stored_dtype"] == qq.dtype_name
        assert ds.kwargs == {"chunks": True, "compression": "gzip", "compression_opts": 4}
    assert np.array_equal(f["convergence/history"].data, np.array([[8, 1e5, 0.5], [9, 1.1e5, 0.09]]))
    assert np.array_equal(f["input/source_indices"].data, np.array([[1, 2, 3], [1, 2, 4]], np.int32))


def test_quantized_fields_attached_by_a_solve_are_used(tmp_path, monkeypatch):
    res = _result(harmonics=(1,))
    q = _oracle_fields(res)
    res.meta["quantized"] = {"max_norm_err": 1e-3, "fields": q}

    def no_device(*a, **k):
        raise AssertionError("the attached fields must be used")

    monkeypatch.setattr(store, "quantize_result", no_device)
    f = _write(tmp_path, monkeypatch, res, None)
    assert np.array_equal(f["output/p_max"].data, q["p_max"].stored)


def test_unquantized_store_keeps_float32(tmp_path, monkeypatch):
    h5stub.install(monkeypatch)
    res = _result(harmonics=(2, 1))
    path = store.save_result(tmp_path / "f.h5", res, _source(), dx=1e-4, grid_shape=(8, 8, 8), quantize=False)
    f = h5stub.tree(path)
    assert f.attrs["harmonics"] == [1, 2]
    assert f["output/p_imag_h2"].dtype == np.float32
    assert np.array_equal(f["output/p_imag_h2"].data, res.phasors[2].imag)
    assert f["output/p_imag_h2"].attrs["scale"] == 1.0


def test_failed_write_leaves_no_file(tmp_path, monkeypatch):
    m = h5stub.install(monkeypatch)

    class Broken(h5stub.File):
        def create_group(self, name):
            raise RuntimeError("disk full")

    m.File = Broken
    res = _result(harmonics=(1,))
    with pytest.raises(RuntimeError, match="disk full"):
        store.save_result(tmp_path / "x.h5", res, _source(), dx=1e-4, grid_shape=(8, 8, 8), quantized=_oracle_fields(res))
    assert list(tmp_path.iterdir()) == []


def test_writing_needs_h5py(tmp_path, monkeypatch):
    monkeypatch.setitem(sys.modules, "h5py", None)  # import h5py -> ImportError
    res = _result(harmonics=(1,))
    with pytest.raises(ImportError, match="h5py"):
        store.save_result(tmp_path / "x.h5", res, _source(), dx=1e-4, grid_shape=(8, 8, 8), quantized=_oracle_fields(res))


@pytest.mark.skipif(REF is None, reason="reference sources not present")
def test_same_file_as_the_reference_writer_and_its_reader_loads_ours(tmp_path, monkeypatch):
    h5stub.install(monkeypatch)
    monkeypatch.syspath_prepend(str(REF))
    for mod in [m for m in sys.modules if m == "caustica" or m.startswith("caustica.")]:
        monkeypatch.delitem(sys.modules, mod)
    ref_store = importlib.import_module("caustica.io.store")
    from caustica.solvers.base import SolverResult as RefResult
    from caustica.sources import CWSource as RefSource

    ours = _result()
    fields = dict(phasor=ours.phasor, p_max=ours.p_max, region=ours.region, dt=ours.dt, spp=ours.spp,
                  steps_total=ours.steps_total, t_end_s=ours.t_end_s, tof_periods=ours.tof_periods,
                  converged_period=ours.converged_period, settle_capped=ours.settle_capped,
                  convergence_history=ours.convergence_history, phasors=ours.phasors, meta=dict(ours.meta))
    ref_res = RefResult(**fields)
    src = _source()
    ref_src = RefSource(indices=src.indices, f0=src.f0, amplitude=src.amplitude, phases=src.phases,
                        ramp_periods=src.ramp_periods, label=src.label)
    kw = dict(dx=1.5e-4, grid_shape=(192, 192, 256), pml_vox=10)
    p_ref = ref_store.save_result(tmp_path / "ref.h5", ref_res, ref_src, **kw)
    p_our = store.save_result(tmp_path / "our.h5", ours, src, quantized=_oracle_fields(ours), **kw)
    a, b = h5stub.tree(p_ref), h5stub.tree(p_our)

    def walk(node, prefix=""):
        yield prefix, node
        for k, v in getattr(node, "children", {}).items():
            yield from walk(v, f"{prefix}/{k}")

    na, nb = dict(walk(a)), dict(walk(b))
    assert sorted(na) == sorted(nb)
    for key in na:
        x, y = na[key], nb[key]
        ax = {k: v for k, v in x.attrs.items() if k != "caustica_version"}
        ay = {k: v for k, v in y.attrs.items() if k != "caustica_version"}
        assert ax.keys() == ay.keys(), key
        for k in ax:
            assert np.array_equal(np.asarray(ax[k]), np.asarray(ay[k])), (key, k)
        if isinstance(x, h5stub.Dataset):
            assert x.dtype == y.dtype and np.array_equal(x.data.view(np.uint8), y.data.view(np.uint8)), key
            assert x.kwargs == y.kwargs, key
    back = ref_store.load_result(p_our)
    for h in (1, 2, 3):
        q_re, q_im = _oracle_fields(ours)[f"p_real_h{h}"], _oracle_fields(ours)[f"p_imag_h{h}"]
        assert np.array_equal(back.phasors[h].real, oq.restore(q_re.stored, q_re.scale))
        assert np.array_equal(back.phasors[h].imag, oq.restore(q_im.stored, q_im.scale))
    assert back.converged_period == 18 and back.region == ours.region


def test_argument_refusals_before_any_device_call():
    with pytest.raises(ValueError, match="complex"):
        store.quantize_arrays([np.zeros(4, np.complex64)])
    with pytest.raises(ValueError, match="max_norm_err"):
        store.quantize_arrays([np.zeros(4, np.float32)], max_norm_err=-1.0)
    with pytest.raises(ValueError, match="1 to 32"):
        store.quantize_arrays([])
    lib = _lib.load()
    info = (ctypes.c_float * 4)()
    assert lib.cg_quantize_f16(None, 1, ctypes.c_double(1e-3), None, None, info, None) == _lib.CG_ERR_INVALID
    f = (_lib.QField * 1)()
    assert lib.cg_quantize_f16(f, 0, ctypes.c_double(1e-3), None, None, info, None) == _lib.CG_ERR_INVALID
    assert b"n_fields" in lib.cg_last_error()
    f[0].n, f[0].stride = 5, 0
    assert lib.cg_quantize_f16(f, 1, ctypes.c_double(1e-3), None, None, info, None) == _lib.CG_ERR_INVALID
    assert b"stride" in lib.cg_last_error()


def test_restore_is_the_reload_recipe():
    q = oq.try_float16(np.array([1.0, -3.5, 0.25], np.float32))
    assert np.array_equal(store.restore(q.stored, q.scale), oq.restore(q.stored, q.scale))
    assert store.Quantized(*q).restore().dtype == np.float32


@pytest.mark.skipif(REF is None, reason="reference sources not present")
def test_the_reference_result_store_saves_through_the_gb300_writer(tmp_path, monkeypatch):
    h5stub.install(monkeypatch)
    monkeypatch.syspath_prepend(str(REF))
    for mod in [m for m in sys.modules if m == "caustica" or m.startswith("caustica.") or m == "caustica_gb300.plugin"]:
        monkeypatch.delitem(sys.modules, mod)
    plugin = importlib.import_module("caustica_gb300.plugin")
    rs = plugin.result_store(tmp_path / "results")
    res = _result()
    q = _oracle_fields(res)
    path = rs.save("cfg2_a", res, _source(), dx=1.5e-4, grid_shape=(192, 192, 256), quantized=q)
    assert path == rs.path("cfg2_a") and rs.is_complete("cfg2_a")
    assert rs.completed() == ["cfg2_a"] and rs.missing(["cfg2_a", "cfg2_b"]) == ["cfg2_b"]
    back = rs.load("cfg2_a")
    assert np.array_equal(back.p_max, oq.restore(q["p_max"].stored, q["p_max"].scale))

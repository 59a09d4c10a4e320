"""Device float16 store quantisation (GPU): bit for bit against the
reference's ``try_float16`` (committed fixture) and the oracle that restates
it, on plain and strided fields, through the solver handle, and into a
``caustica-result/1`` file."""

from __future__ import annotations

import numpy as np
import pytest

import caustica_gb300 as cg
import h5stub
from caustica_gb300 import store
from caustica_gb300.batch import solve_steering
from conftest import GOLDEN
from oracle import quantize as oq

pytestmark = pytest.mark.gpu
F0, C0 = 1.0e6, 1500.0


def bits(a) -> np.ndarray:
    a = np.asarray(a)
    return a.view(np.uint16 if a.dtype == np.float16 else np.uint32)


def same(dev: store.Quantized, ref) -> None:
    assert dev.dtype_name == ref.dtype_name
    assert dev.scale == ref.scale and dev.norm_err == ref.norm_err
    assert np.asarray(dev.stored).shape == np.asarray(ref.stored).shape
    assert np.array_equal(bits(dev.stored), bits(ref.stored))


def test_reference_fixture_cases_bit_for_bit():
    z = np.load(GOLDEN / "quantize_cases.npz")
    for name in (str(n) for n in z["names"]):
        x, bound = z[f"{name}__x"], float(z[f"{name}__bound"])
        (q,) = store.quantize_arrays([x], bound)
        assert q.dtype_name == str(z[f"{name}__dtype"]), name
        assert np.array_equal(bits(q.stored), z[f"{name}__stored_bits"]), name
        assert q.scale == float(z[f"{name}__scale"]), name
        assert q.norm_err == float(z[f"{name}__norm_err"]), name


@pytest.mark.parametrize("n", [1, 31, 255, 256, 257, 4097, 1 << 20, (1 << 24) + 3])
def test_sizes_across_block_and_grid_boundaries(n):
    rng = np.random.default_rng(n)
    x = (rng.standard_normal(n) * 10.0 ** rng.uniform(-6, 6, n)).astype(np.float32)
    x[rng.integers(0, n)] = -np.abs(x).max() * 1.5  # the peak is negative and somewhere inside
    same(store.quantize_arrays([x])[0], oq.try_float16(x))


def test_many_fields_per_call_mixing_float16_and_fallbacks():
    rng = np.random.default_rng(5)
    fields = [rng.normal(0, 10.0 ** k, 1000 + 37 * k).astype(np.float32) for k in range(-3, 9)]
    fields[4][:] = 0.0
    fields[7][3] = np.nan
    fields.append(np.zeros(0, np.float32))
    for bound in (1e-3, 2.5e-4):
        got = store.quantize_arrays(fields, bound)
        with np.errstate(invalid="ignore"):
            want = [oq.try_float16(f, bound) for f in fields]
        for g, w in zip(got, want):
            same(g, w)
        assert {g.dtype_name for g in got} == {"float16", "float32"}


def test_device_inputs_are_read_in_place():
    torch = pytest.importorskip("torch")
    x = torch.randn(3, 50, 7, device="cuda", dtype=torch.float32) * 1e4
    (q,) = store.quantize_arrays([x])
    same(q, oq.try_float16(x.cpu().numpy()))
    assert q.stored.shape == (3, 50, 7)


def _tiny(beta=3.5):
    grid = cg.Grid((24, 20, 28), 0.25e-3, None)
    med = cg.Medium.homogeneous(grid.shape, alpha_np_m=0.0253, rho=1000.0, c=C0, beta=beta)
    src = cg.CWSource(indices=np.array([[12, 10, 6], [12, 11, 6]]), phases=np.zeros(2, np.float32),
                      amplitude=2e5, f0=F0)
    return grid, med, src, cg.CWRunSpec(min_settle_periods=1, max_settle_periods=3)


def test_a_solve_attaches_its_store_fields_equal_to_the_oracle_on_its_result():
    grid, med, src, spec = _tiny()
    solver = cg.WesterveltKSpaceGB300()
    solver.store_quantize = 1e-3
    res = solver.run(grid, med, src, spec, harmonics=(1, 3, 2), record_region=(slice(2, 20), slice(1, 19), slice(3, 25)))
    att = res.meta["quantized"]
    assert att["max_norm_err"] == 1e-3
    want = oq.store_order(res.phasors, res.p_max)
    assert list(att["fields"]) == [n for n, _ in want]
    for name, f in want:
        same(att["fields"][name], oq.try_float16(f))
        assert att["fields"][name].stored.shape == (18, 18, 22)
    # without the option nothing is attached
    assert "quantized" not in cg.WesterveltKSpaceGB300().run(grid, med, src, spec).meta


def test_tight_bound_through_the_handle_falls_back_to_the_float32_result():
    grid, med, src, spec = _tiny(beta=0.0)
    solver = cg.LinearKSpaceGB300()
    solver.store_quantize = 1e-6  # below float16's resolution: every non-zero field keeps float32
    res = solver.run(grid, med, src, spec)
    for name, f in oq.store_order(res.phasors, res.p_max):
        q = res.meta["quantized"]["fields"][name]
        same(q, oq.try_float16(f, 1e-6))
        assert q.dtype_name == "float32" and np.array_equal(q.stored, f)


def test_batched_members_carry_their_own_fields():
    grid, med, src, spec = _tiny(beta=0.0)
    phases = np.array([[0.0, 0.0], [0.0, 1.2], [2.0, -0.4]], np.float32)
    out = solve_steering(grid, med, src.indices, phases, f0=F0, amplitude=2e5, spec=spec, quantize=1e-3)
    for res in out:
        for name, f in oq.store_order(res.phasors, res.p_max):
            same(res.meta["quantized"]["fields"][name], oq.try_float16(f))


def test_save_result_from_a_solve_writes_the_device_fields(tmp_path, monkeypatch):
    grid, med, src, spec = _tiny()
    solver = cg.WesterveltKSpaceGB300()
    solver.store_quantize = 1e-3
    res = solver.run(grid, med, src, spec, harmonics=(1, 2))
    h5stub.install(monkeypatch)
    path = store.save_result(tmp_path / "r.h5", res, src, dx=grid.dx, grid_shape=grid.shape)
    f = h5stub.tree(path)
    for name, f32 in oq.store_order(res.phasors, res.p_max):
        ds = f[f"output/{name}"]
        ref = oq.try_float16(f32)
        assert np.array_equal(bits(ds.data), bits(ref.stored)) and ds.attrs["scale"] == ref.scale
        restored = oq.restore(ds.data, ds.attrs["scale"])
        peak = float(np.abs(f32).max())
        assert float(np.abs(restored - f32).max()) <= 1e-3 * peak
    # a host result without attached fields is quantised on the device the same way
    res.meta.pop("quantized")
    path2 = store.save_result(tmp_path / "r2.h5", res, src, dx=grid.dx, grid_shape=grid.shape)
    g = h5stub.tree(path2)
    for name, _ in oq.store_order(res.phasors, res.p_max):
        assert np.array_equal(bits(g[f"output/{name}"].data), bits(f[f"output/{name}"].data))


@pytest.mark.parametrize("shape", [(96,), (40, 36)])
def test_one_and_two_dimensional_results(shape):
    dx = C0 / (F0 * 6.0)
    grid = cg.Grid(shape, dx, cg.PMLSpec(8 * dx))
    med = cg.Medium.homogeneous(grid.shape, alpha_np_m=0.0253, rho=1000.0, c=C0, beta=3.5)
    idx = np.array([[12] + [n // 2 for n in shape[1:]]])
    src = cg.CWSource(indices=idx, phases=np.zeros(1, np.float32), amplitude=1e5, f0=F0)
    solver = cg.WesterveltKSpaceGB300()
    solver.store_quantize = 5e-4
    res = solver.run(grid, med, src, cg.CWRunSpec(min_settle_periods=2, max_settle_periods=4), harmonics=(1, 2))
    for name, f in oq.store_order(res.phasors, res.p_max):
        q = res.meta["quantized"]["fields"][name]
        same(q, oq.try_float16(f, 5e-4))
        assert q.stored.shape == res.p_max.shape

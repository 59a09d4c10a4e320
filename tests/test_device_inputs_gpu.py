"""Device-resident inputs through the Python fronts (GPU).

Label maps, steering phases, source phases, heating terms, initial
temperatures and doses may be device arrays from another framework, handed
over by ``__cuda_array_interface__`` or DLPack. Each result must equal the
one the same call gives with host NumPy inputs, bit for bit: the device
path changes where the inputs live, not the arithmetic.
"""

from __future__ import annotations

import numpy as np
import pytest

import caustica_gb300 as cg
from caustica_gb300.batch import solve_steering
from caustica_gb300.device import DeviceLabelMedium, as_device

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


class DLPackOnly:
    """Exposes a tensor through DLPack alone (no __cuda_array_interface__)."""

    def __init__(self, t):
        self._t = t

    def __dlpack__(self, stream=None):
        return self._t.__dlpack__()

    def __dlpack_device__(self):
        return self._t.__dlpack_device__()


def _case(nonlinear=True, shape=(32, 48, 64), seed=3):
    rng = np.random.default_rng(seed)
    labels = rng.integers(0, 3, shape).astype(np.uint8)
    table = {0: (0.5, 1000.0, 1500.0, 3.5 if nonlinear else 0.0), 1: (8.0, 1050.0, 1580.0, 4.7 if nonlinear else 0.0),
             2: (20.0, 1090.0, 1610.0, 4.95 if nonlinear else 0.0), 7: (1.0, 1200.0, 1900.0, 0.0)}  # 7 never occurs
    grid = cg.Grid(shape, 0.2e-3, cg.PMLSpec(0.6e-3))
    idx = np.array([[16, 24, 5], [16, 25, 5], [15, 24, 6], [17, 23, 6]], np.int64)
    phases = rng.uniform(-np.pi, np.pi, len(idx)).astype(np.float32)
    spec = cg.CWRunSpec(cfl=0.4, convergence_tol=0.0, min_settle_periods=2, max_settle_periods=3, n_record_periods=1)
    return grid, labels, table, idx, phases, spec


def _same(a, b):
    for h in a.phasors:
        np.testing.assert_array_equal(a.phasors[h], b.phasors[h])
    np.testing.assert_array_equal(a.p_max, b.p_max)
    assert a.steps_total == b.steps_total and a.dt == b.dt


@pytest.mark.parametrize("protocol", ["cuda_array_interface", "dlpack"])
def test_a_device_label_map_gives_the_host_result(protocol):
    grid, labels, table, idx, phases, spec = _case()
    host_med = cg.Medium.from_labels(labels, {k: v for k, v in table.items() if k != 7})
    src = cg.CWSource(indices=idx, phases=phases, amplitude=1.2e6, f0=1e6)
    want = cg.WesterveltKSpaceGB300().run(grid, host_med, src, spec, harmonics=(1, 2))
    t = torch.from_numpy(labels).cuda()
    dev_med = DeviceLabelMedium(t if protocol == "cuda_array_interface" else DLPackOnly(t), table)
    assert list(dev_med.present) == [0, 1, 2]  # the unused row 7 does not set the time step
    got = cg.WesterveltKSpaceGB300().run(grid, dev_med, src, spec, harmonics=(1, 2))
    _same(want, got)
    # heating from the device-labelled solve equals the host one
    q_host = cg.HeatingSource.from_result(want, host_med, grid.dx, alpha_power_law_y=1.1).q
    q_dev = cg.HeatingSource.from_result(got, dev_med, grid.dx, alpha_power_law_y=1.1).q
    np.testing.assert_array_equal(q_host, q_dev)


def test_device_phases_give_the_host_result():
    grid, labels, table, idx, phases, spec = _case(nonlinear=False)
    med = cg.Medium.from_labels(labels, {k: v for k, v in table.items() if k != 7})
    want = cg.LinearKSpaceGB300().run(grid, med, cg.CWSource(indices=idx, phases=phases, amplitude=2e5, f0=1e6), spec)
    got = cg.LinearKSpaceGB300().run(grid, med, cg.CWSource(indices=idx, phases=torch.from_numpy(phases).cuda(),
                                                            amplitude=2e5, f0=1e6), spec)
    _same(want, got)
    rng = np.random.default_rng(5)
    steer = rng.uniform(-np.pi, np.pi, (3, len(idx))).astype(np.float32)
    a = solve_steering(grid, med, idx, steer, f0=1e6, amplitude=2e5, spec=spec)
    b = solve_steering(grid, med, idx, torch.from_numpy(steer).cuda(), f0=1e6, amplitude=2e5, spec=spec)
    for x, y in zip(a, b):
        _same(x, y)


def test_device_heating_temperature_and_dose_give_the_host_result():
    shape = (10, 12, 14)
    rng = np.random.default_rng(8)
    tm = cg.ThermalMedium.homogeneous(shape, k=0.5, rho=1000.0, specific_heat=3600.0, perfusion=5e-4, dx=0.3e-3)
    q = (rng.random(shape) * 3e6).astype(np.float32)
    t0 = (37.0 + rng.random(shape)).astype(np.float32)
    d0 = (rng.random(shape) * 1e-3).astype(np.float32)
    solver = cg.PennesSolverGB300()
    want = solver.solve(t0, q, tm, dt=0.01, n_steps=25, dose=True, dose0=d0)
    got = solver.solve(torch.from_numpy(t0).cuda(), torch.from_numpy(q).cuda(), tm, dt=0.01, n_steps=25, dose=True,
                       dose0=torch.from_numpy(d0).cuda())
    np.testing.assert_array_equal(want.temperature, got.temperature)
    np.testing.assert_array_equal(want.temperature_max, got.temperature_max)
    np.testing.assert_array_equal(want.dose_cem43, got.dose_cem43)


def test_device_arrays_are_checked():
    t = torch.zeros((4, 5), dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError, match="C-contiguous"):
        as_device(t.t(), what="x")
    with pytest.raises(ValueError, match="need float64"):
        as_device(t, dtype=np.float64, what="x")
    with pytest.raises(ValueError, match="expected a device array"):
        as_device(np.zeros(3), what="x")
    lab = torch.tensor([[0, 1], [2, 9]], dtype=torch.uint8, device="cuda")
    with pytest.raises(ValueError, match=r"labels \[9\]"):
        DeviceLabelMedium(lab, {0: (0.0, 1000.0, 1500.0, 0.0), 1: (0.0, 1000.0, 1500.0, 0.0),
                                2: (0.0, 1000.0, 1500.0, 0.0)})
    v = as_device(t)
    assert v.shape == (4, 5) and v.ptr.value == t.data_ptr()

"""One and several bare steps of the fused kernels against the oracle's step (GPU)."""

from __future__ import annotations

import numpy as np
import pytest

from caustica_gb300 import contract as ct
from caustica_gb300 import engine as eng
from oracle import kspace as ok

pytestmark = pytest.mark.gpu

CASES = [((12, 10, 16), False, True), ((9, 12, 10), True, True), ((16, 16, 24), True, False), ((1, 1, 40), False, True),
         ((1, 18, 20), True, True), ((48, 40, 64), True, True),
         # every axis on the size-specialised path
         ((32, 32, 32), True, True), ((24, 48, 96), False, True), ((16, 64, 48), True, False),
         # square transverse planes: the fused cluster passes
         ((64, 64, 32), True, True), ((96, 96, 24), False, True), ((128, 128, 16), True, True),
         ((160, 160, 16), True, False), ((192, 192, 16), True, True),
         # 320-point axes on 20 threads per pencil
         ((16, 32, 320), True, True), ((8, 64, 320), False, True), ((320, 32, 16), True, True),
         ((8, 320, 24), True, False),
         # 400-point axes (20 x 20) on 20 threads per pencil
         ((16, 32, 400), True, True), ((400, 32, 16), False, True), ((8, 400, 24), True, False),
         # 512-point axes on 32 threads per pencil
         ((16, 32, 512), True, True), ((512, 32, 16), False, True), ((8, 512, 24), True, False),
         # 640-point axes (32 x 20) on 32 threads per pencil
         ((640, 32, 16), True, True), ((8, 640, 24), False, True), ((8, 32, 640), True, False),
         ((6, 34, 640), False, True),
         # persistent z-passes with a ragged last y-tile (ny even, not a multiple of 32)
         ((6, 40, 400), True, True), ((4, 18, 512), False, True), ((5, 34, 320), True, False)]
FUSED = {64, 96, 128, 160, 192}


def _setup(shape, nonlinear, hetero, seed=0):
    rng = np.random.default_rng(seed)
    if hetero:
        c = rng.uniform(1450, 1650, shape).astype(np.float32)
        rho = rng.uniform(900, 1100, shape).astype(np.float32)
        alpha = rng.uniform(0, 40, shape).astype(np.float32)
    else:
        c = np.full(shape, 1500, np.float32)
        rho = np.full(shape, 1000, np.float32)
        alpha = np.full(shape, 2.0, np.float32)
    beta = np.full(shape, 4.5 if nonlinear else 0.0, np.float32)
    nd3 = [n for n in shape if n > 1] if shape[0] == 1 else list(shape)
    gshape = tuple(nd3)
    grid = ct.Grid(gshape, 0.25e-3, ct.PMLSpec(2 * 0.25e-3))
    med = ct.Medium(alpha.reshape(gshape), rho.reshape(gshape), c.reshape(gshape), beta.reshape(gshape))
    idx = np.array([[n // 2 for n in gshape]], np.int64)
    src = ct.CWSource(indices=idx, phases=np.zeros(1, np.float32), amplitude=1e5, f0=1e6)
    spec = ct.CWRunSpec(cfl=0.3)
    plan = eng.make_plan("step", grid, med, src, spec, nonlinear=nonlinear)
    return plan, grid, med, rng


@pytest.mark.parametrize("fused", ["0", "1"])
@pytest.mark.parametrize("shape,nonlinear,hetero", CASES)
def test_steps_match_the_oracle_step(shape, nonlinear, hetero, fused, monkeypatch):
    monkeypatch.setenv("CG_FUSED_XY", fused)
    plan, grid, med, rng = _setup(shape, nonlinear, hetero)
    p0 = (rng.standard_normal(plan.padded) * 1e5).astype(np.float32)
    u0 = [(rng.standard_normal(plan.padded) * 0.05).astype(np.float32) for _ in range(plan.nd)]
    nsteps = 3
    with eng.DeviceSolver(plan) as dev:
        u3 = np.zeros((3, 1, plan.ncell), np.float32)
        for i in range(plan.nd):
            u3[3 - plan.nd + i, 0] = u0[i].reshape(-1)
        dev.set_state(p0.reshape(1, -1), u3, 0)
        # the source ramp is exactly zero at t = 0, so step 0 injects nothing
        dev.run_steps(1)
        p1, u1 = dev.get_state()
        on = fused == "1" and shape[0] == shape[1] and shape[0] in FUSED
        assert dev.launches_per_step == (4 if on else 8)
    maps = ok.medium_maps(med.alpha, med.rho, med.c, med.beta, plan.padded, plan.dt, nonlinear, np.float64)
    ks = ok.k_vectors(plan.padded, plan.dx, np.float64)
    kap = ok.kappa_sinc(ks, plan.c_max, plan.dt, np.float64)
    der = ok.spectral_derivative_factors(ks, kap, plan.padded, np.complex128)
    spg = ok.sponge_volume(plan.padded, grid.pml_vox, 2.0, np.float64)
    pr = p0.astype(np.float64)
    ur = [x.astype(np.float64) for x in u0]
    pr, ur = ok.step_fields(p=pr, u=ur, dt_over_rho=maps[0], rhoc2_dt=maps[1], absorb=maps[2], beta2_dt=maps[3],
                            sponge=spg, deriv=der, padded=plan.padded)
    gp = p1[0].reshape(plan.padded)
    assert np.abs(gp - pr).max() / np.abs(pr).max() < 2e-6
    for i in range(plan.nd):
        gu = u1[3 - plan.nd + i, 0].reshape(plan.padded)
        assert np.abs(gu - ur[i]).max() / np.abs(ur[i]).max() < 2e-6
    del nsteps


@pytest.mark.parametrize("shape,nonlinear", [((96, 96, 40), True), ((192, 192, 24), False)])
def test_fused_transverse_passes_equal_the_three_pass_chain(shape, nonlinear, monkeypatch):
    """The opt-in cluster kernels (CG_FUSED_XY=1) do the arithmetic of the y/x/y pass
    sequence: same result to rounding."""
    plan, grid, med, rng = _setup(shape, nonlinear, True, seed=3)
    p0 = (rng.standard_normal((2,) + plan.padded) * 1e5).astype(np.float32).reshape(2, -1)
    u0 = (rng.standard_normal((3, 2, plan.ncell)) * 0.05).astype(np.float32)
    out = []
    for flag in ("1", "0"):
        monkeypatch.setenv("CG_FUSED_XY", flag)
        with eng.DeviceSolver(plan, batch=2) as dev:
            assert dev.launches_per_step == (4 if flag == "1" else 8)
            dev.set_state(p0, u0, 0)
            dev.run_steps(5)
            out.append(dev.get_state())
    (pa, ua), (pb, ub) = out
    assert np.abs(pa - pb).max() / np.abs(pb).max() < 1e-6
    assert np.abs(ua - ub).max() / np.abs(ub).max() < 1e-6


def test_autotuner_picks_a_configuration_resets_the_state_and_caches_it(monkeypatch):
    monkeypatch.delenv("CG_FUSED_XY", raising=False)
    plan, grid, med, rng = _setup((96, 96, 64), True, True, seed=5)
    with eng.DeviceSolver(plan, autotune=True) as dev:
        t = dev.tuning
        # fused or not x (persistent with cp.async staging, persistent with
        # tensor-map staging, one tile per CTA)
        assert t["configurations_timed"] == 6 and not t["cached"]
        p, u = dev.get_state()
        assert not p.any() and not u.any()  # the trial steps left no trace
        dev.run_steps(30)
        pt, _ = dev.get_state()
    with eng.DeviceSolver(plan, autotune=True) as dev:
        assert dev.tuning["cached"] and dev.tuning["fused_transverse"] == t["fused_transverse"]
    with eng.DeviceSolver(plan, autotune=False) as dev:  # three-pass chain, persistent z
        dev.run_steps(30)
        pf, _ = dev.get_state()
    assert np.abs(pt - pf).max() / np.abs(pf).max() < 1e-5

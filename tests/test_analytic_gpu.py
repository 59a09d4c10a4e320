"""Analytic physics gates on the GPU solver (GPU).

The reference pins its solver to closed-form physics as well as to its own
numbers; the same gates run here through the GB300 path, with the same
setups and thresholds:

* 1-D plane wave in water (tests/test_linear_planewave.py): exact-period
  dt, phase-speed error < 0.1 %, |P| within the sampling ceiling of p_max,
  sponge reflection ripple < 3 %, absorption within 1 % of the configured
  alpha, no late-time energy growth.
* 3-D focused bowl (tests/test_linear_oneill_3d.py): focus within one voxel
  of O'Neil's on-axis maximum, axial correlation > 0.99 and -6 dB axial
  width within 5 % of O'Neil, lateral -6 dB width within 5 % and
  correlation > 0.98 of the Rayleigh integral.
* Westervelt plane wave (tests/test_westervelt.py): A2/A1 within 5 % and
  A3/A1 within 10 % of the Fubini solution before shock.

The closed forms are the published ones, written out below: O'Neil's on-axis
pressure of a spherical cap (J. Acoust. Soc. Am. 21, 1949), the Rayleigh
integral over an equal-area cap lattice, and Fubini's harmonic amplitudes
B_n = 2 J_n(n sigma) / (n sigma) with the shock distance rho c^3/(beta w p0).
"""

from __future__ import annotations

import numpy as np
import pytest

import caustica_gb300 as cg
from caustica_gb300.workloads import bowl_source, spherical_cap_points

pytestmark = pytest.mark.gpu

F0, C0 = 1.0e6, 1500.0


def _plane_source(grid, amplitude, pos):
    """A plane source on axis 0 at voxel ``pos`` (one voxel in 1-D), phase 0."""
    other = [np.arange(n) for n in grid.shape[1:]]
    mesh = np.meshgrid(*other, indexing="ij") if other else []
    n_pts = mesh[0].size if other else 1
    idx = np.empty((n_pts, len(grid.shape)), np.int64)
    idx[:, 0] = pos
    for d, m in enumerate(mesh, start=1):
        idx[:, d] = m.reshape(-1)
    return cg.CWSource(indices=idx, phases=np.zeros(n_pts, np.float32), amplitude=amplitude, f0=F0)


# ------------------------------------------------------------ plane wave --
PPW = 4.0
DX = C0 / (F0 * PPW)
K0 = 2.0 * np.pi * F0 / C0
SPAN = slice(80, 200)


def _run_1d(alpha=0.0, n=256, pml_vox=24, src_vox=40, min_settle=40, max_settle=90, tol=0.005, record=2):
    grid = cg.Grid((n,), DX, cg.PMLSpec(pml_vox * DX))
    med = cg.Medium.homogeneous(grid.shape, alpha_np_m=alpha, c=C0, rho=1000.0)
    spec = cg.CWRunSpec(min_settle_periods=min_settle, max_settle_periods=max_settle, convergence_tol=tol,
                        n_record_periods=record)
    return cg.LinearKSpaceGB300().run(grid, med, _plane_source(grid, 1.0e5, src_vox), spec)


@pytest.fixture(scope="module")
def lossless():
    return _run_1d()


def test_exact_period_dt(lossless):
    assert lossless.spp == 8
    assert lossless.dt == pytest.approx(1.0 / F0 / 8, rel=1e-12)
    assert lossless.dt * C0 / DX == pytest.approx(0.5, rel=1e-9)


def test_plane_wave_dispersion_below_0p1_percent(lossless):
    ph = lossless.phasor[SPAN]
    k_num = np.angle(ph[1:] * np.conj(ph[:-1])).mean() / DX
    assert abs(k_num - K0) / K0 < 1e-3


def test_phasor_within_the_sampling_ceiling_of_p_max(lossless):
    ratio = lossless.amp[SPAN] / lossless.p_max[SPAN]
    assert ratio.max() <= (1.0 / np.cos(np.pi / lossless.spp)) * (1 + 1e-3)
    assert ratio.min() > 0.90


def test_sponge_reflection_ripple_below_3_percent(lossless):
    amp = lossless.amp[SPAN]
    assert (amp.max() - amp.min()) / (amp.max() + amp.min()) < 0.03


def test_convergence_metadata(lossless):
    assert lossless.tof_periods >= 50
    assert lossless.converged_period >= lossless.tof_periods
    assert not lossless.settle_capped
    assert lossless.steps_total == (lossless.converged_period + 2) * lossless.spp


def test_absorption_within_1_percent_of_alpha():
    alpha = 30.0
    res = _run_1d(alpha=alpha, pml_vox=32, n=288, min_settle=45, max_settle=95)
    x = np.arange(*SPAN.indices(288)) * DX
    slope = np.polyfit(x, np.log(res.amp[SPAN]), 1)[0]
    assert abs(-slope - alpha) / alpha < 0.01


def test_long_run_has_no_energy_growth():
    res = _run_1d(min_settle=200, max_settle=200, tol=0.0)
    hist = np.array([pk for (_p, pk, _r) in res.convergence_history])
    periods = np.array([p for (p, _pk, _r) in res.convergence_history])
    late = hist[periods >= periods.max() - 100]
    assert res.settle_capped
    assert (late.max() - late.min()) / late.mean() < 0.01


# ------------------------------------------------------ O'Neil / Rayleigh --
ODX = 0.375e-3
A_AP, ROC = 7.5e-3, 18e-3
APEX = (40, 40, 16)
SHAPE = (80, 80, 120)
FOCUS_VOX = (40, 40, 16 + 48)


def oneill_axial(z, a, roc, f0, c0=C0):
    """|p(z)| / (rho c u0) on the axis of a spherical cap (O'Neil 1949).

    p(z) = rho c u0 / (1 - z/R) (e^{ikz} - e^{ik r_e(z)}), r_e = sqrt(a^2 + (z - h)^2),
    h = R - sqrt(R^2 - a^2); at z = R the limit is -i k h e^{ikR}.
    """
    k = 2.0 * np.pi * f0 / c0
    h = roc - np.sqrt(roc ** 2 - a ** 2)
    z = np.asarray(z, np.float64)
    r_e = np.sqrt(a ** 2 + (z - h) ** 2)
    den = 1.0 - z / roc
    at_focus = np.abs(den) < 1e-12
    p = (np.exp(1j * k * z) - np.exp(1j * k * r_e)) / np.where(at_focus, 1.0, den)
    return np.abs(np.where(at_focus, -1j * k * h * np.exp(1j * k * roc), p))


def rayleigh_abs(points, targets, f0, c0=C0):
    """|sum_j e^{ikR_j} / R_j| over an equal-area lattice (the Rayleigh integral up to a constant)."""
    k = 2.0 * np.pi * f0 / c0
    out = np.empty(len(targets), np.complex128)
    for i, t in enumerate(targets):
        r = np.linalg.norm(points - t, axis=1)
        out[i] = np.sum(np.exp(1j * k * r) / r)
    return np.abs(out)


def minus6db_width(coord, prof):
    prof = np.asarray(prof, np.float64)
    i_pk = int(np.argmax(prof))
    half = prof[i_pk] / 2.0
    lo = i_pk
    while lo > 0 and prof[lo] > half:
        lo -= 1
    hi = i_pk
    while hi < prof.size - 1 and prof[hi] > half:
        hi += 1
    assert 0 < lo and hi < prof.size - 1, "-6 dB lobe not inside the profile"

    def cross(i0, i1):
        f = (half - prof[i0]) / (prof[i1] - prof[i0])
        return coord[i0] + f * (coord[i1] - coord[i0])

    return cross(hi - 1, hi) - cross(lo + 1, lo)


@pytest.fixture(scope="module")
def bowl():
    grid = cg.Grid(SHAPE, ODX, cg.PMLSpec(5e-3))
    med = cg.Medium.homogeneous(grid.shape, c=C0, rho=1000.0)
    src = bowl_source(grid, f0=F0, amplitude=1.0e5, aperture_radius=A_AP, roc=ROC, apex_vox=APEX)
    spec = cg.CWRunSpec(min_settle_periods=8, max_settle_periods=30, n_record_periods=2)
    res = cg.LinearKSpaceGB300().run(grid, med, src, spec, reference_point=FOCUS_VOX)
    return grid, res


def test_focus_within_one_voxel_of_oneill(bowl):
    grid, res = bowl
    amp = res.amp
    peak = np.unravel_index(np.argmax(amp), amp.shape)
    z_phys = (np.arange(SHAPE[2]) - APEX[2]) * ODX
    p_on = oneill_axial(z_phys[24:100], A_AP, ROC, F0)
    z_true_vox = APEX[2] + z_phys[24:100][np.argmax(p_on)] / ODX
    assert abs(peak[0] - FOCUS_VOX[0]) <= 1 and abs(peak[1] - FOCUS_VOX[1]) <= 1
    assert abs(peak[2] - z_true_vox) <= 1.0


def test_axial_profile_matches_oneill(bowl):
    grid, res = bowl
    axial = res.amp[APEX[0], APEX[1], :]
    z_phys = (np.arange(SHAPE[2]) - APEX[2]) * ODX
    z_limit = (SHAPE[2] - grid.pml_vox - 2 - APEX[2]) * ODX
    sel = (z_phys > 0.5 * ROC) & (z_phys < min(1.5 * ROC, z_limit))
    b = oneill_axial(z_phys[sel], A_AP, ROC, F0)
    r = np.corrcoef(axial[sel] / axial[sel].max(), b / b.max())[0, 1]
    assert r > 0.99, f"axial correlation {r:.5f}"
    sel_w = (z_phys > 0.5 * ROC) & (z_phys < z_limit)
    w_s = minus6db_width(z_phys[sel_w], axial[sel_w] / axial[sel_w].max())
    bw = oneill_axial(z_phys[sel_w], A_AP, ROC, F0)
    w_o = minus6db_width(z_phys[sel_w], bw / bw.max())
    assert abs(w_s - w_o) / w_o < 0.05


def test_lateral_profile_matches_rayleigh(bowl):
    _grid, res = bowl
    amp = res.amp
    z_pk = int(np.argmax(amp[APEX[0], APEX[1], :]))
    lateral = amp[:, APEX[1], z_pk]
    assert abs(int(np.argmax(lateral)) - APEX[0]) <= 1
    x_phys = (np.arange(SHAPE[0]) - APEX[0]) * ODX
    z_phys = (z_pk - APEX[2]) * ODX
    pts = spherical_cap_points(A_AP, ROC, spacing=C0 / F0 / 5.0)
    targets = np.column_stack([x_phys, np.zeros_like(x_phys), np.full_like(x_phys, z_phys)])
    p_ray = rayleigh_abs(pts, targets, F0)
    sel = np.abs(x_phys) < 6e-3
    a = lateral[sel] / lateral[sel].max()
    b = p_ray[sel] / p_ray[sel].max()
    w_s, w_r = minus6db_width(x_phys[sel], a), minus6db_width(x_phys[sel], b)
    assert abs(w_s - w_r) / w_r < 0.05
    assert np.corrcoef(a, b)[0, 1] > 0.98


# ----------------------------------------------------------------- Fubini --
BETA = 3.5


def fubini(n, sigma):
    """B_n(sigma) = 2 J_n(n sigma) / (n sigma), 0 < sigma <= 1."""
    from scipy.special import jv

    return 2.0 * jv(n, n * sigma) / (n * sigma)


def shock_distance(p0, f0=F0, c0=C0, rho=1000.0, beta=BETA):
    return rho * c0 ** 3 / (beta * 2.0 * np.pi * f0 * p0)


@pytest.fixture(scope="module")
def fubini_run():
    dx = C0 / (F0 * 16.0)
    grid = cg.Grid((600,), dx, cg.PMLSpec(40 * dx))
    med = cg.Medium.homogeneous(grid.shape, c=C0, rho=1000.0, beta=BETA)
    spec = cg.CWRunSpec(min_settle_periods=45, max_settle_periods=100, convergence_tol=0.003)
    res = cg.WesterveltKSpaceGB300().run(grid, med, _plane_source(grid, 2.0e6, 60), spec, harmonics=(1, 2, 3))
    return res, dx


def _shock_axis(res, dx, src_vox=60):
    a1 = res.harmonic_amp(1)
    i0 = 90
    sig0 = ((i0 - src_vox) * dx) / shock_distance(a1[i0])
    return a1, shock_distance(a1[i0] / fubini(1, sig0))


def test_fubini_second_harmonic_within_5_percent(fubini_run):
    res, dx = fubini_run
    a1, x_sh = _shock_axis(res, dx)
    a2 = res.harmonic_amp(2)
    assert res.meta["nonlinear_active"] is True
    checked = 0
    for iv in (150, 250, 350, 450, 540):
        sigma = ((iv - 60) * dx) / x_sh
        if not 0.05 <= sigma <= 0.95:
            continue
        want = fubini(2, sigma) / fubini(1, sigma)
        assert abs(a2[iv] / a1[iv] - want) / want < 0.05, f"sigma {sigma:.3f}"
        checked += 1
    assert checked >= 4


def test_fubini_third_harmonic_within_10_percent(fubini_run):
    res, dx = fubini_run
    a1, x_sh = _shock_axis(res, dx)
    a3 = res.harmonic_amp(3)
    for iv in (350, 450, 540):
        sigma = ((iv - 60) * dx) / x_sh
        want = fubini(3, sigma) / fubini(1, sigma)
        assert abs(a3[iv] / a1[iv] - want) / want < 0.10, f"sigma {sigma:.3f}"


def test_nonlinear_phasor_within_the_sampling_ceiling(fubini_run):
    res, _dx = fubini_run
    band = res.p_max > 0.10 * res.p_max.max()
    ratio = res.amp[band] / res.p_max[band]
    assert ratio.max() <= (1.0 / np.cos(np.pi / res.spp)) * (1 + 1e-3)
    assert 0.85 <= res.amp[90] / res.p_max[90] <= 1.0 + 1e-3

"""Seeded synthetic inputs of the benchmark configurations.

The workloads are built the way the reference builds them, restated here so
they exist on hosts without caustica:

* focused bowls voxelised from an equal-area Fibonacci lattice on the cap
  (analytic/geometry.py:13-64, sources.py:143-175);
* media as integer label maps with one (alpha, rho, c, beta) row per
  material (medium.py:57-81), attenuation converted with
  ``db_cm_to_np_m`` (materials.py:102-104).

Configurations (grid, drive and medium as the benchmark definitions state
them, with the geometry adjustments the survey measured so every source
fits its grid):

* ``config1``: linear, 96x96x128, dx 0.3 mm, 500 kHz bowl (aperture radius
  12 mm, ROC 30 mm) at apex (48, 48, 10), water, 10-cell sponge, cfl 0.3,
  40 periods with the fundamental recorded over the last 10.
* ``config2``: Westervelt, 192x192x256, dx 0.15 mm, 1 MHz bowl scaled to
  aperture radius 8 mm / ROC 20 mm at apex (96, 96, 10), 1 MPa, water /
  skin / fat / muscle slabs along +z whose interfaces are seeded Gaussian
  random surfaces (sigma 0.5 mm, correlation length 3 mm), harmonics 1-3,
  cfl 0.48, 40 periods recording the last 10.
"""

from __future__ import annotations

import numpy as np

from .contract import CWRunSpec, CWSource, Grid, Medium, PMLSpec
from .engine import cw_tof_periods

_GOLDEN_ANGLE = np.pi * (3.0 - np.sqrt(5.0))


def db_cm_to_np_m(alpha_db_cm: float) -> float:
    """dB/cm -> Np/m (materials.py:102-104)."""
    return alpha_db_cm * 100.0 / (20.0 * np.log10(np.e))


def spherical_cap_points(aperture_radius: float, roc: float, spacing: float) -> np.ndarray:
    """Equal-area points on a concave cap, apex at the origin, axis +z.

    Fibonacci lattice: cos(theta) uniform in [cos(theta_max), 1] and azimuth
    stepped by the golden angle (analytic/geometry.py:13-64).
    """
    a, f = float(aperture_radius), float(roc)
    if not 0 < a < f:
        raise ValueError(f"need 0 < aperture_radius < roc, got a={a}, roc={f}")
    cos_tmax = np.sqrt(1.0 - (a / f) ** 2)
    cap_area = 2.0 * np.pi * f**2 * (1.0 - cos_tmax)
    n = max(int(np.ceil(cap_area / spacing**2)), 16)
    j = np.arange(n, dtype=np.float64)
    cos_t = 1.0 - (1.0 - cos_tmax) * (j + 0.5) / n
    sin_t = np.sqrt(np.clip(1.0 - cos_t**2, 0.0, None))
    phi = j * _GOLDEN_ANGLE
    return np.column_stack((f * sin_t * np.cos(phi), f * sin_t * np.sin(phi), f * (1.0 - cos_t)))


def bowl_source(grid: Grid, f0: float, amplitude: float, aperture_radius: float, roc: float, apex_vox,
                spacing: float | None = None) -> CWSource:
    """Uniform-phase bowl voxelised at dx/2 sampling (sources.py:143-175)."""
    ds = grid.dx / 2.0 if spacing is None else float(spacing)
    pts = spherical_cap_points(aperture_radius, roc, ds)
    idx = np.round(pts / grid.dx).astype(np.int64) + np.asarray(apex_vox, np.int64)
    idx = np.unique(idx, axis=0)
    src = CWSource(indices=idx, phases=np.zeros(idx.shape[0], np.float32), amplitude=amplitude, f0=f0,
                   label=f"bowl(a={aperture_radius * 1e3:.1f}mm, roc={roc * 1e3:.1f}mm)")
    src.check_inside(grid)
    return src


def gaussian_surface(n0: int, n1: int, dx: float, sigma: float, corr: float, rng) -> np.ndarray:
    """2-D Gaussian random surface: white noise smoothed by a Gaussian of
    correlation length ``corr`` (periodic, via FFT), rescaled to std ``sigma``."""
    w = rng.standard_normal((n0, n1))
    k0 = np.fft.fftfreq(n0, d=dx) * 2 * np.pi
    k1 = np.fft.fftfreq(n1, d=dx) * 2 * np.pi
    kk = k0[:, None] ** 2 + k1[None, :] ** 2
    s = np.real(np.fft.ifft2(np.fft.fft2(w) * np.exp(-kk * corr**2 / 4.0)))
    s -= s.mean()
    return s * (sigma / s.std())


WATER = (db_cm_to_np_m(0.0022), 1000.0, 1500.0, 3.5)  # 0.0022 dB/cm/MHz^2 at 1 MHz, B/A 5 -> beta 3.5


def config1(*, water_beta: float = 0.0):
    """Plain linear CW solve (96x96x128)."""
    grid = Grid((96, 96, 128), 0.3e-3, PMLSpec(3.0e-3))
    alpha = db_cm_to_np_m(0.0022 * 0.5**2)
    medium = Medium.homogeneous(grid.shape, alpha_np_m=alpha, rho=1000.0, c=1500.0, beta=water_beta)
    source = bowl_source(grid, f0=5e5, amplitude=1e5, aperture_radius=12e-3, roc=30e-3, apex_vox=(48, 48, 10))
    spec = CWRunSpec(cfl=0.3, convergence_tol=0.0, min_settle_periods=8, max_settle_periods=14, n_record_periods=10)
    return {"name": "config1_linear_96x96x128", "grid": grid, "medium": medium, "source": source, "spec": spec,
            "harmonics": (1,), "nonlinear": False, "reference_point": None}


def config2(seed: int = 2):
    """Westervelt CW solve over layered tissue (192x192x256), harmonics 1-3."""
    shape = (192, 192, 256)
    dx = 0.15e-3
    grid = Grid(shape, dx, PMLSpec(10 * dx))
    rng = np.random.default_rng(seed)
    tissues = {
        0: WATER,
        1: (db_cm_to_np_m(2.3), 1090.0, 1610.0, 1.0 + 7.9 / 2.0),  # skin
        2: (db_cm_to_np_m(0.6), 950.0, 1450.0, 1.0 + 10.0 / 2.0),  # fat
        3: (db_cm_to_np_m(1.1), 1050.0, 1580.0, 1.0 + 7.4 / 2.0),  # muscle
    }
    # interfaces (z of the top of skin, fat, muscle) with seeded random relief
    z_skin, t_skin, t_fat = 30 * dx, 2e-3, 5e-3
    tops = [z_skin, z_skin + t_skin, z_skin + t_skin + t_fat]
    z = (np.arange(shape[2]) * dx)[None, None, :]
    labels = np.zeros(shape, np.int32)
    for lab, top in enumerate(tops, start=1):
        surf = top + gaussian_surface(shape[0], shape[1], dx, 0.5e-3, 3e-3, rng)
        labels[z >= surf[:, :, None]] = lab
    medium = Medium.from_labels(labels, tissues)
    source = bowl_source(grid, f0=1e6, amplitude=1e6, aperture_radius=8e-3, roc=20e-3, apex_vox=(96, 96, 10))
    # time of flight to the geometric focus; the settle cap makes the schedule
    # 30 settle + 10 record = 40 periods
    focus = (96, 96, 10 + int(round(20e-3 / dx)))
    tof = cw_tof_periods(shape, dx, float(medium.c.min()), 1e6, source.indices, focus)
    spec = CWRunSpec(cfl=0.48, convergence_tol=0.0, min_settle_periods=8, max_settle_periods=30 - tof,
                     n_record_periods=10)
    return {"name": "config2_westervelt_192x192x256", "grid": grid, "medium": medium, "source": source,
            "spec": spec, "harmonics": (1, 2, 3), "nonlinear": True, "reference_point": focus}

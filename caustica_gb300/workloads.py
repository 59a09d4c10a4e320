"""Seeded synthetic inputs of the benchmark configurations.

The workloads are built the way the reference builds them, restated here so
they exist on hosts without caustica:

* focused bowls voxelised from an equal-area Fibonacci lattice on the cap
  (analytic/geometry.py:13-64, sources.py:143-175);
* media as integer label maps with one (alpha, rho, c, beta) row per
  material (medium.py:57-81), attenuation converted with
  ``db_cm_to_np_m`` (materials.py:102-104).

Configurations (grid, drive and medium as the benchmark definitions state
them, with the geometry adjusted where the stated transducer does not fit
the stated grid):

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


# --------------------------------------------------------- phased arrays --
def archimedean_spiral(n_elements: int, d_outer: float, d_inner: float, roc: float, active_fraction: float = 0.6,
                       n_arc_samples: int = 10000):
    """Element centres, normals and radius of a spherically curved Archimedean
    spiral (arrays/transducer.py:178-226): equal arc-length spacing from
    r_in + r_e to r_out - r_e, element radius from the active shell area."""
    r_out, r_in = d_outer / 2.0, d_inner / 2.0
    cap_h = roc - np.sqrt(roc**2 - r_out**2)
    hole_h = roc - np.sqrt(roc**2 - r_in**2)
    active_area = 2.0 * np.pi * roc * (cap_h - hole_h) * active_fraction
    elem_radius = np.sqrt((active_area / n_elements) / np.pi)
    r_start, r_end = r_in + elem_radius, r_out - elem_radius
    if r_start >= r_end:
        raise ValueError("element radius does not fit between the apertures")
    turns = np.sqrt(((r_end - r_start) * n_elements) / (np.pi * (r_end + r_start)))
    b = (r_end - r_start) / (2.0 * np.pi * turns)
    theta_hr = np.linspace(0.0, 2.0 * np.pi * turns, n_arc_samples)
    g = np.sqrt((r_start + b * theta_hr) ** 2 + b**2)
    arc_len = np.concatenate([[0.0], np.cumsum(0.5 * (g[1:] + g[:-1]) * np.diff(theta_hr))])
    theta = np.interp(np.linspace(0.0, arc_len[-1], n_elements), arc_len, theta_hr)
    r = r_start + b * theta
    positions = np.column_stack((r * np.cos(theta), r * np.sin(theta), roc - np.sqrt(roc**2 - r**2)))
    normals = np.array([0.0, 0.0, roc]) - positions
    normals /= np.linalg.norm(normals, axis=1, keepdims=True)
    return positions, normals, float(elem_radius)


def das_phases(positions: np.ndarray, target_m, f0: float, c0: float = 1500.0) -> np.ndarray:
    """Delay-and-sum focusing phases, -k d wrapped to [0, 2 pi), min 0
    (arrays/transducer.py:59-71)."""
    k0 = 2.0 * np.pi * f0 / c0
    d = np.linalg.norm(positions - np.asarray(target_m, np.float64), axis=1)
    phase = (-k0 * d) % (2.0 * np.pi)
    phase -= phase.min()
    return phase.astype(np.float32)


def voxelize_elements(positions, normals, elem_radius, dx, apex_vox):
    """Element discs as 1-voxel curved shells; a voxel claimed by several
    elements keeps the first (arrays/transducer.py:96-164). Returns the unique
    voxel indices and the element of each voxel."""
    dx_mm = dx * 1e3
    pos_mm = positions * 1e3
    r_vox = int(np.ceil(elem_radius * 1e3 / dx_mm)) + 1
    rows, owners = [], []
    offs = np.arange(-r_vox, r_vox + 1)
    ox, oy = np.meshgrid(offs, offs, indexing="ij")
    ox, oy = ox.reshape(-1), oy.reshape(-1)
    inside = (ox * dx_mm) ** 2 + (oy * dx_mm) ** 2 <= (elem_radius * 1e3) ** 2
    ox, oy = ox[inside], oy[inside]
    for i in range(positions.shape[0]):
        p0, nv = pos_mm[i], normals[i]
        e = [int(np.round(p0[k] / dx_mm)) + apex_vox[k] for k in range(3)]
        oz = np.round(-(nv[0] * ox + nv[1] * oy) / nv[2]).astype(np.int64) if abs(nv[2]) > 1e-6 else 0 * ox
        rows.append(np.column_stack((e[0] + ox, e[1] + oy, e[2] + oz)))
        owners.append(np.full(ox.size, i, np.int32))
    idx = np.concatenate(rows).astype(np.int64)
    elem = np.concatenate(owners)
    uniq, first = np.unique(idx, axis=0, return_index=True)
    return uniq, elem[first]


def ellipsoid_labels(shape, dx, n, rng, *, semi_mm=(2.0, 8.0), z_range_mm=None, start_label=1):
    """Seeded ellipsoid inclusions (random semi-axes and rotation) painted into
    an integer label map; later inclusions overwrite earlier ones."""
    labels = np.zeros(shape, np.int32)
    ext = np.array(shape) * dx
    grids = [np.arange(s) * dx for s in shape]
    for j in range(n):
        axes = rng.uniform(semi_mm[0], semi_mm[1], 3) * 1e-3
        q = rng.standard_normal(4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        zlo, zhi = z_range_mm if z_range_mm is not None else (0.25 * ext[2] * 1e3, 0.85 * ext[2] * 1e3)
        c = np.array([rng.uniform(0.3, 0.7) * ext[0], rng.uniform(0.3, 0.7) * ext[1],
                      rng.uniform(zlo, zhi) * 1e-3])
        r = float(axes.max())
        sl = [slice(max(0, int((c[k] - r) / dx)), min(shape[k], int((c[k] + r) / dx) + 2)) for k in range(3)]
        X, Y, Z = np.meshgrid(grids[0][sl[0]], grids[1][sl[1]], grids[2][sl[2]], indexing="ij")
        d = np.stack([X - c[0], Y - c[1], Z - c[2]], axis=-1) @ R
        inside = ((d / axes) ** 2).sum(-1) <= 1.0
        labels[tuple(sl)][inside] = start_label + j
    return labels


def config4(n_steers: int = 64, seed: int = 4):
    """64 steering positions of a 256-element spiral over one inclusion medium
    (160x160x192, dx 0.25 mm, 1 MHz, linear). The array is scaled to fit the
    grid: d_outer 32 mm, d_inner 8 mm, ROC 38 mm (element radius 0.769 mm,
    7,401 voxels, all 256 elements kept); targets uniform in +-4 mm around
    the natural focus. Schedule: flight time to the focus + 4 periods of
    settling, then 10 recorded periods (41 periods)."""
    shape = (160, 160, 192)
    dx = 0.25e-3
    f0 = 1e6
    grid = Grid(shape, dx, PMLSpec(10 * dx))
    rng = np.random.default_rng(seed)
    labels = ellipsoid_labels(shape, dx, 8, rng)
    table = {0: (db_cm_to_np_m(0.0022), 1000.0, 1500.0, 0.0)}
    for j in range(1, 9):
        table[j] = (db_cm_to_np_m(rng.uniform(0.3, 1.2)), rng.uniform(900.0, 1100.0), rng.uniform(1450.0, 1650.0), 0.0)
    medium = Medium.from_labels(labels, table)
    apex = (80, 80, 12)
    pos, nrm, r_e = archimedean_spiral(256, 32e-3, 8e-3, 38e-3, 0.6)
    idx, elem = voxelize_elements(pos, nrm, r_e, dx, apex)
    focus_m = np.array([0.0, 0.0, 38e-3])
    targets = focus_m + rng.uniform(-4e-3, 4e-3, (n_steers, 3))
    elem_phases = np.stack([das_phases(pos, t, f0) for t in targets])
    phases = np.ascontiguousarray(elem_phases[:, elem])  # (B, S) per voxel
    source = CWSource(indices=idx, phases=phases[0], amplitude=1e5, f0=f0, label="spiral(256)")
    source.check_inside(grid)
    focus = (apex[0], apex[1], apex[2] + int(round(38e-3 / dx)))
    tof = cw_tof_periods(shape, dx, float(medium.c.min()), f0, idx, focus)
    # fixed schedule: time of flight to the focus + the 4-period ramp floor, then 10 recorded periods
    spec = CWRunSpec(cfl=0.48, convergence_tol=0.0, min_settle_periods=4, max_settle_periods=4, n_record_periods=10)
    return {"name": f"config4_steer{n_steers}_160x160x192", "grid": grid, "medium": medium, "source": source,
            "spec": spec, "harmonics": (1,), "nonlinear": False, "reference_point": focus, "phases": phases,
            "element_of_voxel": elem, "targets": targets}


# ------------------------------------------------------- served stream --
CONFIG5_GRIDS = ((64, 64, 64), (96, 96, 128), (128, 128, 160), (192, 192, 256), (256, 256, 320))


def config5_medium(shape, dx, rng, *, nonlinear: bool):
    """Water with seeded random ellipsoid inclusions (the config-4 recipe)."""
    labels = ellipsoid_labels(shape, dx, 4, rng, semi_mm=(1.0, 4.0)).astype(np.uint8)
    beta_w = 3.5 if nonlinear else 0.0
    table = {0: (db_cm_to_np_m(0.0022), 1000.0, 1500.0, beta_w)}
    for j in range(1, 5):
        table[j] = (db_cm_to_np_m(rng.uniform(0.3, 1.2)), rng.uniform(900.0, 1100.0), rng.uniform(1450.0, 1650.0),
                    rng.uniform(4.0, 6.0) if nonlinear else 0.0)
    return Medium.from_labels(labels, table)


_THERMAL_MEDIA: dict = {}


def config5_thermal(shape, dx: float = 0.25e-3) -> dict:
    """The thermal phase a served request carries: soft tissue (k 0.5 W/m/K,
    rho 1000 kg/m^3, cp 3600 J/kg/K, perfusion 0.5/1050 1/s) on the request's
    grid, 0.05 s steps, 400 heating then 1200 cooling, CEM43 dose on."""
    from .thermal import ThermalMedium

    key = (tuple(shape), float(dx))
    if key not in _THERMAL_MEDIA:  # homogeneous: one read-only instance per grid serves every request
        _THERMAL_MEDIA[key] = ThermalMedium.homogeneous(tuple(shape), k=0.5, rho=1000.0, specific_heat=3600.0,
                                                        perfusion=0.5 / 1050.0, dx=dx)
    return {"medium": _THERMAL_MEDIA[key], "dt": 0.05, "n_heat": 400, "n_cool": 1200}


def config5_requests(n: int, seed: int = 5, *, grids=CONFIG5_GRIDS, p_nonlinear: float = 0.3,
                     p_thermal: float = 0.3, p_reuse: float = 0.2):
    """Seeded request stream: grid uniform over ``grids`` (dx 0.25 mm, 1 MHz,
    10-cell sponge), linear or Westervelt, thermal attached with probability
    ``p_thermal`` (k 0.5, rho 1000, cp 3600, perfusion 0.5/1050 1/s; 0.05 s
    steps, 400 heating + 1200 cooling), a bowl scaled to the grid (aperture
    radius 0.3x the lateral interior, ROC 0.6x the axial extent, apex two
    cells inside the sponge), and a medium drawn from a small pool for
    ``p_reuse`` of the requests (those can be packed into one launch).
    Schedule: flight time to the focus + 4 periods, 2 recorded periods.
    Every request asks for its focal metrics (apex and geometric focus)."""
    from .metrics import FieldFrame
    from .serve import Request

    rng = np.random.default_rng(seed)
    dx, f0, pml = 0.25e-3, 1e6, 10
    pool: dict = {}
    reqs = []
    for i in range(n):
        shape = tuple(grids[int(rng.integers(len(grids)))])
        nonlinear = bool(rng.random() < p_nonlinear)
        thermal = bool(rng.random() < p_thermal)
        grid = Grid(shape, dx, PMLSpec(pml * dx))
        reused = bool(rng.random() < p_reuse)
        if reused:
            key = (shape, nonlinear)
            if key not in pool:
                pool[key] = config5_medium(shape, dx, np.random.default_rng((seed, len(pool))), nonlinear=nonlinear)
            med = pool[key]
        else:
            med = config5_medium(shape, dx, rng, nonlinear=nonlinear)
        a = 0.3 * (shape[0] - 2 * pml) * dx
        roc = 0.6 * shape[2] * dx
        apex = (shape[0] // 2, shape[1] // 2, pml + 2)
        src = bowl_source(grid, f0=f0, amplitude=3e5 if nonlinear else 1e5, aperture_radius=a, roc=roc, apex_vox=apex)
        focus = (apex[0], apex[1], apex[2] + int(round(roc / dx)))
        spec = CWRunSpec(cfl=0.48, convergence_tol=0.0, min_settle_periods=4, max_settle_periods=4,
                         n_record_periods=2)
        th = config5_thermal(shape, dx) if thermal else None
        frame = FieldFrame(dx=dx, grid_shape=shape, pml_vox=pml, apex_vox=apex, focus_vox=focus)
        reqs.append(Request(grid=grid, medium=med, source=src, spec=spec, nonlinear=nonlinear,
                            harmonics=(1, 2) if nonlinear else (1,), reference_point=focus, thermal=th, frame=frame,
                            tag={"i": i, "shape": shape, "nonlinear": nonlinear, "thermal": thermal,
                                 "reused": reused}))
    return reqs

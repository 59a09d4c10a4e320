"""Hand-written batched 3-D R2C/C2R against NumPy FP64 (GPU)."""

from __future__ import annotations

import numpy as np
import pytest

from caustica_gb300.fft import FFT3D

pytestmark = pytest.mark.gpu

# the operator-test shapes of the reference padded to 2/3/5-smooth sizes,
# odd/even mixes, 1-D and 2-D embeddings, the radix-3/5 config sizes
SHAPES = [(8, 8, 8), (8, 9, 6), (6, 6, 8), (9, 8, 8), (1, 1, 600), (1, 20, 24), (16, 24, 30), (5, 12, 10),
          (3, 25, 9), (96, 96, 128), (40, 48, 64), (64, 80, 96), (20, 24, 320),
          # every axis on the size-specialised path
          (16, 24, 32), (32, 48, 48), (8, 16, 256), (160, 16, 8), (24, 192, 16), (128, 64, 24),
          # x/y passes on the 20- and 32-thread pencil splits (z on the runtime-plan passes here)
          (320, 8, 6), (6, 400, 8), (512, 6, 4), (4, 640, 6), (8, 4, 400), (4, 6, 512), (4, 8, 640)]


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("shape", SHAPES)
def test_forward_matches_numpy_fp64(shape):
    rng = np.random.default_rng(sum(shape))
    x = rng.standard_normal((2, *shape)).astype(np.float32)
    with FFT3D(shape, batch=2) as f:
        got = FFT3D.to_numpy_layout(f.forward(x))
    want = np.fft.rfftn(x.astype(np.float64), axes=(1, 2, 3))
    assert _rel(got, want) < 3e-6


@pytest.mark.parametrize("shape", SHAPES)
def test_inverse_matches_numpy_fp64(shape):
    rng = np.random.default_rng(1 + sum(shape))
    x = rng.standard_normal(shape)
    spec = np.fft.rfftn(x)  # a legal half spectrum
    with FFT3D(shape) as f:
        got = f.inverse(FFT3D.from_numpy_layout(spec[None].astype(np.complex64)))[0]
    want = np.fft.irfftn(spec, s=shape, axes=(0, 1, 2)) * np.prod(shape)
    assert _rel(got, want) < 3e-6


def test_c2r_reads_only_the_real_part_of_self_paired_bins():
    """A complex-to-real transform must ignore Im of the DC / Nyquist planes, as pocketfft does."""
    shape = (6, 8, 10)
    rng = np.random.default_rng(5)
    spec = np.fft.rfftn(rng.standard_normal(shape))
    bad = spec.copy()
    bad[0, 0, 0] += 3j
    bad[0, 0, -1] += 2j
    with FFT3D(shape) as f:
        a = f.inverse(FFT3D.from_numpy_layout(spec[None].astype(np.complex64)))
        b = f.inverse(FFT3D.from_numpy_layout(bad[None].astype(np.complex64)))
    np.testing.assert_allclose(a, b, atol=1e-5 * np.abs(a).max())


def test_round_trip_scales_by_the_cell_count():
    shape = (12, 10, 16)
    x = np.random.default_rng(9).standard_normal(shape).astype(np.float32)
    with FFT3D(shape) as f:
        back = f.inverse(f.forward(x))[0] / np.prod(shape)
    np.testing.assert_allclose(back, x, atol=2e-6 * np.abs(x).max())

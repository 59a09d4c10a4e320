"""The allocation-free forward FFT against the allocating one (GPU).

``cg_fft3d_forward_noalloc`` serves callers that may not allocate device
memory (a host framework owns the CUDA heap, or a serving loop must avoid
cudaMalloc's implicit synchronisation): they pass their own device buffers
and the transform's twiddle tables live in a fixed array inside the
library. This file is collected last on purpose, and it passes alone in a
fresh process as well as after the rest of the suite.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from caustica_gb300 import _lib
from caustica_gb300.fft import FFT3D

pytestmark = pytest.mark.gpu

REL_TOL = 3e-6  # same bound as the FFT parity tests


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _noalloc(lib, torch, x, out):
    batch, nx, ny, nz = x.shape
    stream = torch.cuda.current_stream().cuda_stream
    return lib.cg_fft3d_forward_noalloc(nx, ny, nz, batch, C.c_void_p(x.data_ptr()),
                                        C.c_void_p(out.data_ptr()), C.c_void_p(stream))


@pytest.mark.parametrize("shape,batch", [
    ((24, 20, 32), 2),
    # the largest axis lengths whose runtime-plan tiles fit 227 KB of shared memory
    ((6, 540, 10), 1),
    ((576, 4, 6), 1),
    ((4, 6, 810), 1),
])
def test_noalloc_forward_matches_the_allocating_entry_point_twice_in_a_row(shape, batch):
    torch = pytest.importorskip("torch")
    nx, ny, nz = shape
    lib = _lib.load()
    rng = np.random.default_rng(11)
    with FFT3D(shape, batch=batch) as f:
        for call in range(2):  # the shared scratch keeps the previous call's tables
            x = rng.standard_normal((batch, *shape)).astype(np.float32)
            want = f.forward(x)
            xin = torch.from_numpy(x).cuda()
            out = torch.zeros((batch, nx, nz // 2 + 1, ny, 2), dtype=torch.float32, device="cuda")
            _lib.check(_noalloc(lib, torch, xin, out), "cg_fft3d_forward_noalloc")
            torch.cuda.synchronize()
            got = out.cpu().numpy().view(np.complex64)[..., 0]
            assert _rel(got, want) < REL_TOL, f"call {call}"


@pytest.mark.parametrize("shape", [(64, 640, 64), (640, 8, 8), (8, 8, 864)])
def test_noalloc_forward_refuses_tiles_beyond_shared_memory_and_writes_nothing(shape):
    """Axis lengths the allocating transform serves with size-specialised
    passes (640) but whose runtime-plan tile does not fit shared memory are
    refused before anything is queued: the output keeps its contents."""
    torch = pytest.importorskip("torch")
    nx, ny, nz = shape
    lib = _lib.load()
    xin = torch.ones((1, *shape), dtype=torch.float32, device="cuda")
    out = torch.full((1, nx, nz // 2 + 1, ny, 2), 7.0, dtype=torch.float32, device="cuda")
    rc = _noalloc(lib, torch, xin, out)
    torch.cuda.synchronize()
    assert rc == _lib.CG_ERR_INVALID
    assert b"shared memory" in lib.cg_last_error()
    assert bool((out == 7.0).all())


def test_noalloc_forward_refuses_shapes_beyond_its_fixed_scratch():
    lib = _lib.load()
    rc = lib.cg_fft3d_forward_noalloc(8, 8, 4096, 1, C.c_void_p(1), C.c_void_p(1), None)
    assert rc == _lib.CG_ERR_INVALID
    assert b"exceeds the fixed scratch" in lib.cg_last_error()

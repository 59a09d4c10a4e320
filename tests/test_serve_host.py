"""Host side of the server's packing rule (no GPU)."""

from __future__ import annotations

import numpy as np

import caustica_gb300 as cg
from caustica_gb300 import serve


def _medium(seed, shape=(12, 10, 16)):
    rng = np.random.default_rng(seed)
    ids = rng.integers(0, 3, shape)
    table = {0: (0.5, 1000.0, 1500.0, 0.0), 1: (8.0, 1050.0, 1580.0, 0.0), 2: (3.0, 950.0, 1450.0, 0.0)}
    return cg.Medium.from_labels(ids, table)


def _req(med, phase=0.0):
    grid = cg.Grid(med.shape, 0.25e-3, cg.PMLSpec(0.5e-3))
    idx = np.array([[5, 5, 3], [6, 5, 3]])
    src = cg.CWSource(indices=idx, phases=np.full(2, phase, np.float32), amplitude=1e5, f0=1e6)
    return serve.Request(grid=grid, medium=med, source=src, spec=cg.CWRunSpec())


def test_equal_media_built_separately_share_a_key_and_compare_equal():
    a, b = _medium(1), _medium(1)
    assert a is not b
    assert serve.medium_fingerprint(a) == serve.medium_fingerprint(b)
    assert serve.same_medium(a, b)
    assert serve._key(_req(a)) == serve._key(_req(b, phase=0.7))  # phases differ per member


def test_different_media_do_not_pack():
    a, c = _medium(1), _medium(2)
    assert not serve.same_medium(a, c)
    # a change the strided fingerprint does not sample still fails the full comparison
    d = _medium(1)
    d.c = d.c.copy()
    d.c.reshape(-1)[1] += 1.0
    assert not serve.same_medium(a, d)


def test_the_fingerprint_is_cached_per_object():
    a = _medium(3)
    f1 = serve.medium_fingerprint(a)
    assert serve._FP_CACHE[id(a)][0] is a
    assert serve.medium_fingerprint(a) == f1

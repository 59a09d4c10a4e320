"""Generate ``quantize_cases.npz``: the reference's float16 store quantisation on seeded fields.

Runs the UNCHANGED reference's ``try_float16`` (``io/quantize.py:45-67``)
on a set of float32 fields that exercise its branches and the float16
rounding: ordinary pressure-like values, a dynamic range wide enough to
reach float16 subnormals and zero, an all-zero field with negative zeros,
an empty field, exact float16 ties after scaling, a negative peak, a bound
tight enough to force the float32 fallback, and NaN / infinity (both fall
back). For each case the fixture holds the input, the bound, and the
reference's stored array (bit pattern), scale, dtype name and measured
error.

Usage (seconds; the fixture is committed, so the tests never need the
reference)::

    python tests/golden/make_quantize_golden.py /path/to/caustica/src
"""

from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def cases() -> dict[str, tuple[np.ndarray, float]]:
    rng = np.random.default_rng(20261204)
    out = {}
    out["normal"] = (rng.normal(0.0, 2.5e5, 3001).astype(np.float32), 1e-3)
    wide = (rng.standard_normal(4000) * 10.0 ** rng.uniform(-12, 6, 4000)).astype(np.float32)
    out["wide"] = (wide, 1e-3)
    z = np.zeros(257, np.float32)
    z[::3] = -0.0
    out["zeros"] = (z, 1e-3)
    out["empty"] = (np.zeros(0, np.float32), 1e-3)
    # peak 1.0; the others sit halfway between float16 neighbours in [0.5, 1)
    k = np.arange(1024, 2047, dtype=np.float64)
    ties = np.concatenate([[1.0], (k + 0.5) / 2048.0, -(k + 0.5) / 2048.0]).astype(np.float32)
    out["ties"] = (ties, 1e-3)
    neg = rng.uniform(-3.0, 1.0, 999).astype(np.float32)
    neg[17] = -7.25
    out["negative_peak"] = (neg, 1e-3)
    out["tight"] = (rng.normal(0.0, 1.0, 2048).astype(np.float32), 1e-5)
    tiny = rng.normal(0.0, 1e-30, 1500).astype(np.float32)
    out["tiny"] = (tiny, 1e-3)
    nan = rng.normal(0.0, 1.0, 100).astype(np.float32)
    nan[42] = np.nan
    out["nan"] = (nan, 1e-3)
    inf = rng.normal(0.0, 1.0, 100).astype(np.float32)
    inf[7] = np.inf
    out["inf"] = (inf, 1e-3)
    out["zero_bound"] = (rng.normal(0.0, 1.0, 64).astype(np.float32), 0.0)
    return out


def main(ref_src: str) -> None:
    sys.path.insert(0, ref_src)
    from caustica.io.quantize import try_float16

    data = {}
    names = []
    for name, (x, bound) in cases().items():
        q = try_float16(x, bound)
        names.append(name)
        data[f"{name}__x"] = x
        data[f"{name}__bound"] = np.float64(bound)
        data[f"{name}__stored_bits"] = q.stored.view(np.uint16 if q.dtype_name == "float16" else np.uint32)
        data[f"{name}__scale"] = np.float64(q.scale)
        data[f"{name}__dtype"] = np.str_(q.dtype_name)
        data[f"{name}__norm_err"] = np.float64(q.norm_err)
    data["names"] = np.array(names)
    np.savez_compressed(HERE / "quantize_cases.npz", **data)
    print(f"wrote {len(names)} cases to {HERE / 'quantize_cases.npz'}")


if __name__ == "__main__":
    src = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CAUSTICA_REFERENCE_SRC")
    if not src:
        raise SystemExit("usage: make_quantize_golden.py /path/to/caustica/src (or set CAUSTICA_REFERENCE_SRC)")
    main(src)

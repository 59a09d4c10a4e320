"""The ``caustica-result/1`` result store with device-side float16 quantisation.

The reference writes a solve result as one HDF5 file
(``io/store.py:92-174``): root attributes describing the run, the drive in
``input/``, the phasor real and imaginary parts of every recorded harmonic
plus ``p_max`` in ``output/`` -- each dynamically quantised to float16 when
the measured round-trip error allows (``try_float16``,
``io/quantize.py:45-67``), else kept float32 -- and the settling history in
``convergence/``. Here the quantisation runs on the GPU
(``cg_quantize_f16`` / ``cg_solver_quantize``): one read of each field to
find its peak, one to scale, round and measure the error, and only the
float16 bytes (half the float32 result) cross to the host. The stored
values, scales and measured errors equal the reference's bit for bit.

* :func:`quantize_arrays` -- fields given as device arrays (or host arrays,
  uploaded first: the arithmetic always runs on the device);
* :func:`quantize_solver` -- a solver handle's finalized result, in the
  order the store writes it, without any float32 copy to the host;
* :func:`save_result` -- the reference's ``save_result`` signature; it takes
  the fields a GB300 solve already quantised (``result.meta["quantized"]``,
  set when the front's ``store_quantize`` is given) or quantises the
  result's arrays on the device, and writes the file atomically (a unique
  ``.tmp`` sibling, then ``os.replace``; ``io/atomic.py:60-125``).

The file layout, attribute names and the two convention strings are the
reference's format, kept alike so its ``load_result`` reads these files.
HDF5 needs ``h5py``; without it :func:`save_result` raises ``ImportError``
and the quantisers still work.
"""

from __future__ import annotations

import ctypes as C
import os
import tempfile
from pathlib import Path
from typing import Any, NamedTuple

import numpy as np

from . import _lib
from .device import as_device, is_device_array

RESULT_FORMAT = "caustica-result/1"
DEFAULT_MAX_NORM_ERR = 1e-3

# the convention strings every result file carries (io/store.py:49-62)
PHASE_CONVENTION = (
    "p(t) = Re{P exp(-i omega t)}; outgoing wave = exp(+ikx) (matches the "
    "analytic O'Neil/Rayleigh references). The absolute phase zero is not "
    "source-referenced; relative phase (voxel-to-voxel) is exact."
)
ABSORPTION_MODEL = (
    "frequency-INDEPENDENT exponential, exp(-alpha*c*dt) per step, applied "
    "symmetrically to p and u so the spatial decay rate equals alpha (NOT "
    "the source notebook's p-only alpha/2). Harmonics above f0 are therefore "
    "under-absorbed relative to power-law tissue."
)
_RELOAD = 'arr = ds[:].astype("float32") * ds.attrs["scale"]'


class Quantized(NamedTuple):
    """One stored field: its values, the reload scale, the stored dtype name
    and the measured round-trip error as a fraction of the peak."""

    stored: np.ndarray
    scale: float
    dtype_name: str
    norm_err: float

    def restore(self) -> np.ndarray:
        return restore(self.stored, self.scale)


def restore(stored, scale: float) -> np.ndarray:
    """The reload recipe of every stored field: ``float32(stored) * float32(scale)``."""
    return np.asarray(stored).astype(np.float32) * np.float32(scale)


def _unpack(shapes, f16: np.ndarray, f32: np.ndarray, info: np.ndarray) -> list[Quantized]:
    out, off = [], 0
    for i, shape in enumerate(shapes):
        n = int(np.prod(shape, dtype=np.int64))
        scale, err, half = float(info[i, 0]), float(info[i, 1]), bool(info[i, 2])
        if half:
            out.append(Quantized(f16[off:off + n].view(np.float16).reshape(shape), scale, "float16", err))
        else:
            out.append(Quantized(f32[off:off + n].reshape(shape).copy(), 1.0, "float32", 0.0))
        off += n
    return out


def _check_bound(max_norm_err: float) -> float:
    v = float(max_norm_err)
    if not v >= 0.0:
        raise ValueError(f"max_norm_err must be >= 0, got {max_norm_err!r}")
    return v


def quantize_arrays(fields, max_norm_err: float = DEFAULT_MAX_NORM_ERR) -> list[Quantized]:
    """Quantise float32 fields on the device, one :class:`Quantized` each.

    Each field is a device array (DLPack / ``__cuda_array_interface__``, a
    library buffer) of float32, or a host array, which is uploaded first.
    Complex inputs are not accepted: pass the real and imaginary parts (the
    store quantises them separately).
    """
    bound = _check_bound(max_norm_err)
    fields = list(fields)
    if not 1 <= len(fields) <= 32:
        raise ValueError("quantize_arrays takes 1 to 32 fields per call")
    keep, owned, shapes = [], [], []
    arr = (_lib.QField * len(fields))()
    for i, f in enumerate(fields):
        if is_device_array(f):
            v = as_device(f, dtype=np.float32, what=f"field {i}")
        else:
            h = np.asarray(f)
            if h.dtype.kind == "c":
                raise ValueError(f"field {i} is complex: pass its real and imaginary parts")
            v = _lib.DeviceArray.from_host(np.ascontiguousarray(h, dtype=np.float32))
            owned.append(v)
        keep.append(v)
        shapes.append(v.shape)
        n = int(np.prod(v.shape, dtype=np.int64))
        arr[i].data = v.ptr.value if n else None
        arr[i].n = n
        arr[i].stride = 1
    total = sum(int(np.prod(s, dtype=np.int64)) for s in shapes)
    f16 = np.empty(total, np.uint16)
    f32 = np.empty(total, np.float32)  # pages are touched only for fields that keep float32
    info = np.zeros((len(fields), 4), np.float32)
    try:
        _lib.call("cg_quantize_f16", arr, len(fields), C.c_double(bound), _lib.ptr(f16), _lib.ptr(f32),
                  _lib.ptr(info), None)
    finally:
        for v in owned:
            v.close()
    return _unpack(shapes, f16, f32, info)


def field_names(harmonics) -> list[str]:
    """Dataset names of ``output/`` in the order the store writes them (io/store.py:146-151)."""
    names = []
    for h in sorted(int(h) for h in harmonics):
        names += [f"p_real_h{h}", f"p_imag_h{h}"]
    return names + ["p_max"]


def quantize_solver(dev, member: int = 0, max_norm_err: float = DEFAULT_MAX_NORM_ERR) -> dict[str, Quantized]:
    """Quantise member ``member`` of a finalized :class:`~caustica_gb300.engine.DeviceSolver` on the device.

    Returns ``{dataset name: Quantized}`` in store order; fields are shaped
    like the record region. Nothing but the stored bytes leaves the device.
    """
    bound = _check_bound(max_norm_err)
    names = field_names(dev.plan.harmonics)
    shape = tuple(s.stop - s.start for s in dev.plan.rec)
    n = int(dev.nrec)
    f16 = np.empty(len(names) * n, np.uint16)
    f32 = np.empty(len(names) * n, np.float32)
    info = np.zeros((len(names), 4), np.float32)
    _lib.call("cg_solver_quantize", dev.h, int(member), C.c_double(bound), _lib.ptr(f16), _lib.ptr(f32),
              _lib.ptr(info))
    return dict(zip(names, _unpack([shape] * len(names), f16, f32, info)))


def quantize_result(result, max_norm_err: float = DEFAULT_MAX_NORM_ERR) -> dict[str, Quantized]:
    """The stored fields of a host ``SolverResult``, quantised on the device."""
    arrays = []
    for h in sorted(result.phasors):
        ph = np.asarray(result.phasors[h])
        arrays += [np.ascontiguousarray(ph.real, np.float32), np.ascontiguousarray(ph.imag, np.float32)]
    arrays.append(np.asarray(result.p_max, np.float32))
    return dict(zip(field_names(result.phasors), quantize_arrays(arrays, max_norm_err)))


def _import_h5py():
    try:
        import h5py  # noqa: PLC0415 - optional dependency of the file format only
    except ImportError as exc:
        raise ImportError("writing caustica-result/1 files needs h5py (the quantisers do not)") from exc
    return h5py


def _stored_fields(result, quantize: bool, max_norm_err: float, quantized) -> dict[str, Quantized]:
    names = field_names(result.phasors)
    if not quantize:
        out = {}
        for h in sorted(result.phasors):
            ph = np.asarray(result.phasors[h])
            out[f"p_real_h{h}"] = Quantized(np.asarray(ph.real, np.float32), 1.0, "float32", 0.0)
            out[f"p_imag_h{h}"] = Quantized(np.asarray(ph.imag, np.float32), 1.0, "float32", 0.0)
        out["p_max"] = Quantized(np.asarray(result.p_max, np.float32), 1.0, "float32", 0.0)
        return out
    if quantized is None:
        pre = (result.meta or {}).get("quantized")
        if pre is not None and pre.get("max_norm_err") == max_norm_err and all(k in pre["fields"] for k in names):
            quantized = pre["fields"]
    if quantized is None:
        quantized = quantize_result(result, max_norm_err)
    missing = [k for k in names if k not in quantized]
    if missing:
        raise ValueError(f"quantized fields missing: {missing}")
    return {k: quantized[k] for k in names}


def save_result(path, result, source, *, dx: float, grid_shape, pml_vox: int = 0, quantize: bool = True,
                max_norm_err: float = DEFAULT_MAX_NORM_ERR, extra_attrs: dict[str, Any] | None = None,
                quantized: dict[str, Quantized] | None = None) -> Path:
    """Write one result as a ``caustica-result/1`` file, atomically (io/store.py:92-174).

    ``quantized`` (``{dataset name: Quantized}``, e.g. from
    :func:`quantize_solver`) skips the quantisation; otherwise the fields a
    GB300 solve attached (``result.meta["quantized"]`` with the same bound)
    are used, or the result's arrays are quantised on the device.
    """
    bound = _check_bound(max_norm_err)
    fields = _stored_fields(result, quantize, bound, quantized)
    h5py = _import_h5py()
    path = Path(path)
    from . import __version__

    fd, tmp = tempfile.mkstemp(dir=path.parent, prefix=f"{path.name}.{os.getpid():x}-", suffix=".tmp")
    os.close(fd)
    try:
        with h5py.File(tmp, "w") as hf:
            a = hf.attrs
            a["format"] = RESULT_FORMAT
            a["caustica_version"] = f"caustica-gb300 {__version__}"
            a["solver"] = str(result.meta.get("solver", ""))
            a["backend"] = str(result.meta.get("backend", ""))
            a["f0_hz"] = float(source.f0)
            a["dt_s"] = float(result.dt)
            a["spp"] = int(result.spp)
            a["steps_total"] = int(result.steps_total)
            a["t_end_s"] = float(result.t_end_s)
            a["tof_periods"] = int(result.tof_periods)
            a["converged_period"] = int(result.converged_period)
            a["settle_capped"] = bool(result.settle_capped)
            a["harmonics"] = sorted(result.phasors)
            a["dx_m"] = float(dx)
            a["grid_shape"] = list(grid_shape)
            a["pml_vox"] = int(pml_vox)
            a["region_start"] = [s.start for s in result.region]
            a["region_stop"] = [s.stop for s in result.region]
            a["phase_convention"] = PHASE_CONVENTION
            a["absorption_model"] = ABSORPTION_MODEL
            for key, val in (extra_attrs or {}).items():
                a[key] = val

            gin = hf.create_group("input")
            gin.create_dataset("source_indices", data=np.asarray(source.indices, dtype=np.int32))
            gin.create_dataset("source_phases_rad", data=np.asarray(source.phases, np.float32))
            gin.attrs["f0_hz"] = float(source.f0)
            gin.attrs["amplitude_pa"] = float(source.amplitude)
            gin.attrs["ramp_periods"] = float(source.ramp_periods)
            gin.attrs["label"] = str(source.label)
            gin.attrs["n_points"] = int(source.n_points)

            gout = hf.create_group("output")
            for name, q in fields.items():
                ds = gout.create_dataset(name, data=q.stored, chunks=True, compression="gzip", compression_opts=4)
                ds.attrs["scale"] = float(q.scale)
                ds.attrs["stored_dtype"] = q.dtype_name
                ds.attrs["quant_norm_err"] = float(q.norm_err)
                ds.attrs["reload"] = _RELOAD
            gout.attrs["stored"] = (
                "p_real_h{n}, p_imag_h{n} (harmonic phasors), p_max (time peak "
                "over the record window)"
            )
            gout.attrs["derived"] = (
                "p_amp = sqrt(p_real^2 + p_imag^2); p_phase = atan2(p_imag, p_real) "
                "— never stored, always recomputed"
            )
            gout.attrs["phase_convention"] = PHASE_CONVENTION
            gout.attrs["absorption_model"] = ABSORPTION_MODEL
            gout.attrs["pmax_window"] = (
                "time-domain peak over the RECORD window only (steady state); "
                "transient/settling peaks are excluded by design"
            )

            hist = np.asarray(result.convergence_history, dtype=np.float64).reshape(-1, 3)
            gconv = hf.create_group("convergence")
            gconv.create_dataset("history", data=hist)
            gconv.attrs["columns"] = "period, peak_pa, rel_change"
        os.replace(tmp, path)
    except BaseException:
        if os.path.exists(tmp):
            os.unlink(tmp)
        raise
    return path

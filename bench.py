"""Benchmark: Westervelt CW solve on 192x192x256 (harmonics 1-3) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One "step" is one time step of the k-space solver over the whole grid
(9,437,184 cells, labelled four-tissue medium, 10,862 source voxels). The
metric is grid-cell-steps/s (cells x steps / device time), whole job over
all ranks. Inputs are larger than L2 between timed steps (p and u are
151 MB, the three spectra 114 MB; L2 is 129 MB), so no flush is needed.

gb300 arm (default): K steps timed with CUDA events on the solver's stream,
barrier + synchronise on both sides, max over ranks; plus the per-launch
profile and roofline of the dominant kernel, a full end-to-end solve
through the public solver front from host numpy inputs (``e2e``), and the
reference CPU path timed on a bounded sample (``cpu_baseline``).

reference arm (``--impl reference``): the reference's CPU path for this step
(the NumPy/SciPy restatement in ``oracle/``, float32 like the reference's
stock path, all host cores) timed on a bounded sample of the same workload.
Under torchrun only rank 0 runs it.

N > 1: one process per GPU (torchrun), each rank solving its own replica of
the workload; ``scaling`` is "weak" and there is no data-path collective.
"""

from __future__ import annotations

import argparse
import json
import os
import shutil
import signal
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "grid-cell-steps/s"
UNIT = "cell-steps/s"
LABEL_BYTES = 1  # uint8 material label per cell


def _jsonable(o):
    if isinstance(o, np.generic):
        return o.item()
    raise TypeError(f"not JSON serialisable: {type(o).__name__}")


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        return dist, rank, ws, local
    return None, 0, 1, 0


def replica_value(cells: int, steps: int, world_size: int, max_ms: float) -> float:
    """Whole-job cell-steps/s of `world_size` independent replicas timed by
    the slowest rank."""
    return world_size * cells * steps / (max_ms * 1e-3)


def _barrier(dist):
    if dist is not None:
        dist.barrier()


def _max_over_ranks(dist, x: float) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling during the timed region (SM clock, limits, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int, path: Path | None = None):
        self.index = index
        self.proc = None
        self.path = path or Path(os.environ.get("TMPDIR", "/tmp")) / f"cg_clocks_{os.getpid()}.csv"

    def __enter__(self):
        exe = shutil.which("nvidia-smi")
        if exe:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen([exe, f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "100"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            time.sleep(0.2)
            self.proc.send_signal(signal.SIGTERM)
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self):
        if self.proc is None or not self.path.exists():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        pw = [float(r[3]) for r in rows if r[3].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        # samples under load: the upper half of SM clock readings
        load = sorted(sm)[len(sm) // 2:] if sm else []
        return {"sm_mhz": float(np.median(load)) if load else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None, "samples": len(rows), "reasons": reasons}


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _traffic_from_profiles(kernel: str):
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary, or None."""
    f = ROOT / "profiles" / "traffic_per_launch.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        parts = line.split()
        if len(parts) >= 2 and parts[0] == kernel:
            try:
                return float(parts[1])
            except ValueError:
                return None
    return None


SLOTS = ["k_ypass:fwd", "k_xpass:grad", "k_ypass:inv_grad", "k_zpass_u", "k_ypass:fwd_div", "k_xpass:div",
         "k_ypass:inv", "k_zpass_p"]
FAST_SIZES = {8, 16, 24, 32, 48, 64, 96, 128, 160, 192, 256}  # every size-specialised kernel family
FAST_XYZ_SIZES = FAST_SIZES | {320, 400, 512, 640}  # x/y passes and the persistent z-passes only


def slot_symbols(padded3, persistent_z: bool = True, tma: bool = False) -> list[str]:
    """The kernel each step slot launches on this grid (size-specialised where the axis allows);
    ``persistent_z`` and ``tma`` are the autotuner's z-pass choices (lengths without a per-tile
    kernel are always persistent when ny is even; ``tma``: tensor-map staging of the z-tiles)."""
    nx, ny, nz = padded3
    y = f"kf_ypass<{ny},{{}}>" if ny in FAST_XYZ_SIZES else "k_ypass"
    x = f"kf_xpass<{nx},{{}}>" if nx in FAST_XYZ_SIZES else "k_xpass"
    zp = "kfp" if ny % 2 == 0 and (persistent_z or nz not in FAST_SIZES) else "kf"
    zfast = nz in (FAST_XYZ_SIZES if zp == "kfp" else FAST_SIZES)
    tma = bool(tma and zp == "kfp" and zfast)
    zu = (f"{zp}_zpass_u<{nz},true>" if tma else f"{zp}_zpass_u<{nz}>") if zfast else "k_zpass_u"
    # the timed steps do not record: the persistent p-pass runs its record-free instantiation
    zpp = ((f"{zp}_zpass_p<{nz},false,false,true>" if tma else f"{zp}_zpass_p<{nz},false>") if zp == "kfp"
           else f"kf_zpass_p<{nz},1>") if zfast else "k_zpass_p"
    return [y.format("Y_FWD"), x.format("X_GRAD"), y.format("Y_INV_GRAD"), zu, y.format("Y_FWD_DIV"),
            x.format("X_DIV"), y.format("Y_INV"), zpp]


def slot_bytes(ncell: int, nspec: int, labels: bool, nonlinear: bool, record: bool = False) -> list[int]:
    """Algorithmic bytes per launch of each slot: every input read once and
    every output written once in the kernel's own layout."""
    c8 = 8 * nspec
    r4 = 4 * ncell
    maps_u = LABEL_BYTES * ncell if labels else 8 * ncell
    maps_p = LABEL_BYTES * ncell if labels else (12 if nonlinear else 8) * ncell
    rec = 6 * r4 if record else 0
    return [2 * c8, 3 * c8, 5 * c8, 6 * c8 + 6 * r4 + maps_u, 5 * c8, 3 * c8, 2 * c8, 2 * c8 + 2 * r4 + maps_p + rec]


def step_algorithmic_bytes(labels: bool, nonlinear: bool) -> int:
    """Compulsory bytes per cell-step of the whole step (all passes fused):
    80 / 84 B with float32 maps, 66 B with label-indexed maps."""
    if labels:
        return 66
    return 84 if nonlinear else 80


def cpu_sample(job, target_s: float = 12.0, workers: int | None = None, max_steps: int = 200, min_steps: int = 1,
               time_cap: float | None = None):
    """Time the reference's float32 NumPy step (oracle restatement) on this host:
    at least ``min_steps`` and ``target_s`` seconds, at most ``max_steps``
    steps, and never past ``time_cap`` seconds."""
    from caustica_gb300 import engine as eng
    from oracle import kspace as ok

    workers = workers or os.cpu_count() or 1
    grid, med, src, spec = job["grid"], job["medium"], job["source"], job["spec"]
    shape = grid.shape
    spp, dt = eng.cw_discretization(grid.dx, float(med.c.max()), src.f0, spec, job["harmonics"])
    maps = ok.medium_maps(med.alpha, med.rho, med.c, med.beta, shape, dt, job["nonlinear"], np.float32)
    ks = ok.k_vectors(shape, grid.dx, np.float32)
    kap = ok.kappa_sinc(ks, float(med.c.max()), dt, np.float32)
    der = ok.spectral_derivative_factors(ks, kap, shape, np.complex64)
    spg = ok.sponge_volume(shape, grid.pml_vox, 2.0, np.float32)
    rng = np.random.default_rng(0)
    p = (rng.standard_normal(shape) * 1e3).astype(np.float32)
    u = [np.zeros(shape, np.float32) for _ in range(3)]
    import scipy.fft as spfft

    n = 0
    t0 = time.perf_counter()
    with spfft.set_workers(workers):
        while True:
            ok.step_fields(p=p, u=u, dt_over_rho=maps[0], rhoc2_dt=maps[1], absorb=maps[2], beta2_dt=maps[3],
                           sponge=spg, deriv=der, padded=shape)
            n += 1
            el = time.perf_counter() - t0
            if n >= max_steps or (el >= target_s and n >= min_steps):
                break
            if time_cap is not None and el >= time_cap:
                break
    cells = int(np.prod(shape))
    return {"value": cells * n / el, "unit": UNIT, "cores": workers, "kind": "port",
            "sample": f"{n} float32 NumPy/SciPy steps of the {shape[0]}x{shape[1]}x{shape[2]} Westervelt step "
                      f"({el:.1f} s, scipy.fft workers={workers})", "steps": n, "seconds": el}


def workload_config(job) -> dict:
    """The ``config`` keys both arms print for the benchmark workload."""
    from caustica_gb300 import engine as eng

    grid, med, src, spec = job["grid"], job["medium"], job["source"], job["spec"]
    spp, _ = eng.cw_discretization(grid.dx, float(med.c.max()), src.f0, spec, job["harmonics"])
    n_mat = len(np.unique(med.id_map)) if getattr(med, "id_map", None) is not None else None
    return {"workload": job["name"], "grid": list(grid.shape), "cells": int(np.prod(grid.shape)),
            "harmonics": list(job["harmonics"]),
            "medium": f"{n_mat} labels (uint8 map)" if n_mat is not None else "dense float32 maps",
            "source_voxels": int(src.indices.shape[0]), "spp": spp,
            "l2": "inputs larger than L2 (p,u 151 MB + spectra 114 MB > 129 MB L2); no flush"}


def run_reference(args, dist, rank):
    """The reference's CPU step (float32 NumPy/SciPy, all host cores): W
    untimed warm-up steps, then K timed steps, both cut short when the
    sample would outlast its time budget (the line reports the steps run)."""
    from caustica_gb300 import workloads as wl

    if rank != 0:
        return
    job = wl.config2()
    budget = float(os.environ.get("CG_REFERENCE_SECONDS", "45"))
    warm = cpu_sample(job, target_s=0.0, max_steps=max(1, int(args.warmup)), min_steps=max(1, int(args.warmup)),
                      time_cap=budget / 4)
    s = cpu_sample(job, target_s=budget, max_steps=int(args.steps), min_steps=int(args.steps), time_cap=budget)
    cfg = workload_config(job)
    cfg["timing"] = "wall clock of each NumPy/SciPy step on the host cores"
    line = {"impl": "reference", "metric": METRIC, "value": s["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": s["steps"], "warmup": warm["steps"], "steps_requested": int(args.steps),
            "warmup_requested": int(args.warmup), "ms_per_step": 1e3 * s["seconds"] / s["steps"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": cfg,
            "cpu_baseline": {k: s[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "e2e": {"value": s["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line, default=_jsonable), flush=True)


def run_gb300(args, dist, rank, ws, local):
    from caustica_gb300 import _lib
    from caustica_gb300 import engine as eng
    from caustica_gb300 import workloads as wl
    from caustica_gb300.solvers import WesterveltKSpaceGB300

    _lib.load()
    _lib.call("cg_set_device", local)
    job = wl.config2()
    grid, med, src, spec = job["grid"], job["medium"], job["source"], job["spec"]
    plan = eng.make_plan("westervelt_gb300", grid, med, src, spec, nonlinear=True, harmonics=job["harmonics"],
                         reference_point=job["reference_point"])
    ncell = plan.ncell
    K, W = int(args.steps), int(args.warmup)
    graph = K % plan.spp == 0 and W % plan.spp == 0
    dev = eng.DeviceSolver(plan)
    launches_per_step = dev.launches_per_step
    tuning = dev.tuning
    staging_tma = dev.config()["tma_staging"]  # the staging in effect (also without the autotuner)
    try:
        # drive table long enough that the source keeps injecting through the timed steps
        dev.extend_drive((plan.eff_min + 4) * plan.spp + W + 2 * K)
        # run far enough to have a developed field, then warm up
        pre = plan.eff_min if args.prerun_periods is None else int(args.prerun_periods)
        dev.run_periods(pre)
        ms = C_float()
        if W:
            _lib.call("cg_solver_timed_run", dev.h, W, 0, int(graph), ms.ref())
        dev.synchronize()
        _barrier(dist)
        with Clocks(local) as clk:
            _lib.call("cg_solver_timed_run", dev.h, K, 0, int(graph), ms.ref())
        dev.synchronize()
        _barrier(dist)
        t_ms = _max_over_ranks(dist, ms.value)
        value = replica_value(ncell, K, ws, t_ms)
        # per-launch profile (events between launches)
        prof = np.zeros(8, np.float32)
        P = 2 * plan.spp
        _lib.call("cg_solver_profile", dev.h, P, 0, _lib.ptr(prof))
    finally:
        dev.close()

    hbm, peak_kind = _peaks()
    info_labels = plan.labels is not None
    nspec = plan.padded3[0] * (plan.padded3[2] // 2 + 1) * plan.padded3[1]
    bytes_slot = slot_bytes(ncell, nspec, info_labels, True)
    per_launch_ms = prof / P
    dom = int(np.argmax(per_launch_ms))
    achieved = bytes_slot[dom] / (per_launch_ms[dom] * 1e-3) / 1e9
    kernel_name = SLOTS[dom]
    symbols = slot_symbols(plan.padded3, bool((tuning or {}).get("persistent_z", True)), bool(staging_tma))
    traffic = _traffic_from_profiles(kernel_name)
    step_b = step_algorithmic_bytes(info_labels, True)
    step_achieved = step_b * value / ws / 1e9
    passes_achieved = sum(bytes_slot) / (t_ms / K * 1e-3) / 1e9

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": t_ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {**workload_config(job),
                       "timing": "CUDA events on the solver stream, " + ("CUDA graph per period" if graph else
                                                                           "direct launches"),
                       "tuning": tuning},
            "roofline": {"bound": "hbm", "kernel": kernel_name, "kernel_symbol": symbols[dom],
                         "achieved": achieved, "peak": hbm, "unit": "GB/s",
                         "frac": achieved / hbm, "peak_kind": peak_kind, "bytes_per_launch": bytes_slot[dom],
                         "ms_per_launch": float(per_launch_ms[dom]), "traffic": traffic,
                         "traffic_source": None if traffic is None else
                         "profiles/traffic_per_launch.txt: ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                         "this kernel in one config-2 step (committed capture, not measured in this run)"},
            "step_roofline": {"bytes_per_cell_step": step_b, "achieved": step_achieved, "peak": hbm,
                              "frac": step_achieved / hbm, "unit": "GB/s",
                              "note": "algorithmic bytes of the fully fused step with label-indexed maps"},
            "passes_roofline": {"bytes_per_step": int(sum(bytes_slot)), "achieved": passes_achieved, "peak": hbm,
                                "frac": passes_achieved / hbm, "unit": "GB/s",
                                "note": "algorithmic bytes of the 8 passes as built (each input read and output "
                                        "written once per pass) over the graph-timed step"},
            "profile_ms_per_launch": {SLOTS[i]: float(per_launch_ms[i]) for i in range(8)},
            "gpu_launches": K * launches_per_step + (K // plan.spp if graph else 1)}

    # end-to-end: one full solve through the public solver front, host numpy in, host numpy out
    if not args.skip_e2e:
        solver = WesterveltKSpaceGB300()
        solver.run(grid, med, src, spec, harmonics=job["harmonics"], reference_point=job["reference_point"])
        _barrier(dist)
        t0 = time.perf_counter()
        res = solver.run(grid, med, src, spec, harmonics=job["harmonics"], reference_point=job["reference_point"])
        el = _max_over_ranks(dist, time.perf_counter() - t0)
        h2d = (plan.labels.nbytes + plan.label_table.nbytes + plan.src_xyz.nbytes + 8 * plan.src_xyz.shape[0]
               + 16 * plan.max_periods * plan.spp)
        d2h = sum(v.nbytes for v in res.phasors.values()) + res.p_max.nbytes
        e2e_value = ws * ncell * res.steps_total / el
        # the metric's step is one time step: the solve's copies spread over its steps
        line["e2e"] = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d / res.steps_total,
                       "d2h_bytes_per_step": d2h / res.steps_total, "h2d_bytes_per_solve": h2d,
                       "d2h_bytes_per_solve": d2h,
                       "step": f"one full solve ({res.steps_total} time steps, {res.steps_total // plan.spp} periods) "
                               f"through WesterveltKSpaceGB300.run() from host numpy",
                       "seconds": el, "solves_per_s": ws / el}
    if rank == 0 and ws == 1 and not args.skip_e2e and not args.skip_store:
        line["store"] = bench_store(grid, med, src, spec, job)
    if rank == 0 and ws == 1 and not args.skip_batched:
        line["batched"] = bench_batched()
    if rank == 0 and ws == 1 and not args.skip_serving:
        line["serving"] = bench_serving()
    if rank == 0 and ws == 1 and not args.skip_thermal:
        line["thermal"] = bench_thermal()
    if rank == 0 and ws == 1 and not args.skip_cpu:
        cb = cpu_sample(job, target_s=float(os.environ.get("CG_CPU_SECONDS", "12")))
        line["cpu_baseline"] = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        # the same step with one FFT worker (the reference's set_cpu_fft_workers(1), core/backend.py:84-91)
        c1 = cpu_sample(job, target_s=float(os.environ.get("CG_CPU1_SECONDS", "8")), workers=1, max_steps=40)
        line["cpu_baseline_1worker"] = {k: c1[k] for k in ("value", "unit", "cores", "kind", "sample")}
    line["clocks"] = clk.summary()
    if rank == 0:
        print(json.dumps(line, default=_jsonable), flush=True)


def bench_store(grid, med, src, spec, job):
    """Store quantisation of one config-2 result (harmonics 1-3 and p_max:
    seven float32 fields of the record region): the device path inside a
    solve (``store_quantize``: two passes over each field on the GPU, then
    only the float16 bytes to the host) against the reference's host
    ``try_float16`` on the same fields (io/quantize.py:45-67, NumPy, one
    core), which its ``save_result`` runs before writing."""
    from caustica_gb300 import store
    from caustica_gb300.solvers import WesterveltKSpaceGB300
    from oracle import quantize as oq

    solver = WesterveltKSpaceGB300()
    solver.store_quantize = store.DEFAULT_MAX_NORM_ERR
    t0 = time.perf_counter()
    res = solver.run(grid, med, src, spec, harmonics=job["harmonics"], reference_point=job["reference_point"])
    solve_s = time.perf_counter() - t0
    att = res.meta["quantized"]
    fields = oq.store_order(res.phasors, res.p_max)
    t1 = time.perf_counter()
    host = [oq.try_float16(f) for _, f in fields]
    host_s = time.perf_counter() - t1
    same = all(np.array_equal(np.asarray(att["fields"][n].stored).view(np.uint8), np.asarray(h.stored).view(np.uint8))
               and att["fields"][n].scale == h.scale for (n, _), h in zip(fields, host))
    return {"workload": f"{len(fields)} float32 fields of {res.p_max.size} voxels (p_real/p_imag of harmonics "
                        f"{sorted(res.phasors)} and p_max, config 2)",
            "device_s": att["seconds"], "stored_bytes": int(sum(q.stored.nbytes for q in att["fields"].values())),
            "float32_bytes": int(sum(f.nbytes for _, f in fields)),
            "dtypes": sorted({q.dtype_name for q in att["fields"].values()}),
            "solve_with_store_s": solve_s, "equal_to_host": bool(same),
            "cpu_baseline": {"value": host_s, "unit": "s", "cores": 1, "kind": "port",
                             "sample": "try_float16 of the same fields (NumPy)"},
            "timing": "device: wall clock of cg_solver_quantize (both passes, the float16 copy to fresh host "
                      "pages) inside the solve; host: wall clock of the NumPy restatement"}


def bench_batched(n_plain: int = 4):
    """Config 4: 64 steering positions over one medium, plain (one solve per
    call) against batched (all members in one handle), both end to end
    through the public API from host numpy."""
    import time as _t

    from caustica_gb300 import workloads as wl
    from caustica_gb300.batch import solve_steering
    from caustica_gb300.contract import CWSource
    from caustica_gb300.solvers import LinearKSpaceGB300

    job = wl.config4(64)
    grid, med, spec = job["grid"], job["medium"], job["spec"]
    idx, phases = job["source"].indices, job["phases"]
    solver = LinearKSpaceGB300()

    def plain(b):
        src = CWSource(indices=idx, phases=phases[b], amplitude=1e5, f0=1e6)
        return solver.run(grid, med, src, spec, reference_point=job["reference_point"])

    plain(0)  # warm
    t0 = _t.perf_counter()
    for b in range(n_plain):
        r = plain(b)
    t_plain = (_t.perf_counter() - t0) / n_plain
    t0 = _t.perf_counter()
    res = solve_steering(grid, med, idx, phases, f0=1e6, amplitude=1e5, spec=spec,
                         reference_point=job["reference_point"])
    t_batch = _t.perf_counter() - t0
    cells = int(np.prod(grid.shape))
    cell_steps = cells * r.steps_total
    return {"workload": job["name"], "members": len(res), "steps_per_solve": r.steps_total,
            "plain_solves_per_s": 1.0 / t_plain, "batched_solves_per_s": len(res) / t_batch,
            "ratio": (len(res) / t_batch) * t_plain, "batched_cell_steps_per_s": len(res) * cell_steps / t_batch,
            "plain_cell_steps_per_s": cell_steps / t_plain, "plain_sample": f"{n_plain} solves",
            "timing": "wall clock of the public calls (host numpy in, host numpy out)"}


# Pennes + CEM43 sub-step, label medium with q and dose: reads theta, label,
# q, running maximum, dose, dose compensation (4+1+4+4+4+4 B) and writes
# theta', maximum, dose, compensation (4x4 B) per cell.
PENNES_BYTES_PER_CELL = 37


def bench_thermal(shape=(256, 256, 320), seed: int = 7):
    """The heat-up phase a served request carries (400 steps of 0.05 s, dose
    on) on the largest serving grid, q a seeded stand-in for the acoustic
    heating: device time of the sub-steps (CUDA events on the handle's
    stream) and the wall clock of the public call (host numpy in and out)."""
    import time as _t

    from caustica_gb300 import workloads as wl
    from caustica_gb300.thermal import PennesSolverGB300

    th = wl.config5_thermal(shape)
    rng = np.random.default_rng(seed)
    q = (rng.random(shape, dtype=np.float32) * np.float32(1e5)).astype(np.float32)
    t0 = np.full(shape, 37.0, np.float32)
    solver = PennesSolverGB300(on_unstable="substep")
    solver.solve(t0, q, th["medium"], dt=th["dt"], n_steps=10, dose=True)  # warm
    timing: dict = {}
    w0 = _t.perf_counter()
    res = solver.solve(t0, q, th["medium"], dt=th["dt"], n_steps=th["n_heat"], dose=True, timing=timing)
    wall = _t.perf_counter() - w0
    cells = int(np.prod(shape))
    n_sub = int(timing["substeps"])
    ms_sub = timing["device_ms"] / n_sub
    peak, kind = _peaks()
    achieved = cells * PENNES_BYTES_PER_CELL / (ms_sub * 1e-3) / 1e9
    return {"workload": f"pennes_cem43 {shape[0]}x{shape[1]}x{shape[2]} labels+q+dose, {th['n_heat']} steps of "
                        f"{th['dt']} s ({res.substeps} sub-step(s) each)",
            "kernel_symbol": "k_pennes_stream2<1, 1, 0>" if shape[2] % 2 == 0 else "k_pennes_stream<1, 1, 0>",
            "substeps": n_sub, "ms_per_substep": ms_sub, "cell_substeps_per_s": cells / (ms_sub * 1e-3),
            "e2e_cell_substeps_per_s": cells * n_sub / wall, "e2e_seconds": wall,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_kind": kind, "bytes_per_cell": PENNES_BYTES_PER_CELL},
            "timing": "device: CUDA events around each run between finite-guards (guards excluded); "
                      "e2e: wall clock of PennesSolverGB300.solve"}


SERVING_RATES = (0.25, 0.5, 1.0, 2.0, 4.0)  # offered load, multiples of the measured capacity


def serving_point_summary(latencies, wall_s: float, stats: dict, n: int, rate) -> dict:
    """One rate point of the served stream: throughput, latency percentiles and packing."""
    lat = np.asarray(latencies, np.float64)
    return {"offered_rate": rate, "requests": n, "solves_per_s": n / wall_s, "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "wall_s": wall_s, "groups": int(stats["groups"]),
            "mean_pack": n / max(1, int(stats["groups"])), "packed_requests": int(stats.get("packed_in_groups", 0)),
            "solo_reruns": int(stats["solo_reruns"]), "max_active": int(stats["max_active"]),
            "peak_gb": stats["peak_bytes"] / 1e9}


def bench_serving(n_req: int | None = None, seed: int = 5):
    """Config 5: a served request stream. Capacity is measured with every
    request queued at once; then the same requests arrive as Poisson streams
    at 0.25x, 0.5x, 1x, 2x and 4x that capacity. Every point serves all
    ``n_req`` requests (200 by default, ``CG_SERVE_REQUESTS`` overrides)."""
    import time as _t

    from caustica_gb300 import serve
    from caustica_gb300 import workloads as wl

    n_req = int(os.environ.get("CG_SERVE_REQUESTS", "200")) if n_req is None else int(n_req)
    t_build = _t.perf_counter()
    reqs = wl.config5_requests(n_req, seed)
    t_build = _t.perf_counter() - t_build

    def run(rate, subset=None):
        todo = reqs if subset is None else subset
        rng = np.random.default_rng(seed + 1)
        arr = np.zeros(len(todo)) if rate is None else np.cumsum(rng.exponential(1.0 / rate, len(todo)))
        with serve.Server(hbm_budget_bytes=160 << 30, max_active=int(os.environ.get("CG_SERVE_SLOTS", "6"))) as srv:
            t0 = _t.perf_counter()
            futs = []
            for r, ta in zip(todo, arr):
                dt = t0 + ta - _t.perf_counter()
                if dt > 0:
                    _t.sleep(dt)
                futs.append(srv.submit(r))
            outs = [f.result() for f in futs]
            wall = _t.perf_counter() - t0
            stats = dict(srv.stats)
        return serving_point_summary([o.latency_s for o in outs], wall, stats, len(outs), rate)

    # warm: one request of every (grid, physics) kind, so plans, tuned launch
    # configurations and allocator pools exist before anything is timed
    seen, warm = set(), []
    for r in reqs:
        k = (r.tag["shape"], r.tag["nonlinear"], r.tag["thermal"])
        if k not in seen:
            seen.add(k)
            warm.append(r)
    run(None, warm)
    cap = run(None)
    points = [cap] + [run(f * cap["solves_per_s"]) for f in SERVING_RATES]
    shapes: dict = {}
    for r in reqs:
        shapes[str(r.tag["shape"])] = shapes.get(str(r.tag["shape"]), 0) + 1
    return {"requests": len(reqs), "grids": shapes, "thermal": sum(r.tag["thermal"] for r in reqs),
            "westervelt": sum(r.tag["nonlinear"] for r in reqs),
            "reused_media": sum(r.tag.get("reused", False) for r in reqs),
            "capacity_solves_per_s": cap["solves_per_s"], "rates_x_capacity": list(SERVING_RATES),
            "points": points, "request_build_s": t_build,
            "note": f"every point serves all {len(reqs)} requests; the first point queues them all at once (capacity)"}


class C_float:
    def __init__(self):
        import ctypes

        self._v = ctypes.c_float(0.0)

    def ref(self):
        import ctypes

        return ctypes.byref(self._v)

    @property
    def value(self):
        return float(self._v.value)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4400)
    ap.add_argument("--warmup", type=int, default=44)
    ap.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--skip-serving", action="store_true")
    ap.add_argument("--skip-thermal", action="store_true")
    ap.add_argument("--skip-store", action="store_true")
    ap.add_argument("--prerun-periods", type=int, default=None,
                    help="periods run before the warm-up (default: the settle floor of the workload)")
    args = ap.parse_args()
    if args.warmup < 3:
        raise SystemExit("--warmup must be >= 3")
    dist, rank, ws, local = _dist()
    try:
        if args.impl == "reference":
            run_reference(args, dist, rank)
        else:
            run_gb300(args, dist, rank, ws, local)
    finally:
        if dist is not None:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()

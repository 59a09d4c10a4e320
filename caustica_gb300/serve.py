"""Continuous-batching request loop for CW solves (with optional thermal phase).

Requests arrive at any time (``Server.submit`` returns a future). A
scheduler thread

* admits pending requests while their device footprint fits the HBM budget
  (the estimate of ``engine.device_footprint``, the same inventory the
  reference planner keeps, planner/model.py:86-115),
* packs compatible pending requests -- same grid, medium, source voxels,
  drive, schedule and record region -- into one batched solver handle (one
  launch per pass for all members),
* keeps every admitted handle on its own CUDA stream and advances each one
  with non-blocking stream queries, so the work of different requests
  overlaps on the GPU and a request that arrives while others run is
  admitted as soon as memory frees,
* follows the reference's settle / record schedule per request
  (solvers/kspace/engine.py:484-557): periods are queued ahead as far as no
  convergence decision needs a period peak,
* computes each request's focal metrics (report/metrics.py:192-313) and,
  for a request with a thermal phase, its heating Q = sum alpha_n |P_n|^2 /
  (rho c) (sensors.py:259-273) on the device from the handle's phasors,
* runs the attached Pennes / CEM43 phase (thermal/pennes.py:451-689) on a
  worker thread from that device Q: the field does not travel through the
  host between the acoustic and the thermal solve.

Each request's result is the one the plain solver returns for it alone: a
packed member whose own convergence decisions differ from the shared
schedule is solved again on its own (``engine.member_schedule``).
"""

from __future__ import annotations

import hashlib
import queue
import threading
import time
from collections import deque
from concurrent.futures import Future
from dataclasses import dataclass, field
from math import ceil
from typing import Any

import numpy as np

from ._lib import DeviceArray
from .contract import CWRunSpec
from .engine import DeviceSolver, _guard_finite, _results, device_footprint, make_plan, member_schedule


@dataclass
class Request:
    grid: Any
    medium: Any
    source: Any
    spec: CWRunSpec
    nonlinear: bool = False
    harmonics: tuple = (1,)
    record_region: tuple | None = None
    reference_point: tuple | None = None
    # {"medium", "dt", "n_heat", "n_cool", "T0", "q_scale", "harmonics", "alpha_power_law_y"}
    thermal: dict | None = None
    frame: Any = None  # a metrics.FieldFrame: focal metrics are computed when given
    # a bound on the relative round-trip error: the result store's float16
    # fields are quantised on the device as well (result.meta["quantized"])
    store_quantize: float | None = None
    tag: Any = None


@dataclass
class Outcome:
    result: Any
    thermal: Any
    t_submit: float
    t_admit: float
    t_done: float
    group_size: int
    member: int
    metrics: dict | None = None

    @property
    def latency_s(self) -> float:
        return self.t_done - self.t_submit


_MEDIA = ("alpha", "rho", "c", "beta")
_FP_CACHE: dict = {}  # id(medium) -> (medium, fingerprint); holds the object, so its id stays unique
_FP_STRIDE = 61


def medium_fingerprint(medium) -> str:
    """A content fingerprint of a medium: shape plus a strided sample of its
    four maps. Equal media always get equal fingerprints; two requests whose
    fingerprints match share a handle only after :func:`same_medium`
    compares the whole maps."""
    hit = _FP_CACHE.get(id(medium))
    if hit is not None and hit[0] is medium:
        return hit[1]
    h = hashlib.sha1()
    for name in _MEDIA:
        a = np.ascontiguousarray(getattr(medium, name), np.float32)
        h.update(str(a.shape).encode())
        h.update(a.reshape(-1)[::_FP_STRIDE].tobytes())
    fp = h.hexdigest()
    _FP_CACHE[id(medium)] = (medium, fp)
    while len(_FP_CACHE) > 64:
        _FP_CACHE.pop(next(iter(_FP_CACHE)))
    return fp


def same_medium(a, b) -> bool:
    """Bitwise equality of two media's maps (the same object trivially)."""
    if a is b:
        return True
    return all(np.array_equal(np.asarray(getattr(a, n), np.float32), np.asarray(getattr(b, n), np.float32))
               for n in _MEDIA)


def _key(req: Request) -> tuple:
    """Requests with equal keys (and equal media, :func:`same_medium`) can
    share one batched handle: media are compared by content, so two
    requests that carry equal media built separately pack as well. The key
    is kept on the request after its first use."""
    cached = req.__dict__.get("_cg_key")
    if cached is not None:
        return cached
    key = _make_key(req)
    req.__dict__["_cg_key"] = key
    return key


def _make_key(req: Request) -> tuple:
    src = req.source
    h = hashlib.sha1(np.ascontiguousarray(src.indices).tobytes()).hexdigest()
    spec = req.spec
    sk = tuple(sorted((spec.model_dump() if hasattr(spec, "model_dump") else dict(spec.__dict__)).items()))
    rr = None if req.record_region is None else tuple((s.start, s.stop) for s in req.record_region)
    return (medium_fingerprint(req.medium), tuple(req.grid.shape), req.grid.dx, req.grid.pml_vox, float(src.f0),
            float(src.amplitude), float(src.ramp_periods), h, sk, bool(req.nonlinear), tuple(req.harmonics), rr,
            None if req.reference_point is None else tuple(req.reference_point))


class _Group:
    """One admitted handle: B packed requests following one schedule."""

    def __init__(self, plan, items, t_admit):
        self.plan = plan
        self.items = items  # [(req, future, t_submit)]
        self.t_admit = t_admit
        phases = np.stack([np.asarray(r.source.phases, np.float32) for r, _, _ in items])
        self.phases = phases
        self.dev = DeviceSolver(plan, batch=len(items), phases=phases)
        self.bytes = device_footprint(plan, len(items))
        spec = plan.spec
        self.stage = "settle"
        self.launched = 0  # settle periods queued
        self.decided = 0  # settle periods whose peaks were read
        self.prev = None
        self.converged = False
        self.converged_period = plan.eff_max
        self.history = []
        self.peaks = []
        self.periods_done = 0
        self.tol = spec.convergence_tol
        self._queue_settle()

    def _queue_settle(self):
        p = self.plan
        if self.tol > 0:
            target = max(self.decided + 1, min(p.eff_max, p.eff_min))
        else:
            target = p.eff_max
        if self.launched < target:
            self.dev.run_periods(target - self.launched)
            self.launched = target

    def advance(self) -> bool:
        """Move the schedule forward if the stream is idle; True when finished."""
        if not self.dev.idle():
            return False
        p = self.plan
        spec = p.spec
        if self.stage == "settle":
            new = self.launched - self.decided
            pk = self.dev.read_peaks(self.decided, new)
            for j in range(new):
                self.decided += 1
                self.peaks.append(pk[:, j].copy())
                peak = float(pk[0, j])
                _guard_finite(peak, f"settling period {self.decided}", p.name)
                rel = abs(peak - self.prev) / max(self.prev, 1e-9) if self.prev is not None else None
                if self.decided >= p.tof:
                    self.history.append((self.decided, peak, float("nan") if rel is None else rel))
                if self.decided >= p.eff_min and rel is not None and peak > 0.0 and rel < self.tol:
                    self.converged = True
                    self.converged_period = self.decided
                    break
                self.prev = peak
            self.periods_done = self.decided
            if not self.converged and self.decided < p.eff_max:
                self._queue_settle()
                return False
            if spec.t_end_min_us is not None:
                need = ceil(spec.t_end_min_us * 1e-6 / p.period) - spec.n_record_periods
                if self.periods_done < need:
                    self.dev.run_periods(need - self.periods_done)
                    self.periods_done = need
            self.dev.begin_record()
            self.dev.run_periods(spec.n_record_periods, record=True)
            self.stage = "record"
            return False
        if self.stage == "record":
            return True
        return True

    def finish(self):
        """Results per member (None for a member that must be solved alone)."""
        p = self.plan
        spec = p.spec
        rec_steps = spec.n_record_periods * p.spp
        ph, pm = self.dev.finalize(rec_steps)
        n = (self.periods_done + spec.n_record_periods) * p.spp
        peaks = np.array(self.peaks).T if self.peaks else np.zeros((len(self.items), 0), np.float32)
        out = []
        for b in range(len(self.items)):
            if b == 0:
                sched = (self.decided, self.converged, self.converged_period, self.history)
            else:
                sched = member_schedule(peaks[b], p)
                if sched[0] != self.decided or sched[1] != self.converged:
                    out.append(None)
                    continue
            _guard_finite(float(pm[b].max()), f"the record window (step {n})", p.name)
            common = dict(dt=p.dt, spp=p.spp, steps_total=n, t_end_s=n * p.dt, tof_periods=p.tof,
                          converged_period=sched[2], settle_capped=not sched[1], convergence_history=sched[3],
                          meta={"solver": p.name, "backend": "gb300", "padded_shape": p.padded, "c_ref": p.c_max,
                                "nonlinear_active": p.nonlinear_active, "batch": len(self.items), "member": b})
            res = _results(p, self.dev, ph, pm, common, b, _result_cls())
            out.append((res, *_post_process(self.dev, b, res, self.items[b][0])))
        self.dev.close()
        return out


def _result_cls():
    from .contract import SolverResult

    return SolverResult


def _post_process(dev, member: int, result, req: Request):
    """Focal metrics, heating Q and store fields of one member from the handle's device phasors."""
    from .metrics import device_focus_metrics
    from .sensors import HeatingSource

    metrics = None
    if req.frame is not None:
        metrics = device_focus_metrics(dev, member, result, req.frame, source_amplitude=float(req.source.amplitude),
                                       medium=req.medium)
    if req.store_quantize is not None:
        from .store import quantize_solver

        result.meta["quantized"] = {"max_norm_err": float(req.store_quantize),
                                    "fields": quantize_solver(dev, member, req.store_quantize)}
    heating = None
    if req.thermal is not None:
        th = req.thermal
        heating = HeatingSource.from_solver(dev, member, result, req.medium, req.grid.dx,
                                            harmonics=tuple(th.get("harmonics", (1,))),
                                            alpha_power_law_y=th.get("alpha_power_law_y"),
                                            scale=float(th.get("q_scale", 1.0)))
    return metrics, heating


def run_thermal(req: Request, result, heating=None) -> Any:
    """The attached heat-up + cool-down Pennes phases with the dose chained.

    ``heating`` is the request's device Q on the grid (``_post_process``);
    without it Q is formed on the device from ``result``'s phasors.
    """
    from .sensors import HeatingSource
    from .thermal import PennesSolverGB300, ThermalResult

    th = req.thermal
    if heating is None:
        heating = HeatingSource.from_result(result, req.medium, req.grid.dx,
                                            harmonics=tuple(th.get("harmonics", (1,))),
                                            alpha_power_law_y=th.get("alpha_power_law_y"),
                                            grid_shape=tuple(req.grid.shape), scale=float(th.get("q_scale", 1.0)))
    tmed = th["medium"]
    t0 = th.get("T0")
    if t0 is None:
        t0 = np.full(tmed.shape, 37.0, np.float32)
    solver = PennesSolverGB300(on_unstable="substep")
    try:
        hot = solver.solve(t0, heating, tmed, dt=th["dt"], n_steps=th["n_heat"], dose=True)
    finally:
        heating.close()
    if th.get("n_cool", 0):
        cool = solver.solve(hot.temperature, None, tmed, dt=th["dt"], n_steps=th["n_cool"], dose=True,
                            dose0=hot.dose_cem43)
        return ThermalResult.chain([hot, cool])
    return hot


class Server:
    """Continuous-batching CW solve server on one GPU."""

    def __init__(self, hbm_budget_bytes: int | None = None, max_pack: int = 8, poll_s: float = 2e-4,
                 thermal_workers: int = 3, max_active: int = 6, plan_workers: int = 4, device: int = 0):
        if hbm_budget_bytes is None:
            hbm_budget_bytes = 200 << 30
        self.budget = int(hbm_budget_bytes)
        self.max_pack = int(max_pack)
        # solver handles advancing at once: a few keep the GPU busy; many more
        # only time-slice it and spread each request's latency
        self.max_active = max(1, int(max_active))
        # host set-up of a request (its plan: labels, tables, drive) runs on a
        # small pool as soon as it is submitted, off the scheduler thread
        from concurrent.futures import ThreadPoolExecutor

        # every thread of the server works on `device` (the CUDA device is per thread)
        self.device = int(device)
        self._planner = ThreadPoolExecutor(max(1, int(plan_workers)), thread_name_prefix="cg-plan",
                                           initializer=self._bind_device)
        self._planning: dict = {}
        self._plans_lock = threading.Lock()
        self.poll_s = float(poll_s)
        self._pending: deque = deque()
        self._lock = threading.Condition()
        self._stop = False
        self._active: list[_Group] = []
        self._in_use = 0
        self._plans: dict = {}
        self._thermal_q: queue.Queue = queue.Queue()
        self.stats = {"groups": 0, "packed_members": 0, "packed_in_groups": 0, "solo_reruns": 0, "peak_bytes": 0,
                      "max_active": 0}
        self._thread = threading.Thread(target=self._loop, name="cg-serve", daemon=True)
        # thermal phases run on their own handles and streams, so several overlap on the GPU
        self._tworkers = [threading.Thread(target=self._thermal_loop, name=f"cg-thermal-{i}", daemon=True)
                          for i in range(max(1, int(thermal_workers)))]
        self._thread.start()
        for t in self._tworkers:
            t.start()

    # -------------------------------------------------------------- api --
    def submit(self, req: Request) -> Future:
        fut: Future = Future()
        ts = time.perf_counter()
        with self._lock:
            self._planning[id(req)] = self._planner.submit(self._plan, req)
            self._pending.append((req, fut, ts))
            self._lock.notify()
        return fut

    def close(self, wait: bool = True) -> None:
        with self._lock:
            self._stop = True
            self._lock.notify()
        if wait:
            self._thread.join()
            for _ in self._tworkers:
                self._thermal_q.put(None)
            for t in self._tworkers:
                t.join()
            self._planner.shutdown(wait=True)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------ worker --
    def _plan(self, req: Request):
        k = _key(req)
        with self._plans_lock:
            hit = self._plans.get(k)
        if hit is not None and same_medium(hit[0], req.medium):
            return k, hit[1]
        plan = make_plan("serve_gb300", req.grid, req.medium, req.source, req.spec,
                         record_region=req.record_region, reference_point=req.reference_point,
                         nonlinear=req.nonlinear, harmonics=req.harmonics)
        if plan.labels is not None and plan.labels_dev is None:
            # the medium's label map stays on the device with the cached plan:
            # every handle built from it copies device to device
            plan.labels_dev = DeviceArray.from_host(plan.labels)
        with self._plans_lock:
            self._plans[k] = (req.medium, plan)
            if len(self._plans) > 32:
                self._plans.pop(next(iter(self._plans)))
        return k, plan

    def _admit(self) -> None:
        while True:
            if len(self._active) >= self.max_active:
                return  # every slot busy: wait for one to finish
            with self._lock:
                if not self._pending:
                    return
                req, fut, ts = self._pending[0]
                pf = self._planning.get(id(req))
            if pf is not None and not pf.done():
                return  # the head request's host set-up is still running
            try:
                key, plan = pf.result() if pf is not None else self._plan(req)
            except Exception as exc:  # noqa: BLE001 - a bad request fails alone
                with self._lock:
                    self._pending.popleft()
                    self._planning.pop(id(req), None)
                fut.set_exception(exc)
                continue
            with self._lock:
                items = [self._pending.popleft()]
                rest = deque()
                while self._pending and len(items) < self.max_pack:
                    it = self._pending.popleft()
                    fits = _key(it[0]) == key and same_medium(it[0].medium, req.medium)
                    (items if fits else rest).append(it)
                rest.extend(self._pending)
                self._pending = rest
                for it in items:  # members share the head's plan
                    done = self._planning.pop(id(it[0]), None)
                    if done is not None and it[0] is not req:
                        done.cancel()
            need = device_footprint(plan, len(items))
            while len(items) > 1 and self._in_use + need > self.budget:
                with self._lock:
                    self._pending.appendleft(items.pop())
                need = device_footprint(plan, len(items))
            if self._in_use + need > self.budget and self._active:
                with self._lock:
                    for it in reversed(items):
                        self._pending.appendleft(it)
                return  # wait for memory to free
            try:
                g = _Group(plan, items, time.perf_counter())
            except Exception as exc:  # noqa: BLE001
                for _, f, _ in items:
                    f.set_exception(exc)
                continue
            self._active.append(g)
            self._in_use += g.bytes
            self.stats["groups"] += 1
            self.stats["packed_members"] += len(items)
            if len(items) > 1:
                self.stats["packed_in_groups"] += len(items)
            self.stats["peak_bytes"] = max(self.stats["peak_bytes"], self._in_use)
            self.stats["max_active"] = max(self.stats["max_active"], len(self._active))

    def _complete(self, g: _Group) -> None:
        try:
            results = g.finish()
        except Exception as exc:  # noqa: BLE001
            for _, f, _ in g.items:
                f.set_exception(exc)
            return
        finally:
            self._in_use -= g.bytes
        t = time.perf_counter()
        for b, ((req, fut, ts), out) in enumerate(zip(g.items, results)):
            if out is None:
                self.stats["solo_reruns"] += 1
                solo_req = Request(**{k: v for k, v in req.__dict__.items() if not k.startswith("_")})
                with self._lock:
                    self._pending.appendleft((solo_req, fut, ts))
                continue
            res, metrics, heating = out
            oc = Outcome(result=res, thermal=None, t_submit=ts, t_admit=g.t_admit, t_done=t,
                         group_size=len(g.items), member=b, metrics=metrics)
            if req.thermal is not None:
                self._thermal_q.put((req, fut, oc, heating))
            else:
                fut.set_result(oc)

    def _bind_device(self) -> None:
        from . import _lib

        _lib.call("cg_set_device", self.device)

    def _loop(self) -> None:
        self._bind_device()
        while True:
            with self._lock:
                if self._stop and not self._pending and not self._active:
                    return
            self._admit()
            progressed = False
            for g in list(self._active):
                try:
                    done = g.advance()
                except Exception as exc:  # noqa: BLE001
                    self._active.remove(g)
                    self._in_use -= g.bytes
                    g.dev.close()
                    for _, f, _ in g.items:
                        f.set_exception(exc)
                    progressed = True
                    continue
                if done:
                    self._active.remove(g)
                    self._complete(g)
                    progressed = True
            if not progressed:
                with self._lock:
                    if not self._pending and not self._active and not self._stop:
                        self._lock.wait(0.05)
                        continue
                time.sleep(self.poll_s)

    def _thermal_loop(self) -> None:
        self._bind_device()
        while True:
            item = self._thermal_q.get()
            if item is None:
                return
            req, fut, oc, heating = item
            try:
                oc.thermal = run_thermal(req, oc.result, heating)
                oc.t_done = time.perf_counter()
                fut.set_result(oc)
            except Exception as exc:  # noqa: BLE001
                fut.set_exception(exc)

"""Continuous-batching request loop over the many-domain batch.

Solve requests (a seeded perturbed-icosphere obstacle, a grid, a Reynolds
number) arrive as a Poisson process. The loop admits a request when a slot
and device memory are free (the domain's footprint counted against an HBM
budget), voxelizes its mesh on the GPU, creates the domain resident on the
device and attaches it to the running batch, so new requests overlap on the
GPU with those already running. Every `check_every` of its own steps a domain
reports its drag coefficient from the control-volume momentum balance; it is
retired when Cd changed by less than `tol` (relative) since the previous
check, or at `max_steps`. Latency is arrival to retirement.

A request can be cancelled at any time (`Server.cancel`, from any thread or
from the `on_check` callback): a waiting request is dropped, a running one
leaves the batch after the chunk in flight. Every finished or cancelled
request can be written as one JSON line (`Server(log=...)`): its step count,
Cd and the Cd readings so far, latency, and its lattice updates and
algorithmic bytes per second over its time in the batch.

A domain's trajectory does not depend on the other members of the batch
(include/aeros_batch.h), and checks fall on the same own-step counts whatever
the mix, so a request gives the same Cd, the same step count and the same
fields alone as under load.

The reference has no request loop; this module has no reference counterpart.
"""
from __future__ import annotations

import dataclasses
import json
import math
import queue
import threading
import time

import numpy as np

from . import capi, geometry
from .batch import Batch
from .solver import Solver, voxel_grid, voxelize

SERVE_GRIDS = ((48, 48, 48), (96, 48, 48), (128, 64, 64), (192, 96, 96), (256, 128, 128))
# geodesic sphere frequencies: 20 n^2 triangles, 20,480 (n = 32) to 499,280 (n = 158)
SERVE_FREQS = (32, 158)
# Algorithmic bytes of one cell update: 19 populations read and written, the
# previous and current velocity (3 floats each) and the one-byte solid mask.
BYTES_PER_CELL = {"fp16": 101, "bf16": 101, "fp32": 177}


@dataclasses.dataclass
class Request:
    rid: int
    arrival: float          # seconds after the start of the session
    grid: tuple
    freq: int               # mesh: perturbed geodesic sphere of 20 freq^2 triangles
    re: float
    seed: int


@dataclasses.dataclass
class Result:
    rid: int
    arrival: float
    admitted: float         # memory reserved, preparation queued
    finished: float
    steps: int
    cd: float
    converged: bool
    cells: int
    tris: int
    footprint: int
    started: float = float("nan")   # attached to the batch (nan: never ran)
    cancelled: bool = False
    cd_trace: list = dataclasses.field(default_factory=list)   # (own step, Cd) at every reading
    storage: str = "fp16"

    @property
    def latency(self) -> float:
        return self.finished - self.arrival

    @property
    def mlups(self) -> float:
        """The request's own cell updates per second of its time in the batch
        (its share of the GPU while it ran beside the others)."""
        t = self.finished - self.started
        return self.cells * self.steps / t / 1e6 if self.steps and t > 0 else 0.0

    @property
    def gbs(self) -> float:
        """Algorithmic bytes per second of the request's own updates."""
        return self.mlups * 1e6 * BYTES_PER_CELL.get(self.storage, 101) / 1e9

    def json_line(self) -> str:
        """One JSON line describing the solve."""
        r = lambda v, n=4: round(v, n) if math.isfinite(v) else None   # noqa: E731
        return json.dumps({
            "rid": self.rid, "status": "cancelled" if self.cancelled else ("converged" if self.converged else "capped"),
            "steps": self.steps, "cells": self.cells, "triangles": self.tris, "storage": self.storage,
            "cd": r(self.cd, 6), "cd_trace": [[k, r(c, 6)] for k, c in self.cd_trace],
            "latency_s": r(self.latency), "queued_s": r(self.admitted - self.arrival),
            "mlups": round(self.mlups, 1), "gbs": round(self.gbs, 1), "footprint_bytes": self.footprint})


def make_requests(n: int, rate: float = 2.0, seed: int = 0x5E12, grids=SERVE_GRIDS, freqs=SERVE_FREQS,
                  re_range=(50.0, 1000.0)) -> list[Request]:
    """n requests with exponential inter-arrival gaps of mean 1/rate (seeded);
    grid uniform over `grids`, mesh frequency uniform over the integers of
    `freqs` (inclusive), Re ~ U(re_range)."""
    g = geometry.splitmix64(seed)
    t = 0.0
    out = []
    for i in range(n):
        u = geometry.uniform(g, 0.0, 1.0)
        t += -math.log(max(1.0 - u, 1e-300)) / rate
        grid = grids[min(len(grids) - 1, int(geometry.uniform(g, 0.0, float(len(grids)))))]
        nf = freqs[1] - freqs[0] + 1
        freq = freqs[0] + min(nf - 1, int(geometry.uniform(g, 0.0, float(nf))))
        re = geometry.uniform(g, re_range[0], re_range[1])
        out.append(Request(i, t, grid, freq, re, 0xA0000 + i))
    return out


def domain_for(req: Request, storage="fp16", u_in=0.05, smag=0.1):
    """Solver, drag box and reference area of a request: obstacle of radius
    ny/8 at (nx/3, ny/2, nz/2) (vertex radii x U(0.85, 1.15), axis scales
    U(0.5, 1.5)), voxelized on the GPU; tau = 0.5 + 3 u ny / Re (the solver
    raises tau < 0.51 to 0.55, aeros/src/lbm.cpp:918-920); TRT + Smagorinsky,
    zero-gradient outlet, free-slip lateral walls."""
    nx, ny, nz = req.grid
    r = ny / 8.0
    c = (nx / 3.0, ny / 2.0, nz / 2.0)
    tris = geometry.perturbed_geodesic(req.freq, r, c, seed=req.seed)
    mask = voxelize(tris, voxel_grid((nx, ny, nz), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)))
    tau = 0.5 + 3.0 * u_in * ny / req.re
    p = capi.make_params(nx, ny, nz, tau=tau, smagorinsky_c=smag, les=True, trt=True, u_in=(u_in, 0.0, 0.0),
                         vel_scale=1.0 / u_in, storage=storage, lateral_bc=capi.AEROS_LATERAL_FREESLIP,
                         outlet_bc=capi.AEROS_OUTLET_ZEROGRAD)
    s = Solver(p, mask)
    ext = 1.5 * 1.15 * r + 2.0   # largest half extent of the obstacle + 2 cells
    box = [max(1, int(c[0] - ext)), min(nx - 2, int(c[0] + ext) + 1),
           max(1, int(c[1] - ext)), min(ny - 2, int(c[1] + ext) + 1),
           max(1, int(c[2] - ext)), min(nz - 2, int(c[2] + ext) + 1)]
    area = s.projected_area(0)
    return s, box, area, len(tris), u_in


# Device memory the library holds in every context that loads it, whether or
# not it is used: the fixed 24 MiB array of the no-allocation voxelizer.
LIBRARY_STATIC_BYTES = 24 << 20


def footprint_estimate(req: Request, storage="fp16") -> int:
    """Device bytes of a request before it is created: per cell populations
    (19 x 2 or 4 B), descriptor, two velocity buffers, rho / |S| / TKE and the
    voxelizer's mask; per triangle the device BVH copy."""
    nx, ny, nz = req.grid
    cells = nx * ny * nz
    pop = 19 * (2 if storage != "fp32" else 4)
    tris = 20 * req.freq * req.freq
    return int(cells * (pop + 4 + 32 + 12 + 4) + tris * 96 + (64 << 20))


class _Active:
    __slots__ = ("req", "solver", "box", "area", "u", "tris", "admitted", "started", "steps", "cd_prev", "cd",
                 "bytes", "trace")


class Server:
    """Continuous batching: admission by slots and HBM footprint, domain
    preparation (mesh, GPU voxelization, domain creation) on a worker thread
    while the batch steps, Cd-convergence retirement, cancellation.

    log: a writable text file; one JSON line per finished or cancelled
    request (`Result.json_line`), flushed as it is written."""

    def __init__(self, storage="fp16", budget_bytes=170 << 30, slots=64, check_every=1000, tol=1e-4,
                 max_steps=30000, chunk=100, log=None):
        if check_every % chunk or chunk % 2:
            raise ValueError("chunk must be even and divide check_every")
        self.storage = storage
        self.budget = int(budget_bytes) - LIBRARY_STATIC_BYTES
        self.slots = int(slots)
        self.check_every = int(check_every)
        self.tol = float(tol)
        self.max_steps = int(max_steps)
        self.chunk = int(chunk)
        self.log = log
        self._lock = threading.Lock()
        self._cancel: set = set()

    def cancel(self, rid: int) -> None:
        """Cancels request rid (safe from any thread). It takes effect at the
        next chunk boundary of the running `run`, or of the next `run` if none
        is running: a waiting or preparing request never runs, a running one
        leaves the batch with the steps it has made. Its result is marked
        cancelled and counts in no throughput or latency figure."""
        with self._lock:
            self._cancel.add(int(rid))

    def _take_cancelled(self) -> set:
        with self._lock:
            out, self._cancel = self._cancel, set()
        return out

    def _cd(self, a: _Active) -> float:
        F = a.solver.cv_force_box(a.box)
        return float(F[0] / (0.5 * a.u * a.u * a.area)) if a.area > 0 else float("nan")

    def _prepare(self, todo: queue.Queue, done: queue.Queue) -> None:
        while True:
            item = todo.get()
            if item is None:
                return
            req, est, t_adm = item
            try:
                done.put((req, est, t_adm, domain_for(req, self.storage)))
            except Exception as e:   # reported on the serving thread
                done.put((req, est, t_adm, e))

    def run(self, requests: list[Request], realtime: bool = True, on_retire=None, on_check=None) -> dict:
        """Serves the requests; returns per-request results and the summary.
        realtime=False admits each request at once (no waiting for arrivals).
        on_retire(result, solver): a request converged or reached max_steps.
        on_check(rid, steps, cd): a Cd reading of a running request."""
        pending = sorted(requests, key=lambda r: r.arrival)
        batch = Batch(self.storage)
        batch.set_tuning(chunk_steps=self.chunk)
        todo: queue.Queue = queue.Queue()
        done: queue.Queue = queue.Queue()
        worker = threading.Thread(target=self._prepare, args=(todo, done), daemon=True)
        worker.start()
        active: list[_Active] = []
        results: list[Result] = []
        used = 0
        preparing = 0
        cell_steps = 0
        t0 = time.perf_counter()
        now = lambda: time.perf_counter() - t0   # noqa: E731
        cancelled: set = set()   # cancellations not yet applied

        def finish(res: Result) -> None:
            results.append(res)
            if self.log is not None:
                self.log.write(res.json_line() + "\n")
                self.log.flush()

        def attach(item):
            nonlocal used, preparing
            req, est, t_adm, built = item
            preparing -= 1
            if isinstance(built, Exception):
                used -= est
                raise built
            if req.rid in cancelled:   # cancelled while it was being prepared
                cancelled.discard(req.rid)
                used -= est
                built[0].close()
                finish(Result(req.rid, req.arrival, t_adm, now(), 0, float("nan"), False, req.grid[0] * req.grid[1]
                              * req.grid[2], built[3], est, cancelled=True, storage=self.storage))
                return
            a = _Active()
            a.req = req
            a.admitted = t_adm
            a.solver, a.box, a.area, a.tris, a.u = built
            a.bytes = max(est, a.solver.device_bytes())
            used += a.bytes - est
            a.steps = 0
            a.cd_prev = a.cd = float("nan")
            a.trace = []
            batch.add(a.solver)
            a.started = now()
            active.append(a)

        def apply_cancellations():
            nonlocal used
            cancelled.update(self._take_cancelled())
            if not cancelled:
                return
            for req in [r for r in pending if r.rid in cancelled]:
                pending.remove(req)
                cancelled.discard(req.rid)
                t = now()
                finish(Result(req.rid, req.arrival, t, t, 0, float("nan"), False, req.grid[0] * req.grid[1]
                              * req.grid[2], 20 * req.freq * req.freq, 0, cancelled=True, storage=self.storage))
            for a in [a for a in active if a.req.rid in cancelled]:
                cancelled.discard(a.req.rid)
                batch.remove(a.solver)
                res = Result(a.req.rid, a.req.arrival, a.admitted, now(), a.steps, a.cd, False, a.solver.n, a.tris,
                             a.bytes, started=a.started, cancelled=True, cd_trace=a.trace, storage=self.storage)
                a.solver.close()
                used -= a.bytes
                active.remove(a)
                finish(res)

        try:
            while pending or active or preparing:
                apply_cancellations()
                # admission: arrived requests in order while a slot and memory are free
                while pending and (not realtime or pending[0].arrival <= now()) \
                        and len(active) + preparing < self.slots:
                    est = footprint_estimate(pending[0], self.storage)
                    if used + est > self.budget and (active or preparing):
                        break
                    req = pending.pop(0)
                    used += est
                    preparing += 1
                    todo.put((req, est, now()))
                while not done.empty():
                    attach(done.get())
                if not active:
                    if preparing:
                        attach(done.get())
                    elif pending:
                        time.sleep(max(0.0, min(0.05, pending[0].arrival - now())))
                    continue
                batch.step(self.chunk)
                cell_steps += sum(a.solver.n for a in active) * self.chunk
                retired = []
                for a in active:
                    a.steps += self.chunk
                    if a.steps % self.check_every == 0:
                        a.cd_prev, a.cd = a.cd, self._cd(a)
                        a.trace.append((a.steps, a.cd))
                        if on_check is not None:
                            on_check(a.req.rid, a.steps, a.cd)
                        conv = (math.isfinite(a.cd) and math.isfinite(a.cd_prev) and a.cd != 0.0
                                and abs(a.cd - a.cd_prev) < self.tol * abs(a.cd))
                        if conv or a.steps >= self.max_steps:
                            retired.append((a, conv))
                for a, conv in retired:
                    batch.remove(a.solver)
                    res = Result(a.req.rid, a.req.arrival, a.admitted, now(), a.steps, a.cd, conv,
                                 a.solver.n, a.tris, a.bytes, started=a.started, cd_trace=a.trace,
                                 storage=self.storage)
                    if on_retire is not None:
                        on_retire(res, a.solver)
                    a.solver.close()
                    used -= a.bytes
                    active.remove(a)
                    finish(res)
        finally:
            todo.put(None)
            worker.join()
            while not done.empty():
                item = done.get()
                if not isinstance(item[3], Exception):
                    item[3][0].close()
            for a in active:
                batch.remove(a.solver)
                a.solver.close()
            batch.close()
        wall = now()
        return {"results": sorted(results, key=lambda r: r.rid), "summary": summarize(results, wall, cell_steps)}


def summarize(results: list[Result], wall: float, cell_steps: int) -> dict:
    """Throughput and latency over the requests that ran to their end
    (cancelled ones are counted apart); cell_steps counts every update made."""
    n_cancel = sum(r.cancelled for r in results)
    results = [r for r in results if not r.cancelled]
    lat = np.array([r.latency for r in results], np.float64)
    pct = (lambda q: float(np.percentile(lat, q))) if len(lat) else (lambda q: float("nan"))
    return {"requests": len(results), "cancelled": int(n_cancel), "converged": int(sum(r.converged for r in results)),
            "wall_s": round(wall, 3), "solves_per_hour": round(3600.0 * len(results) / wall, 1) if wall > 0 else 0.0,
            "converged_per_hour": round(3600.0 * sum(r.converged for r in results) / wall, 1) if wall > 0 else 0.0,
            "p50_s": round(pct(50), 3), "p95_s": round(pct(95), 3), "p99_s": round(pct(99), 3),
            "mlups": round(cell_steps / wall / 1e6, 1) if wall > 0 else 0.0,
            "steps_total": int(sum(r.steps for r in results))}


def sequential_plain(requests: list[Request], storage: str = "fp32", check_every: int = 1000, tol: float = 1e-4,
                     max_steps: int = 30000) -> dict:
    """The same requests solved one at a time in plain FP32, each to its own
    end by the serving loop's rule (Cd every check_every steps, retired when
    it changes by less than tol, or at max_steps): mesh, GPU voxelization,
    domain creation and stepping of one request, then the next. Measured
    wall time, no estimate."""
    t0 = time.perf_counter()
    cell_steps = 0
    per = []
    for req in sorted(requests, key=lambda r: r.arrival):
        ts = time.perf_counter()
        s, box, area, _, u = domain_for(req, storage)
        steps, cd_prev, cd, conv = 0, float("nan"), float("nan"), False
        while steps < max_steps:
            s.step(check_every)
            steps += check_every
            F = s.cv_force_box(box)
            cd_prev, cd = cd, float(F[0] / (0.5 * u * u * area)) if area > 0 else float("nan")
            conv = (math.isfinite(cd) and math.isfinite(cd_prev) and cd != 0.0 and abs(cd - cd_prev) < tol * abs(cd))
            if conv:
                break
        s.close()
        cell_steps += req.grid[0] * req.grid[1] * req.grid[2] * steps
        per.append(dict(rid=req.rid, steps=steps, cd=cd, converged=conv, wall_s=time.perf_counter() - ts))
    wall = time.perf_counter() - t0
    n_conv = sum(p["converged"] for p in per)
    return {"wall_s": round(wall, 3), "solves_per_hour": round(3600.0 * len(per) / wall, 1) if wall > 0 else 0.0,
            "converged_per_hour": round(3600.0 * n_conv / wall, 1) if wall > 0 else 0.0,
            "converged": int(n_conv), "mlups": round(cell_steps / wall / 1e6, 1) if wall > 0 else 0.0,
            "storage": storage, "per_request": per}

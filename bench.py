"""Benchmark of the GB300 LBM solver step (one JSON line on rank 0).

Workload: the Re = 100 sphere, 240 x 120 x 115 = 3.31 M cells, D3Q19 TRT +
Smagorinsky (two-pass |S|), icosphere level 6 (81,920 triangles) voxelized on
the GPU, inlet u = 0.05, zero-gradient outlet, free-slip lateral walls;
populations stored as FP16 shifted deviations (the headline form) with the
plain FP32 form measured beside it. A step is one lattice update of the whole
domain. The working set (populations + two velocity fields + descriptors)
exceeds the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the CPU implementation of the same step (the C
restatement of the reference solver, OpenMP over all host cores; the
reference's own build cannot run on this host) on the same grid.
Under torchrun (N > 1) each rank runs an independent replica on its GPU
(the workload does not shard); value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import contextlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "aeros-engine_gb300"))

# algorithmic bytes per cell update of the step with LES (read + write):
#   populations 2 x 19 x bytes, previous velocity 12 (ux, uy, uz), new
#   velocity 12, a one-byte cell mask
BYTES_PER_CELL = {"fp32": 2 * 19 * 4 + 12 + 12 + 1, "fp16": 2 * 19 * 2 + 12 + 12 + 1, "bf16": 2 * 19 * 2 + 12 + 12 + 1}
# what this layout moves per cell: the velocity as float4 (16 + 16) and a
# 4-byte descriptor in place of the mask (11 bytes more per cell)
LAYOUT_BYTES_PER_CELL = {k: v + 8 + 3 for k, v in BYTES_PER_CELL.items()}
# DRAM bytes per launch of the step kernel (read + write, mean of an odd and
# an even step) from the ncu capture summarised in
# profiles/k_lbm_fused_sphere_240x120x115.md (this build: shell tiles first
# in the queue and the shell cell inline for FP16, one shell block per SM and
# the shell cell out of line for FP32)
NCU_TRAFFIC = {"fp16": (236018688 + 143872512 + 225713920 + 182815232) / 2,
               "fp32": (349847552 + 272347392 + 333710592 + 312974336) / 2}
# the workload both arms run (the reference arm in its own FP32 form)
WORKLOAD_CONFIG = {"workload": "sphere Re=100, 240x120x115 (3.31 M cells), icosphere L6 (81,920 triangles), "
                               "TRT+Smagorinsky, zero-gradient outlet, free-slip lateral walls",
                   "storage": "fp16 shifted by the freestream equilibrium (fp32 plain measured beside it)",
                   "l2": "working set > 129 MB L2, no flush"}
# bytes of the solver's device control block that every aeros_lbm_step call
# reads back (struct Control in aeros-engine_gb300/csrc/lbm_step.cuh)
CONTROL_BYTES = 272


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def rank_barrier(world: int) -> None:
    """Under torchrun: every rank's device work done, then a barrier (both
    sides of a timed region)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.synchronize()
        dist.barrier()


def gather_max(values, world: int) -> list:
    """Element-wise maximum over the ranks of a list of floats (times): the
    replicas' job ends with the slowest rank."""
    if world <= 1:
        return [float(v) for v in values]
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


def replica_rate(cells: int, steps: int, seconds: float, world: int) -> float:
    """Whole-job MLUPS of `world` replicas, each updating `cells` cells
    `steps` times, when the slowest took `seconds`."""
    return world * cells * steps / seconds / 1e6


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, polled about every 50 ms and
    stamped at the middle of each query. `window(kind)` marks a stretch in
    which the GPU runs the stepping workload: "steps" (warm-up and timed
    steps) or "after" (the same steps, untimed, right after the timed
    region: a timed region of a few milliseconds falls between two polls).
    The summary is taken over the samples inside the marked windows."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int, period_s: float = 0.05):
        self.idx = gpu_index
        self.period = period_s
        self.samples = []    # (time, fields)
        self.windows = []    # (t0, t1, kind)
        self.stop = threading.Event()
        self.t = None

    def _run(self):
        while not self.stop.is_set():
            try:
                t0 = time.perf_counter()
                out = subprocess.run(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                t1 = time.perf_counter()
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append((0.5 * (t0 + t1), [v.strip() for v in out.stdout.strip().split(",")]))
            except Exception:
                pass
            self.stop.wait(self.period)

    def __enter__(self):
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *exc):
        self.stop.set()
        if self.t:
            self.t.join(timeout=10)

    @contextlib.contextmanager
    def window(self, kind: str):
        t0 = time.perf_counter()
        try:
            yield
        finally:
            self.windows.append((t0, time.perf_counter(), kind))

    def summary(self):
        inside = lambda t, kinds: any(a <= t <= b for a, b, k in self.windows if k in kinds)   # noqa: E731
        load = [f for t, f in self.samples if inside(t, ("steps", "after"))]
        n_steps = sum(1 for t, _ in self.samples if inside(t, ("steps",)))
        if not load:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0, "samples_steps": 0}
        sm = [float(s[0]) for s in load if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in load if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in load for i in range(4) if len(s) > 3 + i and s[3 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(load), "samples_steps": n_steps,
                "window": "polled every 50 ms during the warm-up and timed steps and during 0.4 s of the same "
                          "steps right after the timed region, for each storage form"}


def load_after(solver, seconds=0.4, chunk=100):
    """The same steps, untimed, for `seconds` after a timed region."""
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        solver.step(chunk)
    solver.synchronize()


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def sphere_case(storage, mask=None):
    from aeros_gb300 import geometry
    return geometry.sphere_config(storage=storage, mask=mask)


def time_steps(solver, steps, warmup, world=1):
    """Device time of `steps` lattice steps (CUDA events around the launches on
    the solver's stream), after `warmup` untimed steps; under torchrun the
    timed region is bracketed by a barrier on both sides."""
    solver.step(warmup)
    solver.synchronize()
    rank_barrier(world)
    solver.step_async(steps)
    ms = solver.last_step_ms()
    rank_barrier(world)
    launches = solver.last_launch_count()
    st = solver.stats()
    return ms, launches, st


def run_gb300(args):
    import ctypes

    from aeros_gb300 import capi, solver
    rank, world, local = dist_env()
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    capi.lib()
    nx, ny, nz = (240, 120, 115)
    cells = nx * ny * nz
    # geometry: the icosphere voxelized on the GPU (BVH path)
    t0 = time.time()
    p16, mask, tris = sphere_case("fp16")
    vox_s = time.time() - t0
    results = {}
    peak, peak_kind = measured_peak()
    with ClockSampler(local) as clk:
        for storage in (("fp32", "fp16") if args.only == "both" else (args.only,)):
            p, _, _ = sphere_case(storage, mask=mask)
            s = solver.Solver(p, mask)
            with clk.window("steps"):
                ms, launches, st = time_steps(s, args.steps, args.warmup, world)
            with clk.window("after"):
                load_after(s)
            mlups = cells * args.steps / (ms * 1e-3) / 1e6
            gbs = BYTES_PER_CELL[storage] * cells * args.steps / (ms * 1e-3) / 1e9
            results[storage] = dict(ms_per_step=ms / args.steps, mlups=mlups, achieved_gbs=gbs, launches=launches,
                                    avg_rho=st["avg_rho"], max_u=st["max_velocity_lb"], bytes=s.device_bytes())
            s.close()
        # end to end through the C ABI with host buffers, the way a frame
        # loop drives the solver: the domain is created from the host mask
        # first (setup, not timed); then per step one aeros_lbm_step_async(1)
        # and the control-volume drag of that step (aeros_lbm_cv_force), which
        # waits for the step and reads back its statistics (the control
        # block, D2H) and the force (D2H); the fields are read back to host
        # memory at the end. A step has no host input: nothing goes host to
        # device inside the timed region.
        return_early = args.only != "both" or args.no_e2e
        e2e_steps = 0 if return_early else args.steps
        if not return_early:
            p, _, _ = sphere_case("fp16", mask=mask)
            s = solver.Solver(p, mask)
            # the frame loop's host mirrors of the fields: page-locked, allocated once
            host = solver.pinned_fields(cells)
            s.step(2)
            s.fields(out=host)
            s.synchronize()
            rank_barrier(world)
            t1 = time.perf_counter()
            forces = []
            for _ in range(e2e_steps):
                s.step_async(1)
                forces.append(s.cv_force(0.3, 0.3, 0.3))
                stats = s.stats()   # the step's statistics, read back with the force
            t2 = time.perf_counter()
            s.fields(out=host)
            e2e_s = time.perf_counter() - t1
            readback_ms = 1000 * (time.perf_counter() - t2)
            rank_barrier(world)
            s.close()
            del host
    if return_early:
        print(json.dumps({k: {kk: round(vv, 4) if isinstance(vv, float) else vv for kk, vv in v.items()}
                          for k, v in results.items()}), flush=True)
        return
    h2d = 0
    # per step: the solver's control block (CONTROL_BYTES) + three doubles of
    # force; at the end six float fields
    d2h = (CONTROL_BYTES + 24) * e2e_steps + 4 * cells * 6
    head = results["fp16"]
    # the slowest rank's times; value = the cells all ranks updated / that time
    ms_step, e2e_s = gather_max([head["ms_per_step"], e2e_s], world)
    value = replica_rate(cells, 1, ms_step * 1e-3, world)
    e2e_value = replica_rate(cells, e2e_steps, e2e_s, world)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_baseline(mask, args.cpu_steps)
    if rank == 0:
        frac = head["achieved_gbs"] / peak
        line = {
            "metric": "MLUPS (D3Q19 TRT+Smagorinsky sphere, FP16-shifted storage)",
            "value": round(value, 1), "unit": "MLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms_step, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp16-storage/fp32-math", "data": "synthetic",
            "config": dict(WORKLOAD_CONFIG, parallelism="replicas" if world > 1 else "single device"),
            "roofline": {"bound": "hbm", "achieved": round(head["achieved_gbs"], 1), "peak": peak, "unit": "GB/s",
                         "frac": round(frac, 4), "traffic": round(NCU_TRAFFIC["fp16"]),
                         "traffic_unit": "bytes per launch (ncu)", "algorithmic_bytes": BYTES_PER_CELL["fp16"] * cells,
                         "peak_kind": peak_kind, "bytes_per_cell": BYTES_PER_CELL["fp16"],
                         "layout_bytes_per_cell": LAYOUT_BYTES_PER_CELL["fp16"],
                         "frac_layout": round(frac * LAYOUT_BYTES_PER_CELL["fp16"] / BYTES_PER_CELL["fp16"], 4)},
            "fp32_plain": {"mlups": round(results["fp32"]["mlups"], 1),
                           "ms_per_step": round(results["fp32"]["ms_per_step"], 4),
                           "achieved_gbs": round(results["fp32"]["achieved_gbs"], 1),
                           "frac": round(results["fp32"]["achieved_gbs"] / peak, 4),
                           "traffic": round(NCU_TRAFFIC["fp32"]), "bytes_per_cell": BYTES_PER_CELL["fp32"],
                           "layout_bytes_per_cell": LAYOUT_BYTES_PER_CELL["fp32"]},
            "fp16_over_fp32": round(results["fp16"]["mlups"] / results["fp32"]["mlups"], 3),
            "e2e": {"value": round(e2e_value, 1), "unit": "MLUPS", "h2d_bytes_per_step": int(h2d // max(1, e2e_steps)),
                    "d2h_bytes_per_step": int(d2h // max(1, e2e_steps)),
                    "readback_ms": round(readback_ms, 3),
                    "what": "per step aeros_lbm_step_async(1) + aeros_lbm_cv_force (one wait: the step's statistics and the "
                            "force read back) + aeros_lbm_get_stats; then the six final fields (rho, u, |S|, TKE: "
                            f"{4 * cells * 6} B) into page-locked host mirrors allocated before the timed region "
                            "(readback_ms of the total); domain created before the timed region; a step has no host "
                            "input, so nothing goes host to device"},
            "gpu_launches": int(head["launches"]),
            "clocks": clk.summary(),
            "voxelize_s": round(vox_s, 3),
        }
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()


def batch_sweep(n_domains=64, steps=10000, storage="fp16", seq_steps=20, chunk=100, autotune=True):
    """The batched design sweep: n_domains seeded domains (sizes 32^3 ...
    160x80x80, perturbed icosphere level 4, Re ~ U(50, 400), u = 0.04, TRT +
    Smagorinsky, FP16 shifted storage) in one batch, autotuned launch shape,
    `steps` steps each in CUDA-graph chunks. Beside it the same domains stepped
    one at a time through the single-domain path (seq_steps each)."""
    from aeros_gb300 import batch, geometry, solver
    t0 = time.time()
    doms = []
    for i in range(n_domains):
        p, mask, _ = geometry.batch_domain(i, storage=storage)
        doms.append(solver.Solver(p, mask))
    setup_s = time.time() - t0
    cells = sum(d.n for d in doms)
    seq_ms = 0.0
    for d in doms:
        d.step(2)
        d.step(seq_steps)
        seq_ms += d.last_step_ms()
    b = batch.Batch(storage)
    for d in doms:
        b.add(d)
    t1 = time.time()
    tune = b.autotune(trial_steps=20) if autotune else b.tuning
    tune_s = time.time() - t1
    b.set_tuning(blocks_per_sm=tune["blocks_per_sm"], tiles_per_item=tune["tiles_per_item"],
                 shell_tiles_per_item=tune["shell_tiles_per_item"], chunk_steps=chunk)
    b.step(100)   # capture + warm-up
    b.step(steps)
    ms = b.last_step_ms()
    launches = b.last_launch_count()
    diverged = sum(d.stats()["diverged"] for d in doms)
    b.close()
    for d in doms:
        d.close()
    mlups = cells / (ms * 1e-3) / 1e6
    seq_mlups = cells * seq_steps / (seq_ms * 1e-3) / 1e6
    return {"domains": n_domains, "cells": cells, "steps": steps, "ms_per_step": round(ms, 4),
            "mlups": round(mlups, 1), "achieved_gbs": round(BYTES_PER_CELL[storage] * cells / (ms * 1e-3) / 1e9, 1),
            "sequential_mlups": round(seq_mlups, 1), "speedup_vs_sequential": round(mlups / seq_mlups, 3),
            "tuning": tune, "autotune_s": round(tune_s, 2), "setup_s": round(setup_s, 2), "gpu_launches": int(launches),
            "diverged_domains": int(diverged)}


def serve_session(n_requests=16, rate=2.0, max_steps=30000, log_path=None):
    """The request loop: n_requests Poisson arrivals (rate per second) served
    by continuous batching (FP16), once in real time (latency percentiles) and
    once with every request queued at the start (throughput); the same
    requests solved one at a time in plain FP32 beside it, each to its own
    convergence (measured). log_path: the real-time session's per-solve JSON
    lines are written there."""
    from aeros_gb300 import serve
    reqs = serve.make_requests(n_requests, rate=rate)
    log = open(log_path, "w") if log_path else None
    try:
        live = serve.Server(storage="fp16", max_steps=max_steps, log=log).run(reqs, realtime=True)
    finally:
        if log is not None:
            log.close()
    srv = serve.Server(storage="fp16", max_steps=max_steps)
    sat = srv.run(reqs, realtime=False)
    seq = serve.sequential_plain(reqs, max_steps=max_steps)
    per_seq = {p["rid"]: p for p in seq.pop("per_request")}
    return {"requests": n_requests, "rate_per_s": rate, "realtime": live["summary"], "saturated": sat["summary"],
            "sequential_fp32": seq,
            "speedup_solves_per_hour": round(sat["summary"]["solves_per_hour"] / seq["solves_per_hour"], 3)
            if seq["solves_per_hour"] > 0 else None,
            "speedup_converged_per_hour": round(sat["summary"]["converged_per_hour"] / seq["converged_per_hour"], 3)
            if seq["converged_per_hour"] > 0 else None,
            "per_request": [dict(rid=r.rid, grid=reqs[r.rid].grid, triangles=20 * reqs[r.rid].freq ** 2,
                                 re=round(reqs[r.rid].re, 1), steps=r.steps, cd=round(r.cd, 5), converged=r.converged,
                                 latency_s=round(r.latency, 3), fp32_steps=per_seq[r.rid]["steps"],
                                 fp32_cd=round(per_seq[r.rid]["cd"], 5), fp32_converged=per_seq[r.rid]["converged"])
                            for r in live["results"]]}


def sdf_bench(res=256, reps=5, cpu=True):
    """The voxel grid's distance field (buildVoxelGrid's distance part) of the
    level-6 icosphere on the reference's grid plan at resolution `res` (box
    = mesh bounds + 14 % of the bounds' diagonal on each side): mask voxelized
    on the device, then `reps` timed builds from the device mask into a device
    field; e2e through the host-array call. CPU baseline: the reference's
    sweeps + FIFO + smoothing restated (single thread, as the reference runs
    them) on the same mask."""
    import ctypes as C

    import torch
    from aeros_gb300 import capi, geometry, solver
    tris = geometry.icosphere(6)
    lo, hi = tris.reshape(-1, 3).min(0), tris.reshape(-1, 3).max(0)
    margin = np.float32(0.14) * np.float32(np.sqrt(np.sum((hi - lo) ** 2, dtype=np.float32)))
    mn, mx = lo - margin, hi + margin
    plan = solver.voxel_plan(mx - mn, res)
    dims = (plan.nx, plan.ny, plan.nz)
    cs = ((mx - mn) / np.array(dims, np.float32)).astype(np.float32)
    grid = solver.voxel_grid(dims, mn, cs)
    n = dims[0] * dims[1] * dims[2]
    L = capi.lib()
    dm = torch.empty(n, dtype=torch.uint8, device="cuda")
    df = torch.empty(n, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    t = np.ascontiguousarray(tris, np.float32)
    capi.check(L.aeros_voxelize_device(t.ctypes.data_as(C.POINTER(C.c_float)), t.shape[0], C.byref(grid),
                                       C.c_void_p(dm.data_ptr())), "voxelize")
    capi.check(L.aeros_sdf_device(C.c_void_p(dm.data_ptr()), C.byref(grid), C.c_void_p(df.data_ptr()), None), "sdf")
    ms = []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        capi.check(L.aeros_sdf_device(C.c_void_p(dm.data_ptr()), C.byref(grid), C.c_void_p(df.data_ptr()), None),
                   "sdf")
        ms.append(1000 * (time.perf_counter() - t0))
    passes, runs = solver.sdf_last_stats()
    mask = dm.cpu().numpy()
    t0 = time.perf_counter()
    field = solver.sdf(mask, grid)
    e2e_ms = 1000 * (time.perf_counter() - t0)
    dev_ms = float(np.median(ms))
    line = {"metric": "distance-field build rate (level-6 icosphere, reference grid plan)",
            "value": round(n / (dev_ms * 1e-3) / 1e6, 1), "unit": "Mcells/s", "higher_is_better": True,
            "ms_per_build": round(dev_ms, 3), "builds": reps, "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"icosphere L6 (81,920 triangles), grid {dims[0]}x{dims[1]}x{dims[2]} "
                                   f"({n} cells), res {res}", "solid_cells": int((mask == 1).sum())},
            "passes": int(passes), "tile_runs": int(runs), "tiles": int(-(-dims[0] // 8) * -(-dims[1] // 8) * -(-dims[2] // 8)),
            "e2e": {"value": round(n / (e2e_ms * 1e-3) / 1e6, 1), "unit": "Mcells/s", "h2d_bytes_per_step": n,
                    "d2h_bytes_per_step": 4 * n, "what": "aeros_sdf: host mask in, host field out"},
            "field_range": [float(field.min()), float(field.max())]}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        oracle.build()
        t0 = time.perf_counter()
        oracle.sdf(mask, dims, cs)
        cpu_s = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": round(n / cpu_s / 1e6, 2), "unit": "Mcells/s", "cores": 1, "kind": "port",
                                "sample": f"one full build of the same {n}-cell grid (the reference's sweeps, FIFO "
                                          "and smoothing restated, single thread as the reference's propagation)"}
    return line


def surface_bench(reps=20, warm_steps=300, cpu=True):
    """Surface-pressure lift and drag (computeLiftDrag) of the level-6
    icosphere (81,920 triangles, radial vertex normals) on the Re = 100
    sphere, 240 x 120 x 115 FP32, after `warm_steps` steps, with the device
    distance field of its mask: `reps` timed calls through the C ABI (the
    three kernels, the 144-byte readback and the host closing formulas; no
    per-triangle Cp copy). CPU baseline: the restatement over the same
    pressure field, FP32 as the reference runs its OpenMP loop on one thread."""
    import torch
    from aeros_gb300 import capi, geometry, solver
    p, mask, tris = geometry.sphere_config("fp32")
    nx, ny, nz = geometry.SPHERE_GRID
    s = solver.Solver(p, mask)
    s.step(warm_steps)
    # the reference's sampler puts cell i's value at min + i * cell (lbm.cpp:1881-1933), the mask's
    # cell centres sit at i + 0.5: min = 0.5 centres the pressure on the mesh
    w = capi.make_world(12.5, 1.225, (0.5, 0.5, 0.5), (1.0, 1.0, 1.0))
    fields, _ = s.world_fields(w)
    v = np.ascontiguousarray(tris, np.float32).reshape(-1, 9)
    c = np.asarray(geometry.SPHERE_CENTER, np.float64)
    nrm = geometry.face_normals(v, c)
    grid = solver.voxel_grid((nx, ny, nz), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0))
    sdf = solver.sdf((mask.reshape(-1) == 1).astype(np.uint8), grid)
    d = torch.from_numpy(sdf).cuda()
    torch.cuda.synchronize()
    r = geometry.SPHERE_RADIUS
    sp = capi.make_surface(velocity=(12.5, 0.0, 0.0), bb_min=c - r, bb_max=c + r, center=c, reynolds=1e7)
    mesh = solver.SurfaceMesh(v, nrm)
    ntri = v.shape[0]
    s.surface_forces(w, sp, mesh, d.data_ptr(), grid, want_cp=False)   # warm-up
    ms = []
    for _ in range(reps):
        t0 = time.perf_counter()
        o, _ = s.surface_forces(w, sp, mesh, d.data_ptr(), grid, want_cp=False)
        ms.append(1000 * (time.perf_counter() - t0))
    dev_ms = float(np.median(ms))
    line = {"metric": "surface-pressure lift and drag rate (computeLiftDrag, level-6 icosphere)",
            "value": round(ntri / (dev_ms * 1e-3) / 1e6, 2), "unit": "Mtriangles/s", "higher_is_better": True,
            "ms_per_call": round(dev_ms, 4), "calls": reps, "dtype": "f32 (warp sums f32, block and grid sums f64)", "data": "synthetic",
            "config": {"workload": f"icosphere L6 ({ntri} triangles) on the Re=100 sphere 240x120x115 FP32 after "
                                   f"{warm_steps} steps, distance field of the mask", "what": "aeros_lbm_surface_forces, "
                                   "host to host (params in, 144 B result out)"},
            "drag_N": float(o.drag), "lift_N": float(o.lift), "ref_area": float(o.ref_area)}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        oracle.build()
        wall = (mask.reshape(-1) != 0).astype(np.uint8)
        t0 = time.perf_counter()
        k = 0
        while True:
            oracle.surface_forces_field(fields["pressure"], wall, (nx, ny, nz), w, sp, v, nrm, sdf, grid,
                                        f32_sums=True)
            k += 1
            if time.perf_counter() - t0 > 2.0:
                break
        cpu_s = (time.perf_counter() - t0) / k
        line["cpu_baseline"] = {"value": round(ntri / cpu_s / 1e6, 3), "unit": "Mtriangles/s", "cores": 1,
                                "kind": "port", "sample": f"{k} full passes over the same {ntri} triangles and "
                                                          "pressure field (the restatement, one thread)"}
    return line


def rb_bench(steps=50000, ras=(1700.0, 2500.0, 1e4)):
    """Rayleigh-Benard convection, 128 x 128 x 32 fluid rows (+ 2 wall rows,
    the reference's y axis up), D3Q19 BGK + D3Q7 thermal with Boussinesq
    feedback, Pr = 0.71, hot bottom / cold top (T = +-0.5), linear initial
    profile + seeded U(-1e-3, 1e-3) noise, `steps` steps, FP32 plain and FP16
    shifted storage for both lattices: MLUPS and the FP64-reduced Nusselt
    number of each run."""
    from aeros_gb300 import geometry, solver
    runs = []
    for ra in ras:
        nus = {}
        for storage in ("fp32", "fp16"):
            p, mask, tp = geometry.rb_config(ra, storage=storage)
            s = solver.Solver(p, mask)
            s.thermal_init(tp)
            s.thermal_upload(geometry.rb_initial_T(p.nx, p.ny, p.nz, ra))
            s.step(steps)
            ms = s.last_step_ms()
            st = s.stats()
            cells = p.nx * p.ny * p.nz
            bpc = (BYTES_PER_CELL[storage] + (56 if storage == "fp32" else 28) + 8)
            runs.append({"ra": ra, "storage": storage, "steps": steps, "ms_per_step": round(ms / steps, 4),
                         "mlups": round(cells * steps / (ms * 1e-3) / 1e6, 1),
                         "achieved_gbs": round(bpc * cells * steps / (ms * 1e-3) / 1e9, 1), "bytes_per_cell": bpc,
                         "nusselt": round(float(st["nusselt"]), 6), "diverged": int(st["diverged"])})
            nus[storage] = float(st["nusselt"])
            s.close()
        runs[-1]["nusselt_fp16_minus_fp32"] = round(nus["fp16"] - nus["fp32"], 6)
    peak, _ = measured_peak()
    return {"metric": "Rayleigh-Benard MLUPS (D3Q19 BGK + D3Q7, 128x34x128) and Nusselt number", "unit": "MLUPS",
            "peak_gbs": peak, "runs": runs, "data": "synthetic"}


def cpu_baseline(mask, steps):
    """The oracle (C restatement of the reference solver, OpenMP) on the same
    grid, `steps` lattice steps (a bounded sample)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    p, _, _ = sphere_case("fp32", mask=mask)
    o = oracle.OracleLBM(p, mask)
    o.step(1)
    t = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t
    cells = p.nx * p.ny * p.nz
    # one thread (the reference's loop without OpenMP), a shorter sample
    oracle.set_threads(1)
    steps1 = max(1, steps // 10)
    t = time.perf_counter()
    o.step(steps1)
    dt1 = time.perf_counter() - t
    oracle.set_threads(cores)
    return {"value": round(cells * steps / dt / 1e6, 2), "unit": "MLUPS", "cores": cores, "kind": "port",
            "value_1thread": round(cells * steps1 / dt1 / 1e6, 2),
            "sample": f"{steps} lattice steps of the full 240x120x115 sphere grid (FP32, OpenMP {cores} threads); "
                      f"value_1thread: {steps1} steps on one thread"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    from aeros_gb300 import geometry
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    nx, ny, nz = geometry.SPHERE_GRID
    # the reference's CPU path voxelizes on the host: brute-force inside test
    tris = geometry.icosphere(6, geometry.SPHERE_RADIUS, geometry.SPHERE_CENTER)
    from aeros_gb300.solver import voxel_grid
    g = voxel_grid((nx, ny, nz), (0, 0, 0), (1, 1, 1))
    mpath = os.path.join(ROOT, "tests", "golden", "masks.npz")
    mask = np.unpackbits(np.load(mpath)["sphere_config_mask"])[: nx * ny * nz].astype(np.uint8)
    del tris, g
    p, _, _ = geometry.sphere_config(storage="fp32", mask=mask)
    o = oracle.OracleLBM(p, mask)
    o.step(args.warmup)
    t = time.perf_counter()
    o.step(args.steps)
    dt = time.perf_counter() - t
    cells = nx * ny * nz
    v = cells * args.steps / dt / 1e6
    line = {"impl": "reference", "metric": "MLUPS (D3Q19 TRT+Smagorinsky sphere, FP16-shifted storage)",
            "value": round(v, 2), "unit": "MLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1000 * dt / args.steps, 2), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic",
            "config": dict(WORKLOAD_CONFIG, parallelism="single device"),
            "cpu_baseline": {"value": round(v, 2), "unit": "MLUPS", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} full-grid lattice steps per timed run, FP32 (the reference "
                                       f"solver's own arithmetic), OpenMP {cores} threads"},
            "e2e": {"value": round(v, 2), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=30)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--only", default="both", choices=["both", "fp32", "fp16", "bf16"],
                    help="time one storage form only (profiling runs)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--workload", default="sphere", choices=["sphere", "batch", "serve", "sdf", "rb", "surface"])
    ap.add_argument("--rb-steps", type=int, default=50000)
    ap.add_argument("--sdf-res", type=int, default=256)
    ap.add_argument("--serve-requests", type=int, default=16)
    ap.add_argument("--serve-rate", type=float, default=2.0)
    ap.add_argument("--serve-max-steps", type=int, default=30000)
    ap.add_argument("--serve-log", default=None, help="file for the real-time session's per-solve JSON lines")
    ap.add_argument("--batch-domains", type=int, default=64)
    ap.add_argument("--batch-steps", type=int, default=10000)
    ap.add_argument("--batch-chunk", type=int, default=100, help="steps per captured CUDA graph")
    ap.add_argument("--batch-fixed", action="store_true", help="default launch shape, no autotuning")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-sweep figures in the sphere line")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "serve":
        r = serve_session(args.serve_requests, args.serve_rate, args.serve_max_steps, args.serve_log)
        print(json.dumps(r), flush=True)
    elif args.workload == "rb":
        print(json.dumps(rb_bench(args.rb_steps)), flush=True)
    elif args.workload == "surface":
        print(json.dumps(surface_bench(reps=max(1, min(args.steps, 200)), cpu=not args.no_cpu)), flush=True)
    elif args.workload == "sdf":
        print(json.dumps(sdf_bench(args.sdf_res, reps=max(1, min(args.steps, 20)), cpu=not args.no_cpu)), flush=True)
    elif args.workload == "batch":
        r = batch_sweep(args.batch_domains, args.batch_steps, chunk=args.batch_chunk, autotune=not args.batch_fixed)
        print(json.dumps(r), flush=True)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()

#!/usr/bin/env python3
"""Benchmark of the FDTD task-graph hot path on GB300.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

One bench step is one complete solve of the workload (all of its time steps).  Default workload:
the plain FDTD graph at 256^3 FP32 (8 seeded dielectric boxes, eps_r 1-10, 8-64 cells, PEC walls,
Courant 0.5, Gaussian Ez source, 1000 steps).  Prints one JSON line (rank 0):

  value  Mcell-updates/s with the inputs already resident in HBM (device events around the solves)
  e2e    the same metric through the public C-ABI path with pinned host buffers, the H2D upload of the
         inputs and the D2H download of the six result fields inside the timed region
  roofline  the fused step kernel against measured HBM bandwidth: 49 algorithmic bytes per cell update
         with the material index (six fields read and written, one id byte), 64 with per-cell arrays
  cpu_baseline  the CPU oracle (our FP32 port of the reference's fdtd_cpu, OpenMP over all host cores)
                timed on a bounded sample of the same workload
  served the workload's batched/served half: the 64-instance batched set, a Poisson trace at the
         workload's 200 req/s and one below saturation, each served by continuous batching and by
         every plain one-at-a-time arm (fused server slot, fused graph dispatch, task-wise graph
         dispatch) on the same requests: solves/s, Mcell/s, p50/p99 and the fraction of peak
  large  the large single-GPU grid (512x512x384, 500 steps) solved from resident fields with the
         autotuned tiles: Mcell-updates/s and the fraction of peak

--impl reference times the reference's CPU implementation of the path instead (the oracle port; the
reference's own build needs its source tree, which is absent where this runs) on the same workload,
loading nothing but the oracle.
Under torchrun each rank runs an independent replica (the path shards by instance; no collective on
the data path) and rank 0 reports the whole-job aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

BYTES_PER_CELL = 64          # 6 fields read + written (48 B) + 4 coefficients read (16 B), FP32
BYTES_PER_CELL_MAT = 49      # 6 fields read + written (48 B) + a one-byte material id (coefficients from a table)
FALLBACK_HBM_GBS = 6800.0

WORKLOADS = {
    # the plain-graph headline workload
    "plain256": dict(shape=(256, 256, 256), boxes=8, eps=(1.0, 10.0), box=(8, 64), steps=1000,
                     desc="plain FDTD graph 256^3 FP32, 8 seeded dielectric boxes (eps_r 1-10, edges 8-64), "
                          "PEC walls, Courant 0.5, Gaussian Ez source at centre, 1000 steps"),
    # the large single-GPU workload
    "large": dict(shape=(512, 512, 384), boxes=32, eps=(1.0, 10.0), box=(8, 64), steps=500,
                  desc="large plain FDTD 512x512x384 FP32, 32 seeded dielectric boxes, 500 steps"),
    # the CPU-runnable case, used for quick checks
    "cpu32": dict(shape=(32, 32, 32), boxes=2, eps=(2.0, 6.0), box=(4, 16), steps=100,
                  desc="32^3 FP32, 2 dielectric boxes (eps_r 2-6), 100 steps"),
}


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Dist:
    """Barrier and max-reduction across ranks (torch.distributed; a no-op on one process)."""

    def __init__(self, world: int, local: int):
        self.world = world
        self.pg = None
        if world > 1:
            import torch
            import torch.distributed as td
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(local)
            td.init_process_group(backend=backend)
            self.td, self.torch = td, torch
            self.dev = torch.device("cuda", local) if backend == "nccl" else torch.device("cpu")

    def barrier(self):
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.lines: list[str] = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                rows.append((float(parts[0]), float(parts[1]), parts[4:8]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, flags in rows for i, f in enumerate(flags) if f.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def hbm_peak():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        try:
            return float(json.loads(f.read_text())["hbm_gbs"]), "measured"
        except (KeyError, ValueError):
            pass
    return FALLBACK_HBM_GBS, "fallback"


def traffic_per_cell(kernel: str, mat: bool = False, rows: int = 0):
    """DRAM bytes per cell update of the given fused step kernel from its committed ncu summary (the
    64-wide 23-row tiles have their own; other staged shapes use the 11-row figure)."""
    name = {("k_yee_step_bulk", True): "yee_step_bulk_mat_256.md", ("k_yee_step_bulk", False): "yee_step_bulk_256.md"}
    if kernel == "k_yee_step_bulk" and mat and rows == 23:
        name[(kernel, mat)] = "yee_step_bulk_mat23_256.md"
    f = ROOT / "profiles" / name.get((kernel, mat), "yee_step_256.md")
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("dram_bytes_per_cell_update:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


def cpu_sample(prob, shape, target_s: float = 10.0):
    """Time the oracle (FP32 port of fdtd_cpu, all host threads) on a bounded sample of the workload."""
    import oracle
    f = oracle.zero_fields(*shape)
    oracle.step_ext_f32(f, 1, prob.params, prob.Ca, prob.Cb, prob.Da, prob.Db, prob.src, prob.wave)  # warm
    t0 = time.perf_counter()
    oracle.step_ext_f32(f, 2, prob.params, prob.Ca, prob.Cb, prob.Da, prob.Db, prob.src, prob.wave)
    one = (time.perf_counter() - t0) / 2
    total = prob.wave.size or 1000
    want = max(1, int(target_s / max(one, 1e-6)))
    steps = min(total, want)
    # a workload shorter than the target is solved again from its initial fields until the sample
    # reaches the target time
    repeats = max(1, min(10000, want // total)) if want > total else 1
    t0 = time.perf_counter()
    for _ in range(repeats):
        oracle.step_ext_f32(f, steps, prob.params, prob.Ca, prob.Cb, prob.Da, prob.Db, prob.src, prob.wave)
    dt = time.perf_counter() - t0
    cells = shape[0] * shape[1] * shape[2]
    what = (f"the whole solve ({steps} steps) {repeats} times" if repeats > 1 else
            f"first {steps} of the workload's time steps")
    return {"value": cells * steps * repeats / dt / 1e6, "unit": "Mcell-updates/s", "cores": oracle.threads(),
            "kind": "port",
            "sample": f"{shape[0]}x{shape[1]}x{shape[2]} grid, {what} ({dt:.1f} s), oracle/fdtd_oracle.c FP32 "
                      f"port of fdtd_cpu, OpenMP on {oracle.threads()} host threads"}


def workload_config(wl, world: int) -> dict:
    """The `config` object of a plain workload, identical in both arms' lines."""
    nx, ny, nz = wl["shape"]
    return {"workload": wl["desc"], "grid": [nx, ny, nz], "time_steps": wl["steps"],
            "l2": "working set %.2f GB > 129 MB L2; no flush needed" % (16 * 4 * (nx + 1) * (ny + 1) * (nz + 1) / 1e9),
            "parallelism": f"replicas x{world}"}


def run_reference(args, wl, world, rank, local):
    """--impl reference: the CPU implementation of the path on the host cores.  Everything it runs is
    the oracle (oracle/: the FP32 port of fdtd_cpu and its own copy of the seeded problem generator);
    nothing of the product library is loaded."""
    if rank != 0:
        return 0
    import oracle
    shape = wl["shape"]
    prob = oracle.problem_generate(*shape, n_boxes=wl["boxes"], eps=wl["eps"], box=wl["box"], steps=wl["steps"],
                                   source_mode=1, seed=2)
    f = oracle.zero_fields(*shape)
    t0 = time.perf_counter()
    oracle.step_ext_f32(f, 1, prob.params, prob.Ca, prob.Cb, prob.Da, prob.Db, prob.src, prob.wave)
    one = time.perf_counter() - t0
    per = max(1, min(wl["steps"], int(2.0 / max(one, 1e-6))))   # ~2 s of CPU work per bench step
    for _ in range(args.warmup):
        oracle.step_ext_f32(f, 1, prob.params, prob.Ca, prob.Cb, prob.Da, prob.Db, prob.src, prob.wave)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.step_ext_f32(f, per, prob.params, prob.Ca, prob.Cb, prob.Da, prob.Db, prob.src, prob.wave)
    dt = time.perf_counter() - t0
    cells = shape[0] * shape[1] * shape[2]
    value = cells * per * args.steps / dt / 1e6
    threads = oracle.threads()
    sample = (f"{shape[0]}x{shape[1]}x{shape[2]} grid, {per} of the workload's {wl['steps']} time steps per "
              f"bench step, oracle/fdtd_oracle.c FP32 port of fdtd_cpu, OpenMP on {threads} host threads")
    line = {"metric": "FDTD Mcell-updates/s", "value": value, "unit": "Mcell-updates/s", "impl": "reference",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded problem generator)",
            "config": workload_config(wl, world),
            "bench_step": f"{per} time steps of the workload on the host cores",
            "cpu_baseline": {"value": value, "unit": "Mcell-updates/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "Mcell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, wl, world, rank, local):
    import ptask_gb300 as P
    from ptask_gb300 import _lib
    from ptask_gb300.device import DeviceBuffer, Event, HostBuffer

    dist = Dist(world, local)
    _lib.call("ptk_runtime_init", local)
    shape = wl["shape"]
    nx, ny, nz = shape
    T = wl["steps"]
    prob = P.Problem.generate(*shape, n_boxes=wl["boxes"], eps=wl["eps"], box=wl["box"], steps=T,
                              source_mode=1, seed=2 + rank)
    cells = nx * ny * nz
    tiles = None
    if args.tiles:   # ROWS,DEPTH[,VEC[,STAGES]]
        tiles = tuple(int(v) for v in args.tiles.split(","))
    elif not args.no_autotune:
        tiles = P.tuned_tiles(nx, ny, nz)

    solver = P.Solver(prob.params)
    if tiles:
        solver.set_tiles(*tiles)
    if args.dense_coefficients:
        solver.use_material_index(False)
    zero = P.zero_fields(*shape)
    # Inputs resident in HBM: dense initial fields on the device, coefficients + source uploaded once.
    dev_init = [DeviceBuffer.from_array(a) for a in zero]
    solver.set_problem(prob)
    ev0, ev1 = Event(), Event()
    run_ev = [(Event(), Event()) for _ in range(args.steps)]

    def device_step(k=None):
        solver.set_fields_device([b.value for b in dev_init])
        solver.reset_clock()
        if k is not None:
            run_ev[k][0].record()
        solver.run(T)
        if k is not None:
            run_ev[k][1].record()

    for _ in range(args.warmup):
        device_step()
    _lib.call("ptk_stream_sync", None)
    dist.barrier()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = P.launch_count()
    ev0.record()
    for k in range(args.steps):
        device_step(k)
    ev1.record()
    ev1.sync()
    launches = P.launch_count() - l0
    clk = clocks.stop()
    dev_ms = ev0.elapsed_ms(ev1)
    run_ms = [a.elapsed_ms(b) for a, b in run_ev]
    dev_ms = dist.max(dev_ms)

    # ---- end to end: pinned host buffers, H2D inputs + D2H results inside the timed region ----------
    hin = [HostBuffer(a.shape) for a in zero]
    for h, a in zip(hin, zero):
        h.array[...] = a
    hcoef = [HostBuffer(a.shape) for a in (prob.Ca, prob.Cb, prob.Da, prob.Db)]
    for h, a in zip(hcoef, (prob.Ca, prob.Cb, prob.Da, prob.Db)):
        h.array[...] = a
    hwave = HostBuffer(prob.wave.shape)
    hwave.array[...] = prob.wave
    hout = [HostBuffer(a.shape) for a in zero]
    import ctypes as C
    V = C.c_void_p
    in_ptrs = (V * 6)(*[h.ptr.value for h in hin])
    out_ptrs = (V * 6)(*[h.ptr.value for h in hout])
    h2d = sum(a.nbytes for a in zero) + 4 * prob.Ca.nbytes + prob.wave.nbytes
    d2h = sum(a.nbytes for a in zero)

    phase_ev = [Event() for _ in range(6)]
    phase_ms = {"upload": 0.0, "solve": 0.0, "download": 0.0,
                "upload_fields": 0.0, "upload_coefficients_and_index": 0.0}

    def e2e_step(record=False):
        if record:
            phase_ev[0].record()
        _lib.call("ptk_solver_set_fields", solver.handle, in_ptrs, _lib.PTK_HOST, None)
        if record:
            phase_ev[4].record()
        _lib.call("ptk_solver_set_coefficients", solver.handle, *[h.ptr.value for h in hcoef], _lib.PTK_HOST, None)
        if record:
            phase_ev[5].record()
        _lib.call("ptk_solver_set_source", solver.handle, *prob.src, hwave.ptr.value, prob.wave.size,
                  _lib.PTK_HOST, None)
        solver.reset_clock()
        if record:
            phase_ev[1].record()
        solver.run(T)
        if record:
            phase_ev[2].record()
        _lib.call("ptk_solver_get_fields", solver.handle, out_ptrs, _lib.PTK_HOST, None)
        if record:
            phase_ev[3].record()
            phase_ev[3].sync()
            for name, a, b in (("upload", 0, 1), ("solve", 1, 2), ("download", 2, 3), ("upload_fields", 0, 4),
                               ("upload_coefficients_and_index", 4, 5)):
                phase_ms[name] += phase_ev[a].elapsed_ms(phase_ev[b])

    for _ in range(max(1, args.warmup)):
        e2e_step()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    e2e_s = dist.max(time.perf_counter() - t0)
    # the same steps again with device events between the phases (not part of the timed value)
    for _ in range(args.steps):
        e2e_step(record=True)
    result_ok = bool(np.isfinite(hout[5].array).all() and np.abs(hout[5].array).max() > 0)

    # ---- the reference-facing path: the PTask FDTD graph with host buffers ---------------------------
    # Cyclic graph (MF_GENERAL_ITERATOR loop, lowered to the fused step): per bench step, push the
    # coefficients and the source (set_problem), push the six fields, run the iteration and pull the
    # six fields, as the reference's driver does with its unrolled graph (graphfdtd.cpp:1076-1125).
    graph_e2e = None
    if not args.no_graph_e2e:
        from ptask_gb300.graph import FDTDGraph
        gout = P.zero_fields(*shape)   # result arrays reused across solves, as a serving loop would
        with FDTDGraph(prob.params, "fused") as g:
            def graph_step():
                g.set_problem(prob)
                return g.solve(zero, T, out=gout)

            for _ in range(max(1, args.warmup)):
                gout = graph_step()
            dist.barrier()
            t0 = time.perf_counter()
            for _ in range(args.steps):
                gout = graph_step()
            g_s = dist.max(time.perf_counter() - t0)
            gst = g.stats()
        graph_e2e = {
            "value": cells * T * args.steps * world / g_s / 1e6, "unit": "Mcell-updates/s",
            "ms_per_step": g_s * 1e3 / args.steps, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "path": "PTask graph API (ptk_fdtd_graph_set_problem + ptk_fdtd_graph_solve: Push, Graph::Run of "
                    "the cyclic FDTD graph lowered to the fused step, Pull), pageable host arrays",
            "same_result_as_solver_path": all(np.array_equal(a, h.array) for a, h in zip(gout, hout)),
            "cycles_lowered": gst["cycles_lowered"]}

    total_cell_updates = cells * T * args.steps * world
    value = total_cell_updates / (dev_ms / 1e3) / 1e6
    e2e_value = total_cell_updates / e2e_s / 1e6
    per_launch_ms = statistics.median(run_ms) / T
    peak, peak_src = hbm_peak()
    run_stages, mat = solver.kernel()
    bpc = BYTES_PER_CELL_MAT if mat else BYTES_PER_CELL
    achieved = bpc * cells / (per_launch_ms / 1e3) / 1e9
    by, kc, vec, stages = solver.tiles()
    kernel = "k_yee_step_bulk" if run_stages else "k_yee_step"
    tpc = traffic_per_cell(kernel, mat, by)
    line = {
        "metric": "FDTD Mcell-updates/s", "value": value, "unit": "Mcell-updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded problem generator)",
        "config": workload_config(wl, world),
        "bench_step": "one complete solve (all time steps) from resident initial fields",
        "kernel": {"tiles": {"rows": by, "z_depth": kc, "cells_per_thread": vec, "staged_planes": run_stages,
                             "kernel": kernel},
                   "coefficients": (f"material index: {solver.material_count()} distinct (Ca, Cb, Da, Db) tuples, "
                                    "one byte per node + table; per-cell arrays given at the API" if mat else
                                    "four per-cell FP32 arrays")},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src,
                     "traffic": (tpc * cells) if tpc else None,
                     "kernel": kernel + " (fused H+E step)",
                     "algorithmic_bytes_per_launch": bpc * cells,
                     "algorithmic_bytes_per_cell": bpc,
                     "frac_of_64B_cell_traffic": BYTES_PER_CELL * cells / (per_launch_ms / 1e3) / 1e9 / peak,
                     "launch_ms": per_launch_ms},
        "e2e_graph": graph_e2e,
        "e2e": {"value": e2e_value, "unit": "Mcell-updates/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_s * 1e3 / args.steps, "result_ok": result_ok,
                "path": "headline: the solver C ABI (ptk_solver_set_fields / set_coefficients / set_source, run, "
                        "get_fields) with pinned host buffers, the call sequence of a C or C++ caller of this "
                        "library; e2e_graph is the reference-facing PTask graph API with pageable arrays, as "
                        "the reference's driver passes them",
                "phases_ms_per_step": {k: v / args.steps for k, v in phase_ms.items()}},
        "gpu_launches": int(launches),
        "clocks": clk,
    }
    solver.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_sample(prob, shape)
    if world == 1 and not args.no_served and args.workload == "plain256":
        # The workload's other half: batched and served solves/s and p50/p99 against every plain arm.
        line["served"] = served_subrecords(args, rank, local)
    if world == 1 and not args.no_large and args.workload == "plain256":
        # The large single-GPU grid, resident, with autotuned tiles.
        line["large"] = large_subrecord(local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


def serve_arms(reqs, scale: float, rows: int, *, cb_runs: int = 1, cb_warmup: int = 0, graph_arms=("fused", "taskwise"),
               local: int = 0) -> dict:
    """Serve one request set with continuous batching and with every plain one-at-a-time arm.

    Arms, all on the same seeded requests and arrival times:
      continuous      ptk_server: requests admitted as they arrive and fit the HBM budget, every active
                      instance advanced by one persistent step launch per time step
      plain_fused     the same server with one slot (max_active = 1): our best single-instance path
      plain_graph_fused     one PTask FDTD graph per request shape, one request at a time: push the
                      coefficients and fields, Graph::Run of the cyclic graph lowered to the fused loop,
                      pull six fields (graphfdtd.cpp:1076-1125 is the loop this mirrors)
      plain_graph_taskwise  the same, with the H and E tasks dispatched one by one per iteration by the
                      scheduler (the reference's dispatch model)
    """
    import ptask_gb300 as P
    from ptask_gb300 import _lib
    from ptask_gb300.serve import Server, graph_dispatch

    cells = sum(r.cell_updates for r in reqs)
    peak, peak_src = hbm_peak()

    def serve(max_active):
        with Server(max_active=max_active, chunk_steps=32, persistent=True, tile_rows=rows) as s:
            for r in reqs:
                s.submit(r)
            l0 = P.launch_count()
            t0 = _lib.lib().ptk_pool_trim_count()
            s.run(time_scale=scale)
            st = s.stats()
            st["launches"] = P.launch_count() - l0
            st["pool_trims"] = _lib.lib().ptk_pool_trim_count() - t0
            return st

    def arm_of(wall, p50, p99, chunk_dev=None):
        a = {"solves_per_s": len(reqs) / wall, "mcell_updates_per_s": cells / wall / 1e6, "wall_s": wall,
             "p50_latency_s": p50, "p99_latency_s": p99}
        if chunk_dev:
            a["frac_of_peak_over_device_time"] = BYTES_PER_CELL_MAT * cells / chunk_dev / 1e9 / peak
        return a

    for _ in range(cb_warmup):
        serve(0)
    clocks = ClockSampler(local)
    clocks.start()
    runs = [serve(0) for _ in range(max(1, cb_runs))]
    clk = clocks.stop()
    best = min(runs, key=lambda st: st["wall_s"])
    wall = statistics.median(st["wall_s"] for st in runs)
    cont = arm_of(wall, best["p50_latency_s"], best["p99_latency_s"], best["chunk_device_s"])
    cont.update({"peak_active": best["peak_active"], "peak_bytes": best["peak_bytes"],
                 "chunks": best["chunks"], "graph_captures": best["graph_captures"],
                 "pool_trims": best["pool_trims"], "admit_waits": best["admit_waits"],
                 "wall_breakdown_s": {k: best[k] for k in ("wall_s", "chunk_device_s", "admit_s", "retire_s",
                                                           "schedule_s")}})
    plain = serve(1)
    out = {"requests": len(reqs), "cell_updates": cells, "tile_rows": rows or 11,
           "tile_width": 64 if rows in (7, 23) else 128, "continuous": cont,
           "plain_fused": arm_of(plain["wall_s"], plain["p50_latency_s"], plain["p99_latency_s"],
                                 plain["chunk_device_s"]),
           "gpu_launches": int(best["launches"]), "clocks": clk,
           "roofline_basis": "49 algorithmic bytes per cell update (material index) over the device time of the "
                             "replayed chunks (every step launch, faces, advances) of the whole request set; "
                             f"peak {peak:.1f} GB/s ({peak_src})"}
    for mode in graph_arms:
        g = graph_dispatch(reqs, scale, mode=mode)
        out[f"plain_graph_{mode}"] = arm_of(g["wall_s"], g["p50_latency_s"], g["p99_latency_s"])
    for name in ["plain_fused"] + [f"plain_graph_{m}" for m in graph_arms]:
        out[f"speedup_vs_{name}"] = cont["solves_per_s"] / out[name]["solves_per_s"]
    return out


def batched_desc():
    return ("batched FDTD: 64 instances in one persistent fused launch per step, edges per axis uniform in "
            "[32,192], steps uniform in [100,2000], 1-8 dielectric boxes, seeded sources, FP32")


def served_desc(n, rate):
    trace = "the workload's 20k-request trace" if n == 20000 else "the workload's 20k-request trace shortened"
    return (f"served FDTD: Poisson arrivals {rate:g} req/s, {n} requests ({trace}"
            f"{'' if rate == 200.0 else '; the workload offers 200 req/s, this rate is below saturation'}), "
            "cube edge log-uniform in [24,256], steps uniform in [50,1000], FP32, admission by HBM budget")


# Staged tile shape per workload, as measured on GB300 (same box, two runs each): the batched mix
# (x extents 32-192) serves 66.6 solves/s on 23-row, 64-wide tiles (twelve warps, one CTA per SM)
# against 64.1 on 7-row and 60.2 on 11-row tiles; the served mix (cubes up to 256) 76.3 on the
# server's default 11-row, 128-wide tiles against 69.2 on 23-row and 67.3 on 7-row tiles.
def default_rows(kind: str) -> int:
    return 23 if kind == "batched" else 0


def large_subrecord(local: int, solves: int = 3) -> dict:
    """The large workload (512x512x384, 32 boxes, 500 steps) solved from resident zero fields with the
    autotuned tiles: Mcell-updates/s over `solves` complete solves (CUDA events) and the step kernel
    against the measured HBM bandwidth at 49 (material index) or 64 bytes per cell update."""
    import ptask_gb300 as P
    from ptask_gb300.device import DeviceBuffer, Event
    wl = WORKLOADS["large"]
    shape, T = wl["shape"], wl["steps"]
    prob = P.Problem.generate(*shape, n_boxes=wl["boxes"], eps=wl["eps"], box=wl["box"], steps=T, source_mode=1,
                              seed=2)
    tiles = P.tuned_tiles(*shape)
    zero = P.zero_fields(*shape)
    dev = [DeviceBuffer.from_array(a) for a in zero]
    cells = shape[0] * shape[1] * shape[2]
    with P.Solver(prob.params) as s:
        s.set_tiles(*tiles)
        s.set_problem(prob)

        def solve():
            s.set_fields_device([b.value for b in dev])
            s.reset_clock()
            s.run(T)

        solve()   # warm-up
        clocks = ClockSampler(local)
        clocks.start()
        e0, e1 = Event(), Event()
        e0.record()
        for _ in range(solves):
            solve()
        e1.record()
        e1.sync()
        clk = clocks.stop()
        ms = e0.elapsed_ms(e1) / solves
        stages, mat = s.kernel()
    for b in dev:
        b.free()
    peak, peak_src = hbm_peak()
    bpc = BYTES_PER_CELL_MAT if mat else BYTES_PER_CELL
    achieved = bpc * cells * T / (ms / 1e3) / 1e9
    return {"workload": wl["desc"], "grid": list(shape), "time_steps": T, "solves": solves,
            "mcell_updates_per_s": cells * T / (ms / 1e3) / 1e6, "ms_per_solve": ms,
            "tiles": {"rows": tiles[0], "z_depth": tiles[1], "cells_per_thread": tiles[2], "staged_planes": stages,
                      "material_index": mat},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "peak_source": peak_src, "algorithmic_bytes_per_cell": bpc,
                         "basis": "whole solves (step launches, faces, advances) over CUDA-event time"},
            "clocks": clk}


def served_subrecords(args, rank: int, local: int) -> dict:
    """Compact batched and served records for the default bench line (one run of every arm)."""
    from ptask_gb300.serve import batched_instances, poisson_trace
    out = {}
    reqs = batched_instances(64, seed=4 + rank)
    out["batched"] = {"workload": batched_desc(),
                      **serve_arms(reqs, 0.0, args.server_rows or default_rows("batched"), cb_warmup=1, local=local)}
    for key, rate in (("served", 200.0), ("served_below_saturation", args.subsat_rate)):
        reqs = poisson_trace(args.served_requests, rate=rate, seed=5 + rank)
        out[key] = {"workload": served_desc(args.served_requests, rate), "rate_req_per_s": rate,
                    **serve_arms(reqs, 1.0, args.server_rows or default_rows("served"), local=local)}
    return out


def run_served(args, kind, world, rank, local):
    """--workload batched|served: batched (all requests at t=0) or served (Poisson arrivals) FDTD,
    continuous batching against every plain one-at-a-time arm on the same requests."""
    from ptask_gb300 import _lib
    from ptask_gb300.serve import batched_instances, poisson_trace

    _lib.call("ptk_runtime_init", local)
    if kind == "batched":
        reqs, scale, desc = batched_instances(args.instances, seed=4 + rank), 0.0, batched_desc()
        if args.instances != 64:
            desc += f"; the first {args.instances} of its 64 instances"
    else:
        reqs, scale, desc = poisson_trace(args.requests, rate=args.rate, seed=5 + rank), 1.0, served_desc(
            args.requests, args.rate)
    rows = args.server_rows or default_rows(kind)
    arms = () if args.no_plain_graph else ("fused", "taskwise")
    rec = serve_arms(reqs, scale, rows, cb_runs=args.steps, cb_warmup=args.warmup if kind == "batched" else 0,
                     graph_arms=arms, local=local)
    cont = rec["continuous"]
    peak, peak_src = hbm_peak()
    line = {
        "metric": f"FDTD {kind} solves/s", "value": cont["solves_per_s"], "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": cont["wall_s"] * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded request generator)",
        "config": {"workload": desc, "requests": len(reqs), "cell_updates": rec["cell_updates"],
                   "tile_rows": rec["tile_rows"], "tile_width": rec["tile_width"],
                   "bench_step": "serve the whole request set", "l2": "working set larger than L2"},
        "mcell_updates_per_s": cont["mcell_updates_per_s"],
        "p50_latency_s": cont["p50_latency_s"], "p99_latency_s": cont["p99_latency_s"],
        "arms": {k: rec[k] for k in rec if k.startswith("plain_") or k == "continuous"},
        "speedups": {k: v for k, v in rec.items() if k.startswith("speedup_vs_")},
        "roofline": {"bound": "hbm", "unit": "GB/s", "peak": peak, "peak_source": peak_src,
                     "achieved": cont["frac_of_peak_over_device_time"] * peak,
                     "frac": cont["frac_of_peak_over_device_time"], "traffic": None,
                     "basis": rec["roofline_basis"]},
        "gpu_launches": rec["gpu_launches"],
        "clocks": rec["clocks"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + ["batched", "served"], default="plain256")
    ap.add_argument("--requests", type=int, default=1000, help="served workload: requests in the trace")
    ap.add_argument("--instances", type=int, default=64,
                    help="batched workload: serve the first N of its 64 seeded instances (profiling runs)")
    ap.add_argument("--rate", type=float, default=200.0,
                    help="served workload: Poisson arrival rate, requests/s (200: the workload's rate)")
    ap.add_argument("--server-rows", type=int, default=0,
                    help="batched / served: staged tile rows (0: 23 for batched, the server's default 11 for "
                         "served; 7 and 23 give 64-wide tiles)")
    ap.add_argument("--tiles", default=None, help="fixed tile shape ROWS,DEPTH (skips the autotuner)")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--dense-coefficients", action="store_true",
                    help="read the four per-cell coefficient arrays instead of the material index")
    ap.add_argument("--no-graph-e2e", action="store_true",
                    help="plain workloads: skip the end-to-end run through the PTask graph API")
    ap.add_argument("--no-plain-graph", action="store_true",
                    help="batched/served: skip the two per-graph plain dispatch arms (fused and task-wise)")
    ap.add_argument("--no-served", action="store_true",
                    help="default line: leave out the batched and served sub-records")
    ap.add_argument("--no-large", action="store_true",
                    help="default line: leave out the large-grid (512x512x384) sub-record")
    ap.add_argument("--served-requests", type=int, default=300,
                    help="default line: requests in each served sub-record's trace")
    ap.add_argument("--subsat-rate", type=float, default=60.0,
                    help="default line: arrival rate of the below-saturation served sub-record, requests/s")
    args = ap.parse_args()
    world, rank, local = dist_env()
    if args.workload in ("batched", "served") and args.impl == "ours":
        return run_served(args, args.workload, world, rank, local)
    wl = WORKLOADS.get(args.workload, WORKLOADS["plain256"])
    if args.impl == "reference":
        return run_reference(args, wl, world, rank, local)
    return run_ours(args, wl, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())

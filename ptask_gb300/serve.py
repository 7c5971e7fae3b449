"""Batched and served FDTD (ptk_server_*): request traces, the server, plain-dispatch comparison."""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from ._lib import ProblemDesc, RequestInfo, ServerConfig, ServerStats, call, lib
from .fdtd import zero_fields


@dataclass
class Request:
    """One solve: a seeded problem (zero initial fields) arriving at `arrival` seconds."""
    nx: int
    ny: int
    nz: int
    steps: int
    n_boxes: int
    seed: int
    arrival: float = 0.0
    eps: tuple = (1.0, 10.0)
    box: tuple = (8, 64)
    source_mode: int = 2

    def desc(self) -> ProblemDesc:
        return ProblemDesc(self.nx, self.ny, self.nz, self.n_boxes, self.eps[0], self.eps[1], self.box[0],
                           self.box[1], 0.5, self.steps, self.source_mode, self.seed)

    @property
    def cell_updates(self) -> int:
        return self.nx * self.ny * self.nz * self.steps


def batched_instances(n: int = 64, seed: int = 4, edge=(32, 192), steps=(100, 2000), boxes=(1, 8)) -> list[Request]:
    """Batched workload: n instances, per-axis edges uniform in `edge`, steps uniform in `steps`,
    1-8 dielectric boxes, seeded source positions; all available at t=0."""
    rng = np.random.default_rng(seed)
    out = []
    for q in range(n):
        e = rng.integers(edge[0], edge[1] + 1, size=3)
        out.append(Request(int(e[0]), int(e[1]), int(e[2]), int(rng.integers(steps[0], steps[1] + 1)),
                           int(rng.integers(boxes[0], boxes[1] + 1)), seed * 100003 + q,
                           box=(4, max(4, int(e.min()) // 2))))
    return out


def poisson_trace(n: int, rate: float, seed: int = 5, edge=(24, 256), steps=(50, 1000), boxes=(1, 8)) -> list[Request]:
    """Served workload: Poisson arrivals at `rate` req/s, cube edge log-uniform in `edge`, steps
    uniform in `steps`, seeded boxes and source per request."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for q in range(n):
        t += float(rng.exponential(1.0 / rate))
        e = int(round(math.exp(rng.uniform(math.log(edge[0]), math.log(edge[1])))))
        out.append(Request(e, e, e, int(rng.integers(steps[0], steps[1] + 1)), int(rng.integers(boxes[0], boxes[1] + 1)),
                           seed * 100003 + q, arrival=t, box=(4, max(4, e // 2))))
    return out


class Server:
    """Continuous-batching FDTD server (max_active=1 gives plain one-at-a-time dispatch)."""

    def __init__(self, budget_bytes: int = 0, max_active: int = 0, chunk_steps: int = 32, tile_rows: int = 0,
                 keep_results: bool = False, persistent: bool = True, stages: int = 0):
        """`tile_rows`: 0 = 11 (128-wide tiles); 7 and 23 give 64-wide tiles (7 rows: four-warp CTAs,
        three per SM), which suit mixes of narrow requests.  `stages`: 0 = TMA-staged step kernel
        with its default ring, 2..6 = that many planes where the rows have that shape, -1 = register
        kernel.  `budget_bytes` 0 = 80 % of the free device memory at creation."""
        lib()
        self._h = C.c_void_p()
        self.cfg = ServerConfig(budget_bytes, max_active, chunk_steps, tile_rows, int(keep_results), int(persistent),
                                stages)
        call("ptk_server_create", C.byref(self.cfg), C.byref(self._h))
        self.requests: list[Request] = []

    def submit(self, r: Request) -> int:
        t = C.c_longlong()
        d = r.desc()
        call("ptk_server_submit", self._h, C.byref(d), r.arrival, C.byref(t))
        self.requests.append(r)
        return t.value

    def run(self, time_scale: float = 1.0) -> None:
        call("ptk_server_run", self._h, time_scale)

    def info(self, ticket: int) -> RequestInfo:
        i = RequestInfo()
        call("ptk_server_request", self._h, ticket, C.byref(i))
        return i

    def fetch(self, ticket: int) -> list[np.ndarray]:
        r = self.requests[ticket]
        out = zero_fields(r.nx, r.ny, r.nz)
        call("ptk_server_fetch", self._h, ticket, (C.c_void_p * 6)(*[a.ctypes.data for a in out]))
        return out

    def stats(self) -> dict:
        s = ServerStats()
        call("ptk_server_stats_get", self._h, C.byref(s))
        return s.as_dict()

    def close(self) -> None:
        if self._h:
            call("ptk_server_destroy", self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def graph_dispatch(reqs: list[Request], time_scale: float = 1.0, mode: str = "taskwise",
                   cache: int = 4, results: dict | None = None) -> dict:
    """Plain per-graph dispatch of the same requests: one PTask FDTD graph per request shape
    (ptaskUnitTest/graphfdtd.cpp builds one graph per problem size), run one request at a time in
    arrival order.  Each request pushes its coefficients and zero fields into the graph, runs its
    steps and pulls the six fields back, as the reference's graph driver does
    (graphfdtd.cpp:1076-1125).  `mode` "taskwise" dispatches the H and E tasks of every iteration
    one by one through the scheduler (the reference's model); "fused" lowers the cycle to the
    fused loop.  The next request's problem is generated on the host while the current one runs.
    Returns wall time, solves, p50/p99 latency (finish minus arrival x time_scale); with `results`
    given, also stores each request's six fields under its index."""
    import threading
    import time
    from collections import OrderedDict

    from .fdtd import Problem
    from .graph import FDTDGraph

    def make(r: Request) -> Problem:
        return Problem.generate(r.nx, r.ny, r.nz, n_boxes=r.n_boxes, eps=r.eps, box=r.box, courant=0.5,
                                steps=r.steps, source_mode=r.source_mode, seed=r.seed)

    order = sorted(range(len(reqs)), key=lambda q: reqs[q].arrival)
    slot: dict = {}

    def prefetch(q: int) -> threading.Thread:
        th = threading.Thread(target=lambda: slot.__setitem__(q, make(reqs[q])))
        th.start()
        return th

    graphs: OrderedDict = OrderedDict()
    lat = []
    pending = prefetch(order[0]) if order else None
    t0 = time.perf_counter()
    try:
        for n, q in enumerate(order):
            r = reqs[q]
            pending.join()
            prob = slot.pop(q)
            pending = prefetch(order[n + 1]) if n + 1 < len(order) else None
            wait = r.arrival * time_scale - (time.perf_counter() - t0)
            if wait > 0:
                time.sleep(wait)
            key = (r.nx, r.ny, r.nz)
            g = graphs.pop(key, None)
            if g is None:
                g = FDTDGraph(prob.params, mode=mode)
                while len(graphs) >= cache:
                    graphs.popitem(last=False)[1].close()
            graphs[key] = g
            g.set_problem(prob)
            out = g.solve(zero_fields(r.nx, r.ny, r.nz), r.steps)
            if results is not None:
                results[q] = out
            lat.append(time.perf_counter() - t0 - r.arrival * time_scale)
        wall = time.perf_counter() - t0
    finally:
        if pending is not None:
            pending.join()
        for g in graphs.values():
            g.close()
    lat_s = sorted(lat)
    pick = (lambda f: lat_s[min(len(lat_s) - 1, int(f * len(lat_s)))]) if lat_s else (lambda f: 0.0)
    return {"wall_s": wall, "solves": len(lat), "p50_latency_s": pick(0.50), "p99_latency_s": pick(0.99)}

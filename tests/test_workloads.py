"""Host side of the batched and served workloads (CPU only): the seeded request generators that
bench.py and the GPU tests use, and the problems they describe.  The same seed must give the same
requests on every host, and the requests must have the shapes the workloads name (edges per axis
uniform in [32, 192] and 100-2000 steps for the batched set; Poisson arrivals, cube edges
log-uniform in [24, 256] and 50-1000 steps for the served trace)."""
import math

import numpy as np

import ptask_gb300 as P
from ptask_gb300.serve import Request, batched_instances, poisson_trace


def test_batched_instances_ranges_and_determinism():
    a, b = batched_instances(64, seed=4), batched_instances(64, seed=4)
    assert a == b and len(a) == 64
    assert batched_instances(64, seed=5) != a
    for r in a:
        assert all(32 <= e <= 192 for e in (r.nx, r.ny, r.nz))
        assert 100 <= r.steps <= 2000 and 1 <= r.n_boxes <= 8 and r.arrival == 0.0
    total = sum(r.cell_updates for r in a)
    assert 5e10 < total < 2e11          # about 8.7e10 cell updates for the seeded set


def test_poisson_trace_statistics():
    reqs = poisson_trace(4000, rate=200.0, seed=5)
    t = np.array([r.arrival for r in reqs])
    assert np.all(np.diff(t) > 0)
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 1 / 200.0) < 0.1 / 200.0          # mean inter-arrival 5 ms
    assert abs(gaps.std() / gaps.mean() - 1.0) < 0.1           # exponential: coefficient of variation 1
    edges = np.array([r.nx for r in reqs])
    assert all(r.nx == r.ny == r.nz for r in reqs)
    assert edges.min() >= 24 and edges.max() <= 256
    logs = np.log(edges)
    mid = (math.log(24) + math.log(256)) / 2
    assert abs(np.median(logs) - mid) < 0.1                    # log-uniform: median at the log midpoint
    steps = np.array([r.steps for r in reqs])
    assert steps.min() >= 50 and steps.max() <= 1000
    assert poisson_trace(50, rate=200.0, seed=5) == reqs[:50]


def test_request_describes_the_generated_problem():
    r = Request(40, 30, 20, 55, 3, 1234, source_mode=2)
    d = r.desc()
    assert (d.Nx, d.Ny, d.Nz, d.steps, d.n_boxes, d.seed) == (40, 30, 20, 55, 3, 1234)
    prob = P.Problem.generate(r.nx, r.ny, r.nz, n_boxes=r.n_boxes, eps=r.eps, box=r.box, steps=r.steps,
                              source_mode=r.source_mode, seed=r.seed)
    again = P.Problem.generate(r.nx, r.ny, r.nz, n_boxes=r.n_boxes, eps=r.eps, box=r.box, steps=r.steps,
                               source_mode=r.source_mode, seed=r.seed)
    for a, b in zip((prob.Ca, prob.Cb, prob.Da, prob.Db, prob.wave), (again.Ca, again.Cb, again.Da, again.Db,
                                                                     again.wave)):
        np.testing.assert_array_equal(a, b)
    assert prob.Ca.shape == (20, 30, 40) and prob.wave.size == 55
    si, sj, sk = prob.src
    assert 1 <= si < 40 and 1 <= sj < 30 and 0 <= sk < 20

"""Batched and served FDTD: every result is the same alone and in the mix (bit for bit), admission
respects the HBM budget, and small requests match the oracle."""
import numpy as np
import pytest

import oracle
import ptask_gb300 as P
from ptask_gb300.serve import Request, Server, batched_instances, graph_dispatch, poisson_trace

pytestmark = pytest.mark.gpu


def alone(r: Request):
    """The same request solved alone by the single-instance solver."""
    pr = P.Problem.generate(r.nx, r.ny, r.nz, n_boxes=r.n_boxes, eps=r.eps, box=r.box, steps=r.steps,
                            source_mode=r.source_mode, seed=r.seed)
    return P.solve(pr, P.zero_fields(r.nx, r.ny, r.nz), r.steps), pr


@pytest.mark.parametrize("rows,stages", [(0, 0), (8, 0), (8, -1), (4, 3), (8, 2), (10, 5), (23, 0), (23, 3), (7, 4)])
def test_mixed_batch_results_equal_alone(rows, stages):
    """Staged (default ring, 2-plane ring, 4 rows) and register kernels all give the solo results."""
    reqs = [Request(24, 20, 16, 40, 2, 1), Request(37, 29, 23, 75, 3, 2), Request(64, 48, 40, 33, 1, 3),
            Request(17, 33, 9, 61, 2, 4), Request(130, 24, 20, 20, 4, 5), Request(40, 36, 230, 9, 3, 6)]
    with Server(keep_results=True, chunk_steps=16, tile_rows=rows, stages=stages) as s:
        tickets = [s.submit(r) for r in reqs]
        s.run(time_scale=0)
        st = s.stats()
        assert st["completed"] == len(reqs) and st["peak_active"] == len(reqs)
        for t, r in zip(tickets, reqs):
            got = s.fetch(t)
            ref, _ = alone(r)
            for q in range(6):
                np.testing.assert_array_equal(got[q], ref[q], err_msg=f"request {t} field {P.FIELDS[q]}")


def test_checksums_are_fp64_sums_and_deterministic():
    """A request's checksums are the FP64 sums of its six result fields, with the same bits on every run."""
    reqs = [Request(24, 20, 16, 40, 2, 21), Request(130, 37, 29, 25, 3, 22), Request(9, 70, 33, 18, 1, 23)]
    runs = []
    for _ in range(2):
        with Server(keep_results=True, chunk_steps=16) as s:
            tickets = [s.submit(r) for r in reqs]
            s.run(time_scale=0)
            runs.append([(list(s.info(t).checksum), s.fetch(t)) for t in tickets])
    for (sums_a, fields), (sums_b, _) in zip(*runs):
        assert sums_a == sums_b
        for q in range(6):
            f64 = fields[q].astype(np.float64)
            assert abs(sums_a[q] - f64.sum()) <= 1e-12 * max(np.abs(f64).sum(), 1e-300)


def test_batched_small_requests_match_oracle():
    reqs = [Request(20, 18, 14, 30, 2, 11), Request(26, 22, 12, 45, 1, 12)]
    with Server(keep_results=True, chunk_steps=8, persistent=False) as s:
        tickets = [s.submit(r) for r in reqs]
        s.run(time_scale=0)
        for t, r in zip(tickets, reqs):
            got = s.fetch(t)
            _, pr = alone(r)
            ref = oracle.step_ext_f32(P.zero_fields(r.nx, r.ny, r.nz), r.steps, pr.params, pr.Ca, pr.Cb, pr.Da,
                                      pr.Db, pr.src, pr.wave)
            for q in range(6):
                assert oracle.normwise_error(got[q], ref[q]) <= 1e-5
                np.testing.assert_array_equal(got[q], ref[q])


def test_continuous_admission_within_budget_and_plain_mode_agrees():
    reqs = poisson_trace(24, rate=400.0, seed=9, edge=(16, 72), steps=(20, 120))
    # a budget that holds only a few instances at a time
    budget = 3 * 16 * 4 * (96 * 73 * 73) + (1 << 20)
    with Server(budget_bytes=budget, keep_results=True, chunk_steps=8) as s:
        tickets = [s.submit(r) for r in reqs]
        s.run(time_scale=1.0)
        st = s.stats()
        assert st["completed"] == len(reqs)
        assert st["peak_bytes"] <= budget
        batched = {t: s.fetch(t) for t in tickets}
        lat = [s.info(t).finish_s - s.info(t).arrival_s for t in tickets]
        assert min(lat) >= 0
    with Server(max_active=1, keep_results=True, chunk_steps=8) as s:
        tickets = [s.submit(r) for r in reqs]
        s.run(time_scale=0)
        assert s.stats()["peak_active"] == 1
        for t in tickets:
            got = s.fetch(t)
            for q in range(6):
                np.testing.assert_array_equal(got[q], batched[t][q])


@pytest.mark.parametrize("mode", ["taskwise", "fused"])
def test_plain_graph_dispatch_matches_server(mode):
    """The per-graph plain arms (one PTask graph per request, task-wise or lowered to the fused loop)
    give the server's results."""
    reqs = poisson_trace(6, rate=2000.0, seed=13, edge=(12, 40), steps=(10, 40))
    reqs.append(Request(reqs[0].nx, reqs[0].ny, reqs[0].nz, 17, 2, 77, arrival=reqs[-1].arrival))  # graph reuse
    got: dict = {}
    st = graph_dispatch(reqs, time_scale=1.0, mode=mode, cache=2, results=got)
    assert st["solves"] == len(reqs) and st["p99_latency_s"] >= st["p50_latency_s"] >= 0
    with Server(keep_results=True, chunk_steps=8) as s:
        tickets = [s.submit(r) for r in reqs]
        s.run(time_scale=0)
        for q, t in enumerate(tickets):
            ref = s.fetch(t)
            for f in range(6):
                np.testing.assert_array_equal(got[q][f], ref[f], err_msg=f"request {q} field {P.FIELDS[f]}")


def test_request_larger_than_budget_is_rejected():
    with Server(budget_bytes=1 << 20) as s:
        with pytest.raises(P.PtkError):
            s.submit(Request(64, 64, 64, 10, 1, 1))


def test_server_rejects_unknown_staged_shape():
    with pytest.raises(P.PtkError):
        Server(tile_rows=16, stages=3)


def test_batched_config_generator_shapes():
    reqs = batched_instances(64)
    assert len(reqs) == 64
    e = np.array([[r.nx, r.ny, r.nz] for r in reqs])
    assert e.min() >= 32 and e.max() <= 192
    assert all(100 <= r.steps <= 2000 for r in reqs)
    assert all(1 <= r.n_boxes <= 8 for r in reqs)


def test_many_work_lists_evict_cached_graphs_and_stay_exact():
    """Hundreds of small requests finishing at staggered steps give hundreds of different work lists;
    the server keeps at most 256 chunk graphs (evicting all but the one a queued chunk replays) and
    every result still equals the solo solve."""
    # every request finishes at a step of its own: 320 chunk boundaries, each a new work list
    reqs = [Request(8 + q % 7, 8 + (q * 3) % 5, 6 + q % 4, 3 + q, 1, 1000 + q) for q in range(320)]
    with Server(keep_results=True, chunk_steps=4) as s:
        tickets = [s.submit(r) for r in reqs]
        s.run(time_scale=0)
        st = s.stats()
        assert st["completed"] == len(reqs) and st["graph_captures"] > 256
        for q in range(0, len(reqs), 29):
            got = s.fetch(tickets[q])
            ref, _ = alone(reqs[q])
            for f in range(6):
                np.testing.assert_array_equal(got[f], ref[f], err_msg=f"request {q} field {P.FIELDS[f]}")


@pytest.mark.parametrize("rows", [23, 7, 0])
def test_full_batched_set_matches_oracle(rows):
    """The whole 64-instance batched workload (per-axis edges 32-192, 100-2000 steps, the set the
    benchmark serves), run in one continuous-batching mix with the benchmark's 23-row, 64-wide tiles,
    the 7-row, 64-wide ones and the server's default 11-row, 128-wide ones.  A seeded subset of 8 instances, always
    including the largest, is compared with the FP32 oracle (graphfdtd.cpp:314-340 restated) bit for
    bit, and the checksums of those instances with their fields."""
    reqs = batched_instances(64, seed=4)
    largest = max(range(len(reqs)), key=lambda q: reqs[q].cell_updates)
    rng = np.random.default_rng(17 + rows)
    pick = sorted({largest, *(int(q) for q in rng.choice(len(reqs), 7, replace=False))})
    with Server(keep_results=True, chunk_steps=32, tile_rows=rows) as s:
        tickets = [s.submit(r) for r in reqs]
        s.run(time_scale=0)
        st = s.stats()
        assert st["completed"] == len(reqs) and st["peak_active"] == len(reqs)
        fetched = {q: s.fetch(tickets[q]) for q in pick}
        sums = {q: list(s.info(tickets[q]).checksum) for q in pick}
    for q in pick:
        r = reqs[q]
        pr = P.Problem.generate(r.nx, r.ny, r.nz, n_boxes=r.n_boxes, eps=r.eps, box=r.box, steps=r.steps,
                                source_mode=r.source_mode, seed=r.seed)
        ref =oracle.step_ext_f32(P.zero_fields(r.nx, r.ny, r.nz), r.steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db,
                                  pr.src, pr.wave)
        for f in range(6):
            got = fetched[q][f]
            assert oracle.normwise_error(got, ref[f]) <= 1e-5
            np.testing.assert_array_equal(got, ref[f], err_msg=f"instance {q} ({r.nx}x{r.ny}x{r.nz} x {r.steps}) "
                                                               f"field {P.FIELDS[f]}")
            f64 = got.astype(np.float64)
            assert abs(sums[q][f] - f64.sum()) <= 1e-12 * max(np.abs(f64).sum(), 1e-300)


def test_served_trace_matches_oracle():
    """The first 200 requests of the served workload's Poisson trace (200 req/s, cube edges 24-256,
    50-1000 steps, the trace the benchmark serves) admitted as they arrive, by HBM budget, with the
    server's default tiles.  Eight requests, always including the largest (255^3, 971 steps), are
    compared with the FP32 oracle bit for bit."""
    reqs = poisson_trace(200, rate=200.0, seed=5)
    largest = max(range(len(reqs)), key=lambda q: reqs[q].cell_updates)
    rng = np.random.default_rng(23)
    pick = sorted({largest, *(int(q) for q in rng.choice(len(reqs), 7, replace=False))})
    with Server(keep_results=True) as s:
        tickets = [s.submit(r) for r in reqs]
        s.run(time_scale=1.0)
        assert s.stats()["completed"] == len(reqs)
        fetched = {q: s.fetch(tickets[q]) for q in pick}
    for q in pick:
        r = reqs[q]
        pr = P.Problem.generate(r.nx, r.ny, r.nz, n_boxes=r.n_boxes, eps=r.eps, box=r.box, steps=r.steps,
                                source_mode=r.source_mode, seed=r.seed)
        ref = oracle.step_ext_f32(P.zero_fields(r.nx, r.ny, r.nz), r.steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db,
                                  pr.src, pr.wave)
        for f in range(6):
            assert oracle.normwise_error(fetched[q][f], ref[f]) <= 1e-5
            np.testing.assert_array_equal(fetched[q][f], ref[f], err_msg=f"request {q} ({r.nx}^3 x {r.steps}) "
                                                                         f"field {P.FIELDS[f]}")

"""Init/teardown cycles leave no device memory behind.

The reference stresses its runtime's setup and teardown with repeated create-run-destroy cycles
(ptaskUnitTest/rttests.cpp, entry points in rttests.h:10-145).  Here every host object on the FDTD
path (the unrolled and cyclic PTask graphs in each lowering, the resident solver, the serving
engine) is created, used and destroyed several times; after the first cycle, which may set up
process-wide state once (pinned staging, autotuned shapes, kernel attributes), the device pool's
used bytes never grow from one cycle to the next, and every result matches the oracle.
"""
import ctypes as C
import gc

import numpy as np
import pytest

import oracle
import ptask_gb300 as P
from ptask_gb300 import _lib
from ptask_gb300.graph import FDTDGraph
from ptask_gb300.serve import Request, Server

pytestmark = pytest.mark.gpu


def pool_used() -> int:
    gc.collect()   # objects left by earlier tests are freed now, not in the middle of the check
    _lib.call("ptk_device_sync")
    reserved, used = C.c_size_t(), C.c_size_t()
    _lib.call("ptk_pool_stats", C.byref(reserved), C.byref(used))
    return used.value


def one_cycle():
    shape, steps = (30, 22, 17), 6
    pr = P.Problem.generate(*shape, n_boxes=2, eps=(2, 6), box=(3, 9), steps=steps, seed=71)
    f = P.random_fields(*shape, seed=72, scale=1e-3)
    ref = oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    for mode in ("fused", "captured", "taskwise"):
        with FDTDGraph(pr.params, mode) as g:
            g.set_problem(pr)
            got = g.solve(f, steps)
        for q in range(6):
            np.testing.assert_array_equal(got[q], ref[q], err_msg=f"cyclic graph ({mode}) {P.FIELDS[q]}")
    p = P.reference_params(*shape)
    vref = oracle.step_ref_f32(f, 3, p)
    with FDTDGraph(p, "unrolled", unrolled_steps=3) as g:
        got = g.solve(f, 3)
    for q in range(6):
        np.testing.assert_array_equal(got[q], vref[q], err_msg=f"unrolled graph {P.FIELDS[q]}")
    with P.Solver(pr.params) as s:
        s.set_tiles(11, 0, 4, 4)
        s.set_problem(pr)
        s.set_fields(f)
        s.run(steps)
        got = s.get_fields()
    for q in range(6):
        np.testing.assert_array_equal(got[q], ref[q], err_msg=f"solver {P.FIELDS[q]}")
    reqs = [Request(24, 20, 16, 12, 2, 81), Request(37, 29, 23, 9, 1, 82), Request(70, 18, 12, 15, 3, 83)]
    with Server(keep_results=True, chunk_steps=8) as srv:
        tickets = [srv.submit(r) for r in reqs]
        srv.run(time_scale=0)
        assert srv.stats()["completed"] == len(reqs)
        srv.fetch(tickets[0])


def test_create_use_destroy_cycles_leave_no_device_memory():
    one_cycle()            # process-wide one-time setup happens here
    base = pool_used()
    with P.Solver(P.reference_params(30, 22, 17)) as s:   # the measure sees a live object's arrays
        s.set_vacuum()
        assert pool_used() > base
    for _ in range(3):
        one_cycle()
        assert pool_used() <= base, "device memory left allocated after graphs, solvers and servers were destroyed"

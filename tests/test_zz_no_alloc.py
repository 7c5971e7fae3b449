"""The allocation-free entry point, ptk_fdtd_solve_static, checked against the allocating one.

Who needs it: callers that cannot let a library allocate GPU memory -- code that runs while another
component captures the stream into a CUDA graph, plugins whose host application owns the device
memory, latency-critical loops that must not risk an allocation failure.  The entry point keeps its
scratch in one static device array shared by all calls, so the test runs two calls in a row (the
second one sees the first call's leftovers) and compares each with ptk_solver_* (which allocates),
within the tolerance the other parity tests use.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
import ptask_gb300 as P
from ptask_gb300 import _lib
from ptask_gb300.device import DeviceBuffer, Stream

pytestmark = pytest.mark.gpu
TOL = 1e-5
V = C.c_void_p


def static_solve(pr, fields, steps, vacuum=False):
    """Run ptk_fdtd_solve_static on device copies of `fields` (the test allocates; the call does not)."""
    bufs = [DeviceBuffer.from_array(a) for a in fields]
    coefs = [] if vacuum else [DeviceBuffer.from_array(a) for a in (pr.Ca, pr.Cb, pr.Da, pr.Db)]
    wave = DeviceBuffer.from_array(pr.wave) if (pr.has_source and pr.wave.size) else None
    src = pr.src if wave is not None else (-1, -1, -1)
    st = Stream()
    _lib.call("ptk_fdtd_solve_static", C.byref(pr.params), (V * 6)(*[b.ptr for b in bufs]),
              *([c.ptr for c in coefs] if coefs else [None] * 4), *src,
              wave.ptr if wave is not None else None, int(pr.wave.size) if wave is not None else 0, steps,
              st.handle)
    st.sync()
    st.close()
    out = [b.download(a.shape) for b, a in zip(bufs, fields)]
    for b in bufs + coefs + ([wave] if wave is not None else []):
        b.free()
    return out


def solver_solve(pr, fields, steps, vacuum=False):
    with P.Solver(pr.params) as s:
        s.set_fields(fields)
        if vacuum:
            s.set_vacuum()
        else:
            s.set_problem(pr)
        s.run(steps)
        return s.get_fields()


def close(got, ref, what):
    for q, (g, r) in enumerate(zip(got, ref)):
        err = oracle.normwise_error(g, r)
        assert err <= TOL, f"{what} {P.FIELDS[q]}: normwise error {err:.3e}"


def test_static_solve_matches_solver_twice_in_a_row():
    # first call: dielectric problem with a source, larger grid
    pr1 = P.Problem.generate(48, 40, 36, n_boxes=4, eps=(1, 10), box=(4, 20), steps=45, seed=11)
    f1 = P.random_fields(48, 40, 36, seed=61, scale=1e-3)
    got1 = static_solve(pr1, f1, 45)
    close(got1, solver_solve(pr1, f1, 45), "call 1")
    # second call: smaller grid, odd step count, vacuum coefficients, no source; the scratch still
    # holds the first call's larger state
    p2 = P.reference_params(30, 22, 17)
    pr2 = P.Problem.vacuum(p2)
    f2 = P.random_fields(30, 22, 17, seed=62)
    got2 = static_solve(pr2, f2, 13, vacuum=True)
    close(got2, solver_solve(pr2, f2, 13, vacuum=True), "call 2")


def test_static_solve_rejects_grids_beyond_its_scratch():
    limit = int(_lib.lib().ptk_fdtd_static_scratch_bytes())
    assert limit == 48 << 20
    p = P.reference_params(128, 128, 128)
    bufs = [DeviceBuffer(16) for _ in range(6)]   # never touched: the size check comes first
    rc = _lib.lib().ptk_fdtd_solve_static(C.byref(p), (V * 6)(*[b.ptr for b in bufs]), None, None, None, None,
                                          -1, -1, -1, None, 0, 1, None)
    for b in bufs:
        b.free()
    assert rc == 6   # PTK_ERR_BUDGET
    assert b"limited to" in _lib.lib().ptk_last_error()

"""The allocation-free entry point, ptk_fdtd_solve_static.

Some callers cannot let this library allocate device memory: a plugin inside an application that
hands out all GPU memory from its own arena and budget, and latency-critical loops for which a
cudaMalloc (which may synchronise the device and may fail partway through a run) is not acceptable.
ptk_fdtd_solve_static serves them by keeping its scratch in one fixed-size static device array that
every call shares, so these tests check:

  * two calls in a row (the second one sees the first call's leftovers in the shared array) give
    the oracle's results bit for bit, and the same results as the allocating entry point
    (ptk_solver_*);
  * a call allocates nothing: the runtime's pool counters and the device's free memory are the same
    before and after it;
  * grids beyond the array's size are rejected before any device work, and the largest cube that
    fits (89^3) is accepted.

This file is collected last on purpose, so that a run stopping at its first failure has already run
every other test.  The test allocates its own inputs and outputs; only the calls under test must not.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
import ptask_gb300 as P
from ptask_gb300 import _lib
from ptask_gb300.device import DeviceBuffer, Stream

pytestmark = pytest.mark.gpu
TOL = 1e-5   # normwise tolerance of every parity test; bit-exactness is asserted as well
V = C.c_void_p


class StaticCall:
    """Device copies of one problem's inputs, made by the test, and the call under test on them."""

    def __init__(self, pr, fields, vacuum=False):
        self.pr, self.fields, self.vacuum = pr, fields, vacuum
        self.bufs = [DeviceBuffer.from_array(a) for a in fields]
        self.coefs = [] if vacuum else [DeviceBuffer.from_array(a) for a in (pr.Ca, pr.Cb, pr.Da, pr.Db)]
        self.wave = DeviceBuffer.from_array(pr.wave) if (pr.has_source and pr.wave.size) else None
        self.stream = Stream()

    def run(self, steps):
        """Upload the initial fields, call ptk_fdtd_solve_static, return the six fields."""
        for b, a in zip(self.bufs, self.fields):
            b.upload(a)
        src = self.pr.src if self.wave is not None else (-1, -1, -1)
        _lib.call("ptk_fdtd_solve_static", C.byref(self.pr.params), (V * 6)(*[b.ptr for b in self.bufs]),
                  *([c.ptr for c in self.coefs] if self.coefs else [None] * 4), *src,
                  self.wave.ptr if self.wave is not None else None,
                  int(self.pr.wave.size) if self.wave is not None else 0, steps, self.stream.handle)
        self.stream.sync()
        return [b.download(a.shape) for b, a in zip(self.bufs, self.fields)]

    def close(self):
        self.stream.close()
        for b in self.bufs + self.coefs + ([self.wave] if self.wave is not None else []):
            b.free()


def oracle_solve(pr, fields, steps, vacuum=False):
    if vacuum:
        return oracle.step_ref_f32(fields, steps, pr.params)
    return oracle.step_ext_f32(fields, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)


def solver_solve(pr, fields, steps, vacuum=False):
    with P.Solver(pr.params) as s:
        s.set_fields(fields)
        if vacuum:
            s.set_vacuum()
        else:
            s.set_problem(pr)
        s.run(steps)
        return s.get_fields()


def same(got, ref, what):
    for q, (g, r) in enumerate(zip(got, ref)):
        err = oracle.normwise_error(g, r)
        assert err <= TOL, f"{what} {P.FIELDS[q]}: normwise error {err:.3e}"
        assert np.array_equal(g, r), f"{what} {P.FIELDS[q]}: not bit-identical (normwise {err:.3e})"


def dielectric_case():
    pr = P.Problem.generate(48, 40, 36, n_boxes=4, eps=(1, 10), box=(4, 20), steps=45, seed=11)
    return pr, P.random_fields(48, 40, 36, seed=61, scale=1e-3), 45


def vacuum_case():
    p = P.reference_params(30, 22, 17)
    return P.Problem.vacuum(p), P.random_fields(30, 22, 17, seed=62), 13


def test_static_solve_twice_in_a_row_matches_oracle_and_solver():
    # first call: dielectric boxes and a source on the larger grid
    pr1, f1, n1 = dielectric_case()
    c1 = StaticCall(pr1, f1)
    got1 = c1.run(n1)
    c1.close()
    same(got1, oracle_solve(pr1, f1, n1), "call 1 vs oracle")
    same(got1, solver_solve(pr1, f1, n1), "call 1 vs ptk_solver")
    # second call: a smaller grid, an odd step count, vacuum coefficients and no source, while the
    # shared array still holds the first call's larger state
    pr2, f2, n2 = vacuum_case()
    c2 = StaticCall(pr2, f2, vacuum=True)
    got2 = c2.run(n2)
    c2.close()
    same(got2, oracle_solve(pr2, f2, n2, vacuum=True), "call 2 vs oracle")
    same(got2, solver_solve(pr2, f2, n2, vacuum=True), "call 2 vs ptk_solver")


def pool_and_free():
    reserved, used = C.c_size_t(), C.c_size_t()
    _lib.call("ptk_pool_stats", C.byref(reserved), C.byref(used))
    return reserved.value, used.value, P.device_info()["free"]


def test_static_solve_allocates_nothing():
    pr, f, n = dielectric_case()
    call = StaticCall(pr, f)        # inputs and outputs: allocated by the caller, before the check
    first = call.run(n)             # a first call on the device looks up the array's address
    before = pool_and_free()
    again = call.run(n)
    after = pool_and_free()
    call.close()
    assert after == before, f"pool (reserved, used) and device free bytes changed: {before} -> {after}"
    same(again, first, "repeated call")


def test_static_solve_size_limit():
    limit = int(_lib.lib().ptk_fdtd_static_scratch_bytes())
    assert limit == 48 << 20
    # 90^3 is the first cube that needs more than the array: rejected before any device access
    p = P.reference_params(90, 90, 90)
    bufs = [DeviceBuffer(16) for _ in range(6)]   # never touched: the size check comes first
    rc = _lib.lib().ptk_fdtd_solve_static(C.byref(p), (V * 6)(*[b.ptr for b in bufs]), None, None, None, None,
                                          -1, -1, -1, None, 0, 1, None)
    for b in bufs:
        b.free()
    assert rc == 6   # PTK_ERR_BUDGET
    assert b"limited to" in _lib.lib().ptk_last_error()
    # 89^3 (pitch 96 x 90 x 90 padded nodes) is the largest cube that fits
    p = P.reference_params(89, 89, 89)
    pr = P.Problem.vacuum(p)
    f = P.random_fields(89, 89, 89, seed=63)
    call = StaticCall(pr, f, vacuum=True)
    got = call.run(3)
    call.close()
    same(got, oracle_solve(pr, f, 3, vacuum=True), "89^3 vs oracle")

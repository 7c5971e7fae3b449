"""Parity of the sm_103a FDTD kernels with the oracle, through the C ABI.

Bar: bit-exact equality with the FP32 oracle (the kernels round every operation separately, like the
reference's host code), and in every case also the stated tolerance of max normwise relative error
1e-5 per field.  The error against the FP64 oracle is reported.
"""
import ctypes as C
import hashlib

import numpy as np
import pytest

import oracle
import ptask_gb300 as P
from ptask_gb300 import _lib
from ptask_gb300.device import DeviceBuffer
from conftest import params_of

pytestmark = pytest.mark.gpu
TOL = 1e-5          # max_i |gpu - ref| / max_i |ref|, per field


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def assert_parity(got, ref, what=""):
    for q, (g, r) in enumerate(zip(got, ref)):
        err = oracle.normwise_error(g, r)
        assert err <= TOL, f"{what} {P.FIELDS[q]}: normwise error {err:.3e} > {TOL}"
        if not np.array_equal(g, r):
            bad = np.argwhere(g != r)
            raise AssertionError(f"{what} {P.FIELDS[q]}: {len(bad)} cells differ, first at (k,j,i)="
                                 f"{tuple(bad[0])}: gpu={g[tuple(bad[0])]!r} ref={r[tuple(bad[0])]!r}")


def run_field_tasks(fields, steps, p):
    """The reference's six tasks per step (HxComputation..EzComputation), dense layout, ping-pong."""
    nx, ny, nz = p.Nx, p.Ny, p.Nz
    cur = [DeviceBuffer.from_array(f) for f in fields]
    nxt = [DeviceBuffer(f.nbytes) for f in fields]
    ins = {0: (0, 4, 5), 1: (1, 3, 5), 2: (2, 3, 4), 3: (3, 1, 2), 4: (4, 0, 2), 5: (5, 0, 1)}
    for _ in range(steps):
        for f in range(6):
            a, b, c = ins[f]
            # H tasks read old E; E tasks read new H (graphfdtd.cpp:606-615)
            src = [cur[a], nxt[b] if f >= 3 else cur[b], nxt[c] if f >= 3 else cur[c]]
            _lib.call("ptk_launch_field_update", f, src[0].ptr, src[1].ptr, src[2].ptr, C.byref(p),
                      nxt[f].ptr, None)
        cur, nxt = nxt, cur
    out = [cur[f].download(P.field_shape(f, nx, ny, nz)) for f in range(6)]
    for b in cur + nxt:
        b.free()
    return out


@pytest.mark.parametrize("shape,steps", [((5, 7, 3), 3), ((33, 17, 9), 5), ((64, 64, 4), 4),
                                         ((1, 1, 1), 2), ((130, 9, 6), 3)])
def test_reference_task_kernels_bitwise(shape, steps):
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=21)
    assert_parity(run_field_tasks(f, steps, p), oracle.step_ref_f32(f, steps, p), "task kernels")


@pytest.mark.parametrize("shape,steps", [((5, 7, 3), 3), ((40, 24, 10), 6)])
def test_half_step_kernels_bitwise(shape, steps):
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=22)
    cur = [DeviceBuffer.from_array(a) for a in f]
    nxt = [DeviceBuffer(a.nbytes) for a in f]
    V = C.c_void_p
    for _ in range(steps):
        _lib.call("ptk_launch_h_half_step", (V * 6)(*[b.ptr for b in cur]), (V * 3)(*[b.ptr for b in nxt[:3]]),
                  C.byref(p), None)
        _lib.call("ptk_launch_e_half_step", (V * 3)(*[b.ptr for b in cur[3:]]), (V * 3)(*[b.ptr for b in nxt[:3]]),
                  (V * 3)(*[b.ptr for b in nxt[3:]]), C.byref(p), None)
        cur, nxt = nxt, cur
    got = [cur[q].download(P.field_shape(q, *shape)) for q in range(6)]
    assert_parity(got, oracle.step_ref_f32(f, steps, p), "half steps")


def test_golden_cases_through_solver(golden):
    """The fused solver in vacuum mode reproduces the reference's own outputs (golden hashes)."""
    for case in golden["cases"]:
        p = params_of(case)
        f = P.random_fields(case["Nx"], case["Ny"], case["Nz"], seed=case["seed"])
        assert [sha(a) for a in f] == case["input_sha256"]
        with P.Solver(p) as s:
            s.set_fields(f)
            s.set_vacuum()
            s.run(case["steps"])
            out = s.get_fields()
        assert [sha(a) for a in out] == case["output_sha256"], case["name"]


SHAPES = [(5, 7, 3), (1, 1, 1), (2, 2, 2), (1, 5, 3), (4, 1, 6), (129, 3, 2), (127, 11, 5),
          (33, 17, 9), (200, 13, 17), (64, 48, 40)]


@pytest.mark.parametrize("shape", SHAPES)
def test_solver_reference_mode_bitwise(shape):
    steps = 7
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=31)
    ref = oracle.step_ref_f32(f, steps, p)
    with P.Solver(p) as s:
        s.set_fields(f)
        s.set_vacuum()
        s.run(steps)
        assert_parity(s.get_fields(), ref, f"solver {shape}")


@pytest.mark.parametrize("by", [4, 8, 16])
@pytest.mark.parametrize("kc", [0, 1, 3, 16])
@pytest.mark.parametrize("vec", [1, 2, 4])
def test_tile_shapes_agree(by, kc, vec):
    shape, steps = (150, 37, 21), 5
    pr = P.Problem.generate(*shape, n_boxes=3, eps=(1, 10), box=(5, 30), steps=steps, seed=4)
    f = P.random_fields(*shape, seed=32, scale=1e-2)
    ref = oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    with P.Solver(pr.params) as s:
        s.set_tiles(by, kc, vec)
        s.set_fields(f)
        s.set_problem(pr)
        s.run(steps)
        assert_parity(s.get_fields(), ref, f"tiles by={by} kc={kc} vec={vec}")


@pytest.mark.parametrize("shape,boxes,steps", [((32, 32, 32), 2, 100), ((48, 40, 36), 8, 120),
                                               ((67, 45, 23), 5, 64)])
def test_dielectric_source_problem_bitwise(shape, boxes, steps):
    """Config-1 style problems: zero-init fields, dielectric boxes, Courant 0.5, Gaussian source."""
    pr = P.Problem.generate(*shape, n_boxes=boxes, eps=(2, 6), box=(4, 16), steps=steps, seed=1)
    f = P.zero_fields(*shape)
    ref = oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    got = P.solve(pr, f, steps)
    assert_parity(got, ref, f"problem {shape}")
    ref64 = oracle.step_ext_f64(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    e64 = max(oracle.normwise_error(g, r) for g, r in zip(got, ref64))
    print(f"\n{shape} x {steps}: max normwise error vs FP64 oracle = {e64:.2e}")
    assert e64 < 1e-3


def test_run_split_and_chunking_is_invisible():
    """run(a)+run(b) == run(a+b): step counter, ping-pong parity and source clock carry across calls."""
    shape, steps = (40, 30, 20), 77
    pr = P.Problem.generate(*shape, n_boxes=2, steps=steps, seed=6)
    f = P.zero_fields(*shape)
    outs = []
    for parts in ([77], [1, 76], [33, 31, 13], [32, 32, 13]):
        with P.Solver(pr.params) as s:
            s.set_fields(f)
            s.set_problem(pr)
            for n in parts:
                s.run(n)
            outs.append(s.get_fields())
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("tiles", [(11, 5, 4, 4), (8, 0, 4, 0)])
def test_reset_clock_after_odd_steps(tiles):
    """reset_clock after an odd step count swaps the buffer roles; the next run (staged kernel
    tensor maps included) must continue from the current fields.  No source, so the clock
    restart does not change the result: run(3) + reset + run(4) == run(7)."""
    shape = (150, 37, 21)
    pr = P.Problem.generate(*shape, n_boxes=3, eps=(1, 10), box=(5, 30), steps=7, seed=16)
    pr = P.Problem(pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, (-1, -1, -1), np.zeros(0, np.float32))
    f = P.random_fields(*shape, seed=75, scale=1e-2)
    ref = oracle.step_ext_f32(f, 7, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db)
    with P.Solver(pr.params) as s:
        s.set_tiles(*tiles)
        s.set_fields(f)
        s.set_problem(pr)
        s.run(3)
        s.reset_clock()
        s.run(4)
        assert_parity(s.get_fields(), ref, f"reset_clock {tiles}")


def test_one_call_solve_with_host_buffers():
    shape, steps = (24, 20, 16), 30
    pr = P.Problem.generate(*shape, n_boxes=2, steps=steps, seed=9)
    f = P.random_fields(*shape, seed=3, scale=1e-3)
    ref = oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    arrs = [a.copy() for a in f]
    V = C.c_void_p
    ms = C.c_float()
    _lib.call("ptk_fdtd_solve", C.byref(pr.params), (V * 6)(*[a.ctypes.data for a in arrs]),
              pr.Ca.ctypes.data, pr.Cb.ctypes.data, pr.Da.ctypes.data, pr.Db.ctypes.data, *pr.src,
              pr.wave.ctypes.data, pr.wave.size, steps, C.byref(ms))
    assert_parity(arrs, ref, "ptk_fdtd_solve")
    assert ms.value > 0


def test_launch_counter_counts_graph_nodes():
    p = P.reference_params(16, 16, 16)
    with P.Solver(p) as s:
        before = P.launch_count()
        s.run(70)
        assert s.last_launches() == 70 + 3          # 3 graphs (32+32+6 steps) each with one advance node
        assert P.launch_count() - before >= 73


def test_bad_source_rejected():
    p = P.reference_params(8, 8, 8)
    with P.Solver(p) as s:
        w = np.ones(4, np.float32)
        with pytest.raises(_lib.PtkError):
            _lib.call("ptk_solver_set_source", s.handle, 0, 3, 3, w.ctypes.data, 4, 0, None)
        with pytest.raises(_lib.PtkError):
            s.set_tiles(5, 0)
        with pytest.raises(_lib.PtkError):
            s.set_tiles(8, 0, 4, 1)      # a one-stage ring cannot make progress: rejected
        with pytest.raises(_lib.PtkError):
            s.set_tiles(16, 0, 4, 3)     # three 16-row stages exceed shared memory: no such kernel


# ------------------------------------------------------------------------------------------------
# Full-size properties (256^3, the plain-graph benchmark size).  The oracle checks a few steps at full
# size exactly; longer runs are checked through properties that hold bit for bit.
# ------------------------------------------------------------------------------------------------
FULL = (256, 256, 256)


@pytest.fixture(scope="module")
def full_problem():
    return P.Problem.generate(*FULL, n_boxes=8, eps=(1, 10), box=(8, 64), steps=1000, seed=2)


def test_full_size_first_steps_match_oracle(full_problem):
    pr = full_problem
    f = P.random_fields(*FULL, seed=41, scale=1e-3)
    steps = 3
    ref = oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    got = P.solve(pr, f, steps)
    assert_parity(got, ref, "256^3 x 3")


@pytest.mark.parametrize("tiles", [(11, 82, 4, 4), (23, 82, 2, 4), (11, 84, 4, 4)])
def test_full_size_thin_last_layer_matches_oracle(full_problem, tiles):
    """256^3 cut into three layers of 82 or 84 planes that occupy 144 of the resident CTAs and a thin
    last layer of 4-10 planes that the remaining CTAs claim one tile after another while the layers
    run (the solver's late tile claim); 12 steps, bit for bit against the oracle."""
    pr = full_problem
    f = P.random_fields(*FULL, seed=43, scale=1e-3)
    steps = 12
    ref = oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    with P.Solver(pr.params) as s:
        s.set_tiles(*tiles)
        s.set_problem(pr)
        s.set_fields(f)
        s.run(steps)
        assert s.kernel() == (4, True)
        assert_parity(s.get_fields(), ref, f"256^3 x {steps}, tiles {tiles}")


def test_full_size_full_length_matches_oracle(full_problem):
    """The plain-graph workload itself (256^3, 1000 steps from zero fields) with the autotuned
    tiles, bit for bit against the FP32 oracle."""
    pr = full_problem
    f = P.zero_fields(*FULL)
    with P.Solver(pr.params) as s:
        s.set_tiles(*P.tuned_tiles(*FULL))
        s.set_fields(f)
        s.set_problem(pr)
        s.run(1000)
        got = s.get_fields()
    ref = oracle.step_ext_f32(f, 1000, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    assert_parity(got, ref, "256^3 x 1000")


LARGE = (512, 512, 384)


def test_large_config_full_length_matches_oracle():
    """The large single-GPU workload itself (512x512x384, 32 seeded dielectric boxes, 500 steps from
    zero fields, as the benchmark's `--workload large` generates it) with the autotuned tiles, bit
    for bit against the FP32 oracle (about 30 s of host time on 16 cores)."""
    pr = P.Problem.generate(*LARGE, n_boxes=32, eps=(1, 10), box=(8, 64), steps=500, seed=2)
    f = P.zero_fields(*LARGE)
    with P.Solver(pr.params) as s:
        s.set_tiles(*P.tuned_tiles(*LARGE))
        s.set_fields(f)
        s.set_problem(pr)
        s.run(500)
        stages, mat = s.kernel()
        assert stages > 0 and mat, "the large workload runs the staged material-index kernel"
        got = s.get_fields()
    ref = oracle.step_ext_f32(f, 500, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    assert_parity(got, ref, "512x512x384 x 500")


def test_full_size_tiling_and_chunking_invariance(full_problem):
    pr = full_problem
    f = P.zero_fields(*FULL)
    with P.Solver(pr.params) as s:
        s.set_fields(f)
        s.set_problem(pr)
        s.run(1000)
        a = s.get_fields()
    with P.Solver(pr.params) as s:
        s.set_tiles(4, 16)
        s.set_fields(f)
        s.set_problem(pr)
        s.run(333)
        s.set_tiles(16, 0, 2)
        s.run(667)
        b = s.get_fields()
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    assert np.isfinite(a[5]).all() and np.abs(a[5]).max() > 0


def test_full_size_source_linearity(full_problem):
    """Doubling the source doubles every field.  Power-of-two scaling is exact for normal numbers;
    the subnormal tail ahead of the wavefront rounds differently, hence a tolerance (1e-6)."""
    pr = full_problem
    steps = 200
    f = P.zero_fields(*FULL)
    a = P.solve(pr, f, steps)
    pr2 = P.Problem(pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave * np.float32(2))
    b = P.solve(pr2, f, steps)
    for x, y in zip(a, b):
        assert oracle.normwise_error(y, x * np.float32(2)) <= 1e-6


# ------------------------------------------------------------------------------------------------
# The staged kernel (operands brought into shared memory by TMA tensor copies).
# ------------------------------------------------------------------------------------------------
STAGED = [(4, 2), (4, 3), (4, 4), (4, 5), (8, 2), (8, 3), (8, 4)]


@pytest.mark.parametrize("by,stages", STAGED)
@pytest.mark.parametrize("kc", [0, 1, 5])
def test_staged_kernel_bitwise(by, stages, kc):
    shape, steps = (261, 37, 23), 6      # x tiles 128+128+5: both halo ends clipped
    pr = P.Problem.generate(*shape, n_boxes=3, eps=(1, 10), box=(5, 30), steps=steps, seed=14)
    f = P.random_fields(*shape, seed=71, scale=1e-2)
    ref = oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    with P.Solver(pr.params) as s:
        s.set_tiles(by, kc, 4, stages)
        s.set_fields(f)
        s.set_problem(pr)
        s.run(steps)
        assert_parity(s.get_fields(), ref, f"staged by={by} stages={stages} kc={kc}")


@pytest.mark.parametrize("shape", [(5, 7, 3), (1, 1, 1), (2, 3, 2), (128, 9, 4), (129, 17, 6), (33, 64, 40)])
def test_staged_kernel_small_and_edge_shapes(shape):
    steps = 5
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=72)
    ref = oracle.step_ref_f32(f, steps, p)
    for by, stages, kc in ((8, 2, 3), (4, 5, 3), (23, 4, 3), (7, 4, 3), (11, 4, 0)):   # 7, 23 rows: 64 wide
        with P.Solver(p) as s:
            s.set_tiles(by, kc, 4, stages)
            s.set_fields(f)
            s.set_vacuum()
            s.run(steps)
            assert_parity(s.get_fields(), ref, f"staged {shape} by={by} stages={stages}")


# ------------------------------------------------------------------------------------------------
# Material index: one byte per node + a table instead of the four coefficient arrays.
# ------------------------------------------------------------------------------------------------
@pytest.mark.parametrize("by,stages", [(8, 4), (8, 6), (4, 3), (4, 5), (8, 2), (10, 4), (10, 5), (11, 4), (23, 3),
                                      (23, 4), (7, 3), (7, 4)])
def test_material_index_equals_per_cell_arrays(by, stages):
    shape, steps = (261, 37, 23), 7
    pr = P.Problem.generate(*shape, n_boxes=5, eps=(1, 10), box=(5, 30), steps=steps, seed=15)
    f = P.random_fields(*shape, seed=73, scale=1e-2)
    ref = oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    outs = []
    for use in (True, False):
        with P.Solver(pr.params) as s:
            s.set_tiles(by, 5, 4, stages)
            s.set_problem(pr)
            s.use_material_index(use)
            assert (s.material_count() > 0) == use and s.material_count() <= 6
            st, mat = s.kernel()
            dense = {4: (2, 3, 4, 5), 8: (2, 3, 4), 10: (3,), 11: (3,), 23: (), 7: ()}   # per-cell-array kernels
            fallback = stages if stages in dense[by] else (3 if 3 in dense[by] else 4)
            assert mat == use and st == (stages if use else fallback)
            s.set_fields(f)
            s.run(steps)
            outs.append(s.get_fields())
    assert_parity(outs[0], ref, f"material index by={by} stages={stages}")
    assert_parity(outs[1], ref, f"per-cell arrays by={by} stages={stages}")


def coefficient_set(shape, k, seed):
    """Coefficients with exactly k distinct (Ca, Cb, Da, Db) tuples, spread over the cells."""
    p = P.reference_params(*shape)
    n = shape[0] * shape[1] * shape[2]
    rng = np.random.default_rng(seed)
    ids = rng.permutation(np.arange(n) % k).reshape(shape[::-1])
    cb = (np.float32(p.Dt / p.eps0) * (1 + np.arange(k, dtype=np.float32) / np.float32(512)))[ids]
    one = np.ones(shape[::-1], np.float32)
    return p, one, cb.astype(np.float32), one.copy(), one * np.float32(p.Dt / p.mu0)


@pytest.mark.parametrize("k,expect", [(1, 1), (256, 256), (257, 0), (5000, 0)])
def test_material_count_limit_and_fallback(k, expect):
    shape, steps = (40, 30, 20), 5
    p, ca, cb, da, db = coefficient_set(shape, k, seed=k)
    f = P.random_fields(*shape, seed=74, scale=1e-2)
    with P.Solver(p) as s:
        s.set_tiles(8, 0, 4, 4)
        s.set_coefficients(ca, cb, da, db)
        assert s.material_count() == expect
        assert s.kernel() == (4, expect > 0)
        s.set_fields(f)
        s.run(steps)
        got = s.get_fields()
    assert_parity(got, oracle.step_ext_f32(f, steps, p, ca, cb, da, db), f"{k} materials")


def test_staged_full_size_matches_register_kernel(full_problem):
    pr = full_problem
    f = P.zero_fields(*FULL)
    outs = []
    for tiles in ((4, 8, 4, 0), (8, 32, 4, 3), (4, 0, 4, 4), (11, 86, 4, 4), (23, 86, 2, 4), (7, 86, 2, 4)):
        with P.Solver(pr.params) as s:
            s.set_tiles(*tiles)
            s.set_fields(f)
            s.set_problem(pr)
            s.run(300)
            outs.append(s.get_fields())
    for o in outs[1:]:
        for a, b in zip(outs[0], o):
            np.testing.assert_array_equal(a, b)


# ------------------------------------------------------------------------------------------------
# Bounded waits: a wait that cannot complete runs out, reports, and leaves the context usable.
# ------------------------------------------------------------------------------------------------
def test_bounded_wait_runs_out_and_context_stays_usable():
    word, ms = C.c_int(-1), C.c_float(-1)
    rc = _lib.lib().ptk_selftest_wait_expiry(C.byref(word), C.byref(ms))
    assert rc == 5, _lib.lib().ptk_last_error()          # PTK_ERR_TIMEOUT
    assert word.value == 1
    assert 0 < ms.value < 30000, ms.value                # the poll limit ends the wait within seconds
    assert b"bounded wait expired" in _lib.lib().ptk_last_error()
    # the same process still solves bit for bit
    shape, steps = (40, 33, 17), 6
    pr = P.Problem.generate(*shape, n_boxes=2, eps=(1, 6), box=(4, 12), steps=steps, seed=31)
    f = P.random_fields(*shape, seed=75, scale=1e-2)
    with P.Solver(pr.params) as s:
        s.set_tiles(11, 0, 4, 4)
        s.set_fields(f)
        s.set_problem(pr)
        s.run(steps)
        got = s.get_fields()
    assert_parity(got, oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave),
                  "solve after an expired wait")


def test_pinned_host_buffers_are_reused_by_size():
    lib = _lib.lib()
    a, b, c = C.c_void_p(), C.c_void_p(), C.c_void_p()
    n = 3 * 1024 * 1024 + 12   # a size nothing else in the process allocates
    assert lib.ptk_host_alloc(n, C.byref(a)) == 0
    C.memset(a, 7, n)
    assert lib.ptk_host_free(a) == 0
    assert lib.ptk_host_alloc(n, C.byref(b)) == 0
    assert b.value == a.value                       # the freed buffer came back
    assert lib.ptk_host_alloc(n, C.byref(c)) == 0   # a second one of the same size is a new buffer
    assert c.value != b.value
    for p in (b, c):
        assert lib.ptk_host_free(p) == 0


# ------------------------------------------------------------------------------------------------
# Randomised parity: seeded shapes x every staged tile shape x depths x material index on / off.
# ------------------------------------------------------------------------------------------------
STAGED_SHAPES = [(4, 3), (8, 4), (10, 4), (11, 4), (11, 3), (7, 4), (23, 4), (23, 3), (8, 6), (4, 5)]


@pytest.mark.parametrize("case", range(24))
def test_staged_kernel_random_shapes(case):
    rng = np.random.default_rng(9000 + case)
    shape = tuple(int(v) for v in rng.integers(1, 72, size=3))
    by, stages = STAGED_SHAPES[case % len(STAGED_SHAPES)]
    kc = int(rng.choice([0, 1, 2, 5, 17]))
    steps = int(rng.integers(2, 8))
    use_mat = bool(case % 3)
    n_boxes = int(rng.integers(1, 4)) if min(shape) >= 4 else 0
    pr = P.Problem.generate(*shape, n_boxes=n_boxes, eps=(1, 9), box=(2, max(2, min(shape) // 2)), steps=steps,
                            source_mode=1 if min(shape) >= 3 else 0, seed=700 + case)
    f = P.random_fields(*shape, seed=800 + case, scale=1e-2)
    ref = oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    with P.Solver(pr.params) as s:
        s.set_tiles(by, kc, 4, stages)
        s.set_problem(pr)
        s.use_material_index(use_mat)
        s.set_fields(f)
        s.run(steps)
        assert_parity(s.get_fields(), ref, f"{shape} by={by} stages={stages} kc={kc} mat={use_mat}")

"""The oracle is pinned before it is trusted: against the reference's own fdtd_cpu (golden fixtures
generated from oracle/_ref, and oracle/_ref itself where it was built), and internally (the
per-cell-coefficient form reduces bit-for-bit to the reference's scalar form in vacuum)."""
import hashlib

import numpy as np
import pytest

import oracle
import ptask_gb300 as P
from conftest import params_of


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def inputs_of(case):
    f = P.random_fields(case["Nx"], case["Ny"], case["Nz"], seed=case["seed"])
    assert [sha(a) for a in f] == case["input_sha256"], "seeded input generator drifted"
    return f


def test_oracle_matches_golden(golden):
    """oracle.step_ref_f32 reproduces the reference's outputs bit for bit on every golden case."""
    for case in golden["cases"]:
        if case["Nx"] * case["Ny"] * case["Nz"] * case["steps"] * max(1, case["blocks"]) > 4e6:
            continue
        f = inputs_of(case)
        out = oracle.step_ref_f32(f, case["steps"], params_of(case))
        assert [sha(a) for a in out] == case["output_sha256"], case["name"]


def test_oracle_matches_golden_arrays(golden_small):
    import json
    from conftest import ROOT
    cases = {c["name"]: c for c in json.loads((ROOT / "tests/golden/fdtd_golden.json").read_text())["cases"]}
    for key, ref in golden_small.items():
        name, field = key.split("/")
        c = cases[name]
        out = oracle.step_ref_f32(inputs_of(c), c["steps"], params_of(c))
        np.testing.assert_array_equal(out[P.FIELDS.index(field)], ref)


def test_multiple_inputs_is_repeat_of_single(golden):
    """fdtd_cpu_multiple_inputs (graphfdtd.cpp:344-391) returns the last of numBlocks identical solves."""
    c = next(c for c in golden["cases"] if c["blocks"] > 0)
    out = oracle.step_ref_f32(inputs_of(c), c["steps"], params_of(c))
    assert [sha(a) for a in out] == c["output_sha256"]


@pytest.mark.skipif(not oracle.have_ref(), reason="oracle/_ref not built (no reference tree)")
@pytest.mark.parametrize("shape,steps", [((5, 7, 3), 3), ((16, 9, 12), 6), ((1, 1, 1), 2), ((2, 3, 1), 4)])
def test_oracle_equals_reference_binary(shape, steps):
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=99)
    a = oracle.step_ref_f32(f, steps, p)
    b = oracle.ref_fdtd_cpu(f, steps, p)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("shape,steps", [((5, 7, 3), 4), ((12, 10, 8), 9), ((33, 17, 9), 5)])
def test_ext_reduces_to_reference_in_vacuum(shape, steps):
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=5)
    v = P.Problem.vacuum(p)
    a = oracle.step_ref_f32(f, steps, p)
    b = oracle.step_ext_f32(f, steps, p, v.Ca, v.Cb, v.Da, v.Db)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)


def test_generated_vacuum_cells_match_reference_coefficients():
    pr = P.Problem.generate(20, 18, 16, n_boxes=0, steps=10)
    ce = np.float32(np.float32(pr.params.Dt) / np.float32(pr.params.eps0))
    ch = np.float32(np.float32(pr.params.Dt) / np.float32(pr.params.mu0))
    assert np.all(pr.Cb == ce) and np.all(pr.Db == ch)
    assert np.all(pr.Ca == 1) and np.all(pr.Da == 1)


def test_f64_twin_close_to_f32():
    pr = P.Problem.generate(24, 20, 16, n_boxes=2, steps=60, seed=3)
    f = P.zero_fields(24, 20, 16)
    a = oracle.step_ext_f32(f, 60, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    b = oracle.step_ext_f64(f, 60, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    errs = [oracle.normwise_error(x, y) for x, y in zip(a, b)]
    assert max(errs) < 1e-3, errs
    assert np.max(np.abs(a[5])) > 0   # the source excited the field


def test_source_is_soft_and_linear():
    """Superposition: fields from (initial state A, source) = fields(A, no source) + fields(0, source)."""
    pr = P.Problem.generate(12, 12, 12, n_boxes=1, steps=20, seed=8)
    f = P.random_fields(12, 12, 12, seed=1, scale=1e-3)
    with_src = oracle.step_ext_f64(f, 20, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    no_src = oracle.step_ext_f64(f, 20, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db)
    only = oracle.step_ext_f64(P.zero_fields(12, 12, 12), 20, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db,
                               pr.src, pr.wave)
    for a, b, c in zip(with_src, no_src, only):
        np.testing.assert_allclose(a, b + c, rtol=1e-9, atol=1e-12 * max(1.0, float(np.abs(a).max())))


def test_pec_walls_stay_fixed():
    pr = P.Problem.generate(10, 9, 8, n_boxes=1, steps=15, seed=2)
    f = P.random_fields(10, 9, 8, seed=4)
    out = oracle.step_ext_f32(f, 15, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    Ex0, Ex1 = f[3], out[3]          # shape (Nz+1, Ny+1, Nx)
    np.testing.assert_array_equal(Ex1[:, 0, :], Ex0[:, 0, :])
    np.testing.assert_array_equal(Ex1[:, -1, :], Ex0[:, -1, :])
    np.testing.assert_array_equal(Ex1[0], Ex0[0])
    np.testing.assert_array_equal(Ex1[-1], Ex0[-1])
    Ez0, Ez1 = f[5], out[5]          # (Nz, Ny+1, Nx+1)
    np.testing.assert_array_equal(Ez1[:, :, 0], Ez0[:, :, 0])
    np.testing.assert_array_equal(Ez1[:, :, -1], Ez0[:, :, -1])


@pytest.mark.parametrize("shape,kw", [
    ((256, 256, 256), dict(n_boxes=8, eps=(1.0, 10.0), box=(8, 64), steps=1000, source_mode=1, seed=2)),
    ((512, 512, 384), dict(n_boxes=32, eps=(1.0, 10.0), box=(8, 64), steps=500, source_mode=1, seed=2)),
    ((37, 29, 23), dict(n_boxes=3, eps=(1.0, 10.0), box=(4, 11), steps=75, source_mode=2, seed=400002)),
    ((130, 24, 20), dict(n_boxes=4, eps=(1.0, 10.0), box=(8, 64), steps=20, source_mode=2, seed=5)),
    ((1, 1, 1), dict(n_boxes=2, eps=(2.0, 6.0), box=(4, 16), steps=3, source_mode=1, seed=1)),
    ((5, 1, 7), dict(n_boxes=0, steps=0, source_mode=0, seed=9)),
])
def test_oracle_problem_generator_is_the_products(shape, kw):
    """The oracle's own copy of the seeded problem generator (used by the CPU baseline, which loads
    nothing of the product) gives the same bits as ptk_problem_generate."""
    a = P.Problem.generate(*shape, **kw)
    b = oracle.problem_generate(*shape, **kw)
    for f, _ in oracle.Params._fields_:
        assert np.array(getattr(a.params, f)).tobytes() == np.array(getattr(b.params, f)).tobytes(), f
    assert a.src == b.src
    for x, y in zip((a.Ca, a.Cb, a.Da, a.Db, a.wave), (b.Ca, b.Cb, b.Da, b.Db, b.wave)):
        assert x.shape == y.shape and np.array_equal(x.view(np.uint32), y.view(np.uint32))
    for f, g in zip(P.zero_fields(*shape), oracle.zero_fields(*shape)):
        assert f.shape == g.shape and f.dtype == g.dtype and not g.any()

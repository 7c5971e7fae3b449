"""The FDTD task graph on the PTask-compatible runtime, against the oracle (bit for bit).

Covers the reference's unrolled graph (six per-field tasks per step, numBlocks instances pipelined,
graphfdtd.cpp:1008-1167) and the cyclic graph driven by an MF_GENERAL_ITERATOR meta port in its three
execution forms (fused lowering, captured CUDA-graph replay, task-by-task dispatch).
"""
import numpy as np
import pytest

import oracle
import ptask_gb300 as P
from ptask_gb300.graph import FDTDGraph

pytestmark = pytest.mark.gpu


def assert_same(got, ref, what):
    for q, (g, r) in enumerate(zip(got, ref)):
        assert oracle.normwise_error(g, r) <= 1e-5, (what, P.FIELDS[q])
        np.testing.assert_array_equal(g, r, err_msg=f"{what} {P.FIELDS[q]}")


@pytest.mark.parametrize("shape,steps", [((32, 32, 4), 4), ((9, 7, 5), 3), ((64, 64, 4), 4)])
def test_unrolled_reference_graph(shape, steps, tmp_path):
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=51)
    with FDTDGraph(p, "unrolled", unrolled_steps=steps) as g:
        got = g.solve(f, steps)
        st = g.stats()
        g.write_dot(tmp_path / "graphfdtd.dot")
    assert_same(got, oracle.step_ref_f32(f, steps, p), "unrolled")
    assert st["dispatches"] == 6 * steps and st["cycles_lowered"] == 0
    dot = (tmp_path / "graphfdtd.dot").read_text()
    assert dot.count("ComTask_") >= 6 * steps


@pytest.mark.parametrize("n", [4, 24])
def test_unrolled_pipelined_instances(n):
    """numBlocks instances pushed back to back (graphfdtd.cpp:1076-1097): every result equals one solve.
    With 24 instances the pushes outrun the graph's capacity-4 channels and block until it drains
    them (the pipelining stress of ptaskUnitTest/pipelinestresstest.cpp)."""
    shape, steps = (16, 12, 4), 4
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=52)
    with FDTDGraph(p, "unrolled", unrolled_steps=steps) as g:
        res = g.solve_many(f, n, steps)
        assert g.stats()["dispatches"] == 6 * steps * n
    ref = oracle.step_ref_f32(f, steps, p)
    for r in res:
        assert_same(r, ref, "pipelined")


def test_graphs_run_concurrently_from_two_threads():
    """Two graphs of different shapes, each driven from its own host thread at the same time (the
    runtime's concurrency stress, as in ptaskUnitTest/rttests.cpp): both results bit-exact."""
    import threading

    cases = [((40, 28, 20), 23, "fused", 91), ((33, 45, 18), 17, "taskwise", 92)]
    out, errs = {}, []

    def run(shape, steps, mode, seed):
        try:
            pr = P.Problem.generate(*shape, n_boxes=2, eps=(1, 9), box=(4, 12), steps=steps, seed=seed)
            f = P.random_fields(*shape, seed=seed + 100, scale=1e-3)
            with FDTDGraph(pr.params, mode) as g:
                g.set_problem(pr)
                res = [g.solve(f, steps) for _ in range(3)]
            out[seed] = (pr, f, steps, res)
        except Exception as e:   # reported below, on the test's thread
            errs.append(e)

    threads = [threading.Thread(target=run, args=c) for c in cases]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errs, errs
    for seed, (pr, f, steps, res) in out.items():
        ref = oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
        for got in res:
            assert_same(got, ref, f"concurrent graph {seed}")


@pytest.mark.parametrize("mode", ["fused", "captured", "taskwise"])
def test_cyclic_graph_forms(mode):
    shape, steps = (40, 28, 20), 37
    pr = P.Problem.generate(*shape, n_boxes=3, eps=(1, 10), box=(4, 16), steps=steps, seed=3)
    f = P.random_fields(*shape, seed=53, scale=1e-3)
    ref = oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    with FDTDGraph(pr.params, mode) as g:
        g.set_problem(pr)
        got = g.solve(f, steps)
        st = g.stats()
        # a second solve on the same graph instance (sticky inputs retained, blocks recycled)
        got2 = g.solve(f, steps)
    assert_same(got, ref, mode)
    assert_same(got2, ref, mode + " second solve")
    if mode == "taskwise":
        assert st["dispatches"] == 2 * steps and st["cycles_lowered"] == 0
    else:
        assert st["cycles_lowered"] == 1 and st["cycle_iterations"] == steps and st["dispatches"] == 0
        assert st["last_cycle_ms"] > 0


def test_cyclic_graph_vacuum_equals_reference():
    """The cyclic graph with the reference's scalar coefficients reproduces fdtd_cpu."""
    shape, steps = (24, 20, 12), 10
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=54)
    for mode in ("fused", "captured"):
        with FDTDGraph(p, mode) as g:
            g.set_problem(None)
            got = g.solve(f, steps)
        assert_same(got, oracle.step_ref_f32(f, steps, p), mode)


def test_cyclic_one_iteration_and_pipelining():
    shape = (16, 16, 16)
    pr = P.Problem.generate(*shape, n_boxes=1, steps=5, seed=4)
    f = P.random_fields(*shape, seed=55, scale=1e-3)
    with FDTDGraph(pr.params, "fused") as g:
        g.set_problem(pr)
        one = g.solve(f, 1)
        many = g.solve_many(f, 3, 5)
    assert_same(one, oracle.step_ext_f32(f, 1, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave), "1 step")
    ref5 = oracle.step_ext_f32(f, 5, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave)
    for r in many:
        assert_same(r, ref5, "pipelined cyclic")


# ------------------------------------------------------------------------------------------------
# Graph files: a saved graph, loaded into a new graph, computes the same results.
# ------------------------------------------------------------------------------------------------
def test_saved_unrolled_graph_loads_and_runs(tmp_path):
    shape, steps = (24, 20, 6), 3
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=61)
    path = tmp_path / "unrolled.xml"
    with FDTDGraph(p, "unrolled", unrolled_steps=steps) as g:
        g.save(path)
        first = g.solve(f, steps)
    with FDTDGraph.load(p, path) as g:
        again = g.solve(f, steps)
        assert g.stats()["dispatches"] == 6 * steps
    ref = oracle.step_ref_f32(f, steps, p)
    assert_same(first, ref, "original")
    assert_same(again, ref, "loaded")


@pytest.mark.parametrize("mode", ["fused", "taskwise"])
def test_saved_cyclic_graph_loads_in_any_lowering(tmp_path, mode):
    shape, steps = (33, 21, 17), 29
    pr = P.Problem.generate(*shape, n_boxes=3, eps=(1, 10), box=(4, 12), steps=steps, seed=8)
    f = P.random_fields(*shape, seed=62, scale=1e-3)
    path = tmp_path / "cyclic.xml"
    with FDTDGraph(pr.params, "captured") as g:
        g.save(path)
    with FDTDGraph.load(pr.params, path, mode) as g:
        g.set_problem(pr)
        got = g.solve(f, steps)
        st = g.stats()
    assert_same(got, oracle.step_ext_f32(f, steps, pr.params, pr.Ca, pr.Cb, pr.Da, pr.Db, pr.src, pr.wave),
                "loaded " + mode)
    assert (st["cycles_lowered"] == 1) == (mode == "fused")


def test_reference_layout_file_runs(tmp_path):
    """A file with only the reference's action kinds, its whitespace and foreign channel names."""
    from test_graph_xml import reference_style
    from ptask_gb300.graph import export_graph
    shape, steps = (16, 12, 5), 2
    p = P.reference_params(*shape)
    src, ref_file = tmp_path / "ours.xml", tmp_path / "ref.xml"
    export_graph(p, src, "unrolled", steps)
    ref_file.write_text(reference_style(src.read_text()))
    f = P.random_fields(*shape, seed=63)
    with FDTDGraph.load(p, ref_file) as g:
        got = g.solve(f, steps)
    assert_same(got, oracle.step_ref_f32(f, steps, p), "reference-layout file")


def test_load_rejects_a_file_for_another_grid(tmp_path):
    path = tmp_path / "g.xml"
    from ptask_gb300.graph import export_graph
    export_graph(P.reference_params(8, 8, 8), path, "fused")
    with pytest.raises(P.PtkError):
        FDTDGraph.load(P.reference_params(9, 8, 8), path)
    with pytest.raises(P.PtkError):
        FDTDGraph.load(P.reference_params(8, 8, 8), path, "unrolled")


# ------------------------------------------------------------------------------------------------
# Host tasks (hosttask.h:28-31): the same graph with its tasks on the host, on the GPU, or mixed.
# ------------------------------------------------------------------------------------------------
@pytest.fixture(scope="module")
def host_library(tmp_path_factory):
    """tests/hosttasks/fdtd_hosttasks.c built against the oracle into a shared library."""
    import subprocess
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    odir = root / "oracle" / "_build"
    out = tmp_path_factory.mktemp("hosttasks") / "libfdtd_hosttasks.so"
    subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-ffp-contract=off",
                    str(root / "tests" / "hosttasks" / "fdtd_hosttasks.c"), "-L", str(odir), "-loracle",
                    "-Wl,-rpath," + str(odir), "-o", str(out)], check=True)
    return out


@pytest.mark.parametrize("host_fields", [0x3F, 0x07, 0x38, 0x15])
def test_host_task_graph_matches_gpu_graph(host_library, host_fields):
    shape, steps = (20, 14, 6), 3
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=64)
    with FDTDGraph.with_host_tasks(p, steps, host_library, host_fields) as g:
        got = g.solve(f, steps)
        st = g.stats()
    n_host = bin(host_fields).count("1")
    assert st["host_dispatches"] == n_host * steps and st["dispatches"] == 6 * steps
    assert st["kernel_launches"] == (6 - n_host) * steps
    assert_same(got, oracle.step_ref_f32(f, steps, p), f"host fields {host_fields:#x}")


def test_host_tasks_by_reference_dll_name(host_library):
    """The reference names host libraries "x.dll": looked up as libx.so beside it."""
    shape, steps = (9, 7, 5), 2
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=65)
    dll = host_library.parent / "fdtd_hosttasks.dll"
    with FDTDGraph.with_host_tasks(p, steps, dll, 0x3F) as g:
        got = g.solve(f, steps)
    assert_same(got, oracle.step_ref_f32(f, steps, p), "dll name")


def test_host_task_graph_file_roundtrip(host_library, tmp_path):
    shape, steps = (12, 10, 4), 2
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=66)
    path = tmp_path / "host.xml"
    with FDTDGraph.with_host_tasks(p, steps, host_library, 0x07) as g:
        g.save(path)
    assert path.read_text().count("<AcceleratorClass>4</AcceleratorClass>") == 3 * steps   # HOST
    with FDTDGraph.load(p, path) as g:
        got = g.solve(f, steps)
        assert g.stats()["host_dispatches"] == 3 * steps
    assert_same(got, oracle.step_ref_f32(f, steps, p), "loaded host graph")


@pytest.fixture(scope="module", params=[True, False], ids=["with_streams", "without_streams"])
def dep_host_library(request, tmp_path_factory):
    """tests/hosttasks/fdtd_dephosttasks.c built against the product's C ABI, in the
    LPFNDEPHOSTTASKEX (with streams) or LPFNDEPHOSTTASK form."""
    import subprocess
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    bdir = root / "ptask_gb300" / "_build"
    out = tmp_path_factory.mktemp("dephosttasks") / "libfdtd_dephosttasks.so"
    subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-I", str(root / "include")] +
                   ([] if request.param else ["-DPTK_LEGACY_FORM"]) +
                   [str(root / "tests" / "hosttasks" / "fdtd_dephosttasks.c"), "-L", str(bdir), "-lptask_gb300",
                    "-Wl,-rpath," + str(bdir), "-o", str(out)], check=True)
    return out, request.param


@pytest.mark.parametrize("host_fields", [0x3F, 0x15])
def test_dependent_host_task_graph_matches_oracle(dep_host_library, host_fields):
    """Host tasks bound to the GPU as a dependent accelerator (hosttask.h:33-144) get device
    pointers for the ports bound to it and run the field updates through the C ABI; the graph's
    result is the oracle's, bit for bit, for every mix with native GPU tasks."""
    library, with_streams = dep_host_library
    shape, steps = (20, 14, 6), 3
    p = P.reference_params(*shape)
    f = P.random_fields(*shape, seed=67)
    with FDTDGraph.with_dependent_host_tasks(p, steps, library, host_fields, with_streams) as g:
        got = g.solve(f, steps)
        st = g.stats()
    n_host = bin(host_fields).count("1")
    assert st["host_dispatches"] == n_host * steps and st["dispatches"] == 6 * steps
    assert st["kernel_launches"] == (6 - n_host) * steps   # the host tasks' own launches are theirs
    assert_same(got, oracle.step_ref_f32(f, steps, p), f"dependent host fields {host_fields:#x}")


def test_missing_host_library_or_entry(tmp_path, host_library):
    p = P.reference_params(8, 8, 4)
    with pytest.raises(P.PtkError):
        FDTDGraph.with_host_tasks(p, 1, tmp_path / "absent.so", 0x3F)
    with pytest.raises(P.PtkError):
        FDTDGraph.with_host_tasks(p, 1, host_library.parent / "libm_absent.so", 0x01)

"""C-ABI checks that need no GPU: the library loads, exports every declared entry point, validates
arguments, and the host-side problem generator is deterministic."""
import ctypes as C
import re

import numpy as np
import pytest

import ptask_gb300 as P
from ptask_gb300 import _lib
from conftest import ROOT


# header -> shared library that must export its entry points
HEADERS = {"ptask_gb300.h": "libptask_gb300.so", "ptask_graph.h": "libptask_rt.so"}


def declared_symbols(header=None):
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        if header and h.name != header:
            continue
        text = h.read_text()
        names |= set(re.findall(r"\b(ptk_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_every_header_is_mapped_to_a_library():
    assert {h.name for h in (ROOT / "include").glob("*.h")} == set(HEADERS)


@pytest.mark.parametrize("header,libname", sorted(HEADERS.items()))
def test_library_exports_every_declared_symbol(header, libname):
    C.CDLL(str(_lib.LIB_PATH), mode=C.RTLD_GLOBAL)
    lib = C.CDLL(str(_lib.LIB_PATH.parent / libname))
    names = declared_symbols(header)
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert len(names) >= 7


def test_python_binding_covers_headers():
    from ptask_gb300 import graph
    bound = set(_lib.exported_symbols()) | set(graph._SIGS)
    assert set(declared_symbols()) <= bound, sorted(set(declared_symbols()) - bound)


def test_kernel_registry_resolves_reference_entries():
    lib = _lib.lib()
    kid = C.c_int()
    for q, name in enumerate(["HxComputation", "HyComputation", "HzComputation", "ExComputation",
                              "EyComputation", "EzComputation"]):
        assert lib.ptk_kernel_lookup(b"C:\\x\\fdtdMain.compute_10.ptx", name.encode(), C.byref(kid)) == 0
        assert kid.value == q
        ni, no, cb = C.c_int(), C.c_int(), C.c_int()
        assert lib.ptk_kernel_signature(kid, C.byref(ni), C.byref(no), C.byref(cb)) == 0
        assert (ni.value, no.value, cb.value) == (3, 1, 40)
    assert lib.ptk_kernel_lookup(b"x.ptx", b"NoSuchKernel", C.byref(kid)) == 7
    assert b"NoSuchKernel" in lib.ptk_last_error()
    assert lib.ptk_can_execute_kernel(b"quack.ptx") == 1
    assert lib.ptk_can_execute_kernel(b"quack.hlsl") == 0


def test_params_struct_layout_matches_fdtd_params():
    assert C.sizeof(_lib.FdtdParams) == 40


def test_reference_params_match_graphfdtd_constants():
    p = P.reference_params(64, 64, 4)
    assert p.Cx == np.float32(64 / np.float32(0.05)) and p.Cz == np.float32(4 / np.float32(0.03))
    assert p.eps0 == np.float32(8.8541878e-12)
    assert p.mu0 == np.float32(np.float32(4e-7) * np.float32(3.1415))
    assert 0 < p.Dt < 1e-12


def test_problem_generator_deterministic_and_seeded():
    a = P.Problem.generate(40, 30, 20, n_boxes=4, eps=(1, 10), box=(8, 16), steps=50, seed=7)
    b = P.Problem.generate(40, 30, 20, n_boxes=4, eps=(1, 10), box=(8, 16), steps=50, seed=7)
    c = P.Problem.generate(40, 30, 20, n_boxes=4, eps=(1, 10), box=(8, 16), steps=50, seed=8)
    np.testing.assert_array_equal(a.Cb, b.Cb)
    assert not np.array_equal(a.Cb, c.Cb)
    assert a.src == (20, 15, 10)
    assert a.wave.shape == (50,) and 0.99 < a.wave.max() <= 1.0
    eps = a.params.Dt / (a.params.eps0 * a.Cb.astype(np.float64))
    assert eps.min() > 0.99 and eps.max() < 10.01
    # Courant 0.5
    cfl = a.params.c0 * a.params.Dt * np.sqrt(a.params.Cx ** 2 + a.params.Cy ** 2 + a.params.Cz ** 2)
    assert abs(cfl - 0.5) < 1e-5


def test_seeded_source_positions_interior():
    for s in range(20):
        pr = P.Problem.generate(9, 5, 4, n_boxes=1, steps=5, source_mode=2, seed=s)
        i, j, k = pr.src
        assert 1 <= i <= 8 and 1 <= j <= 4 and 0 <= k <= 3


def test_invalid_arguments_are_reported_not_fatal():
    lib = _lib.lib()
    p = _lib.FdtdParams(0, 4, 4)
    h = C.c_void_p()
    rc = lib.ptk_solver_create(C.byref(p), C.byref(h))
    assert rc in (1, 2)           # INVALID (or CUDA when no device is present)
    assert lib.ptk_last_error()
    with pytest.raises(_lib.PtkError):
        _lib.call("ptk_fill_uniform", None, 10, C.c_float(1.0), C.c_uint64(1))

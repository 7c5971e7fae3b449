"""ctypes binding of the PTask FDTD graph C ABI (include/ptask_graph.h, libptask_rt.so)."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from ._lib import FdtdParams, PtkError, lib
from .fdtd import Problem, zero_fields

RT_PATH = Path(__file__).resolve().parent / "_build" / "libptask_rt.so"

CYCLIC_FUSED, CYCLIC_CAPTURED, CYCLIC_TASKWISE, UNROLLED = 0, 1, 2, 3
MODES = {"fused": CYCLIC_FUSED, "captured": CYCLIC_CAPTURED, "taskwise": CYCLIC_TASKWISE, "unrolled": UNROLLED}


class GraphStats(C.Structure):
    _fields_ = [("dispatches", C.c_ulonglong), ("kernel_launches", C.c_ulonglong),
                ("cycles_lowered", C.c_ulonglong), ("cycle_iterations", C.c_ulonglong),
                ("graph_replays", C.c_ulonglong), ("last_cycle_ms", C.c_float), ("last_solve_ms", C.c_float),
                ("host_dispatches", C.c_ulonglong)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


_rt = None
_P = C.c_void_p
_SIGS = {
    "ptk_fdtd_graph_create": [C.POINTER(FdtdParams), C.c_int, C.c_int, C.POINTER(_P)],
    "ptk_fdtd_graph_set_problem": [_P, _P, _P, _P, _P, C.c_int, C.c_int, C.c_int, _P, C.c_int],
    "ptk_fdtd_graph_solve": [_P, C.POINTER(_P), C.c_int],
    "ptk_fdtd_graph_solve_many": [_P, C.POINTER(_P), C.c_int, C.POINTER(_P), C.c_int],
    "ptk_fdtd_graph_stats": [_P, C.POINTER(GraphStats)],
    "ptk_fdtd_graph_write_dot": [_P, C.c_char_p],
    "ptk_fdtd_graph_destroy": [_P],
    "ptk_fdtd_graph_save": [_P, C.c_char_p],
    "ptk_fdtd_graph_create_host": [C.POINTER(FdtdParams), C.c_int, C.c_char_p, C.c_uint, C.POINTER(_P)],
    "ptk_fdtd_graph_create_dephost": [C.POINTER(FdtdParams), C.c_int, C.c_char_p, C.c_uint, C.c_int, C.POINTER(_P)],
    "ptk_fdtd_graph_load": [C.POINTER(FdtdParams), C.c_int, C.c_char_p, C.POINTER(_P)],
    "ptk_fdtd_graph_export": [C.POINTER(FdtdParams), C.c_int, C.c_int, C.c_char_p],
    "ptk_graph_xml_roundtrip": [C.c_char_p, C.c_char_p],
}


def rt() -> C.CDLL:
    global _rt
    if _rt is None:
        lib()   # the CUDA library first (libptask_rt.so links against it)
        if not RT_PATH.exists():
            raise ImportError(f"{RT_PATH} is missing: build with __graft_entry__.build()")
        L = C.CDLL(str(RT_PATH))
        for n, a in _SIGS.items():
            getattr(L, n).argtypes = a
            getattr(L, n).restype = C.c_int
        _rt = L
    return _rt


def _check(rc: int, where: str) -> None:
    if rc != 0:
        raise PtkError(rc, where, lib().ptk_last_error().decode(errors="replace"))


class FDTDGraph:
    """The FDTD task graph on the PTask runtime (see ptask_graph.h for the forms)."""

    def __init__(self, params: FdtdParams, mode: str = "fused", unrolled_steps: int = 0, *, _handle=None):
        self.params = params
        self.mode = mode
        self._h = C.c_void_p()
        if _handle is not None:
            self._h = _handle
            return
        _check(rt().ptk_fdtd_graph_create(C.byref(params), MODES[mode], unrolled_steps, C.byref(self._h)),
               "ptk_fdtd_graph_create")

    @classmethod
    def with_host_tasks(cls, params: FdtdParams, steps: int, library, host_fields: int = 0x3F) -> "FDTDGraph":
        """The unrolled graph whose tasks for the fields in `host_fields` (bit f = field f) are host
        tasks from the shared library `library` (entry points HxComputation .. EzComputation)."""
        h = C.c_void_p()
        _check(rt().ptk_fdtd_graph_create_host(C.byref(params), steps, str(library).encode(), host_fields,
                                               C.byref(h)), "ptk_fdtd_graph_create_host")
        return cls(params, "unrolled", _handle=h)

    @classmethod
    def with_dependent_host_tasks(cls, params: FdtdParams, steps: int, library, host_fields: int = 0x3F,
                                  with_streams: bool = True) -> "FDTDGraph":
        """The unrolled graph whose tasks for the fields in `host_fields` are host tasks that use the
        GPU as a dependent accelerator: their field arguments are device pointers.  `with_streams`
        selects the entry-point form: a DEPENDENTCONTEXT with the stream to order work on
        (LPFNDEPHOSTTASKEX), or the argument-list form without streams (LPFNDEPHOSTTASK)."""
        h = C.c_void_p()
        _check(rt().ptk_fdtd_graph_create_dephost(C.byref(params), steps, str(library).encode(), host_fields,
                                                  int(bool(with_streams)), C.byref(h)),
               "ptk_fdtd_graph_create_dephost")
        return cls(params, "unrolled", _handle=h)

    @classmethod
    def load(cls, params: FdtdParams, path, mode: str = "fused") -> "FDTDGraph":
        """A graph built from a graph file (Graph::Deserialize); `mode` is the lowering of a cyclic
        file and ignored for an unrolled one."""
        h = C.c_void_p()
        _check(rt().ptk_fdtd_graph_load(C.byref(params), MODES[mode], str(path).encode(), C.byref(h)),
               "ptk_fdtd_graph_load")
        return cls(params, mode, _handle=h)

    def save(self, path) -> None:
        """Write the graph's structure (Graph::Serialize)."""
        _check(rt().ptk_fdtd_graph_save(self._h, str(path).encode()), "ptk_fdtd_graph_save")

    def set_problem(self, prob: Problem | None) -> None:
        if prob is None:
            _check(rt().ptk_fdtd_graph_set_problem(self._h, None, None, None, None, -1, -1, -1, None, 0),
                   "set_problem")
            return
        self._coefs = [np.ascontiguousarray(a, np.float32) for a in (prob.Ca, prob.Cb, prob.Da, prob.Db)]
        self._wave = np.ascontiguousarray(prob.wave, np.float32)
        si, sj, sk = prob.src if prob.has_source else (-1, -1, -1)
        _check(rt().ptk_fdtd_graph_set_problem(self._h, *[a.ctypes.data for a in self._coefs], si, sj, sk,
                                               self._wave.ctypes.data if self._wave.size else None,
                                               int(self._wave.size)), "set_problem")

    def solve(self, fields, steps: int, out: list[np.ndarray] | None = None) -> list[np.ndarray]:
        """Push the six fields, run `steps` iterations, pull the results into `out` (six C-contiguous
        float32 arrays of the fields' shapes, reused across calls) or into new arrays.  The inputs
        are left as they are."""
        ins = [np.ascontiguousarray(f, np.float32) for f in fields]
        if out is None:
            out = [np.empty_like(a) for a in ins]
        elif len(out) != 6 or any(o.shape != a.shape or o.dtype != np.float32 or not o.flags.c_contiguous
                                  for o, a in zip(out, ins)):
            raise ValueError("out must be six C-contiguous float32 arrays shaped like the fields")
        _check(rt().ptk_fdtd_graph_solve_many(self._h, (C.c_void_p * 6)(*[a.ctypes.data for a in ins]), 1,
                                              (C.c_void_p * 6)(*[a.ctypes.data for a in out]), steps),
               "ptk_fdtd_graph_solve")
        return out

    def solve_many(self, fields, instances: int, steps: int) -> list[list[np.ndarray]]:
        ins = [np.ascontiguousarray(f, np.float32) for f in fields]
        nx, ny, nz = self.params.Nx, self.params.Ny, self.params.Nz
        res = [zero_fields(nx, ny, nz) for _ in range(instances)]
        rptrs = (C.c_void_p * (6 * instances))(*[a.ctypes.data for r in res for a in r])
        _check(rt().ptk_fdtd_graph_solve_many(self._h, (C.c_void_p * 6)(*[a.ctypes.data for a in ins]),
                                              instances, rptrs, steps), "solve_many")
        return res

    def stats(self) -> dict:
        s = GraphStats()
        _check(rt().ptk_fdtd_graph_stats(self._h, C.byref(s)), "stats")
        return s.as_dict()

    def write_dot(self, path: str) -> None:
        _check(rt().ptk_fdtd_graph_write_dot(self._h, str(path).encode()), "write_dot")

    def close(self) -> None:
        if self._h:
            rt().ptk_fdtd_graph_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def export_graph(params: FdtdParams, path, mode: str = "fused", unrolled_steps: int = 0) -> None:
    """Write the structure of the FDTD graph of `mode` without starting it (no device needed)."""
    _check(rt().ptk_fdtd_graph_export(C.byref(params), MODES[mode], unrolled_steps, str(path).encode()),
           "ptk_fdtd_graph_export")


def xml_roundtrip(in_path, out_path) -> None:
    """Read a graph file into a new graph and write it out again (no device needed)."""
    _check(rt().ptk_graph_xml_roundtrip(str(in_path).encode(), str(out_path).encode()), "ptk_graph_xml_roundtrip")

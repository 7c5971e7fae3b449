"""ctypes binding of libptask_gb300.so (the C ABI declared in include/ptask_gb300.h).

Loading fails loudly when the native library is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_BUILD = Path(__file__).resolve().parent / "_build"
LIB_PATH = _BUILD / "libptask_gb300.so"

PTK_OK = 0
PTK_HOST = 0
PTK_DEVICE = 1
ERRORS = {1: "INVALID", 2: "CUDA", 3: "NOMEM", 4: "STATE", 5: "TIMEOUT", 6: "BUDGET", 7: "NOTFOUND"}


class FdtdParams(C.Structure):
    """ptk_fdtd_params == FDTD_PARAMS (ptaskUnitTest/graphfdtd.h:6-19)."""
    _fields_ = [("Nx", C.c_int), ("Ny", C.c_int), ("Nz", C.c_int),
                ("Cx", C.c_float), ("Cy", C.c_float), ("Cz", C.c_float),
                ("eps0", C.c_float), ("mu0", C.c_float), ("c0", C.c_float), ("Dt", C.c_float)]

    def as_tuple(self):
        return tuple(getattr(self, f) for f, _ in self._fields_)


class TileConfig(C.Structure):
    _fields_ = [("by", C.c_int), ("kc", C.c_int), ("vec", C.c_int), ("stages", C.c_int)]


class ProblemDesc(C.Structure):
    _fields_ = [("Nx", C.c_int), ("Ny", C.c_int), ("Nz", C.c_int), ("n_boxes", C.c_int),
                ("eps_min", C.c_float), ("eps_max", C.c_float), ("box_min", C.c_int),
                ("box_max", C.c_int), ("courant", C.c_float), ("steps", C.c_int),
                ("source_mode", C.c_int), ("seed", C.c_uint64)]


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_size_t), ("max_active", C.c_int), ("chunk_steps", C.c_int),
                ("tile_rows", C.c_int), ("keep_results", C.c_int), ("persistent", C.c_int), ("stages", C.c_int)]


class RequestInfo(C.Structure):
    _fields_ = [("ticket", C.c_longlong), ("Nx", C.c_int), ("Ny", C.c_int), ("Nz", C.c_int), ("steps", C.c_int),
                ("arrival_s", C.c_double), ("admit_s", C.c_double), ("finish_s", C.c_double),
                ("checksum", C.c_double * 6), ("done", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong), ("wall_s", C.c_double),
                ("solves_per_s", C.c_double), ("p50_latency_s", C.c_double), ("p99_latency_s", C.c_double),
                ("mean_latency_s", C.c_double), ("cell_updates", C.c_double), ("mcells_per_s", C.c_double),
                ("chunks", C.c_longlong), ("kernel_launches", C.c_longlong), ("peak_active", C.c_int),
                ("peak_bytes", C.c_size_t), ("chunk_device_s", C.c_double), ("admit_s", C.c_double),
                ("retire_s", C.c_double), ("schedule_s", C.c_double), ("graph_captures", C.c_longlong),
                ("admit_waits", C.c_longlong)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class PtkError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: PTK_ERR_{ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None

_P = C.c_void_p
_FP = C.POINTER(C.c_float)
_SIGS = {
    "ptk_last_error": (C.c_char_p, []),
    "ptk_runtime_init": (C.c_int, [C.c_int]),
    "ptk_runtime_shutdown": (C.c_int, []),
    "ptk_device_info": (C.c_int, [C.c_char_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_size_t),
                                  C.POINTER(C.c_size_t)]),
    "ptk_can_execute_kernel": (C.c_int, [C.c_char_p]),
    "ptk_kernel_lookup": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_int)]),
    "ptk_kernel_signature": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ptk_mem_alloc": (C.c_int, [C.c_size_t, _P, C.POINTER(_P)]),
    "ptk_mem_free": (C.c_int, [_P, _P]),
    "ptk_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(_P)]),
    "ptk_host_free": (C.c_int, [_P]),
    "ptk_memcpy_h2d": (C.c_int, [_P, _P, C.c_size_t, _P]),
    "ptk_memcpy_d2h": (C.c_int, [_P, _P, C.c_size_t, _P]),
    "ptk_memcpy_d2d": (C.c_int, [_P, _P, C.c_size_t, _P]),
    "ptk_memset": (C.c_int, [_P, C.c_int, C.c_size_t, _P]),
    "ptk_stream_create": (C.c_int, [C.POINTER(_P)]),
    "ptk_stream_destroy": (C.c_int, [_P]),
    "ptk_stream_sync": (C.c_int, [_P]),
    "ptk_device_sync": (C.c_int, []),
    "ptk_device_ordinal": (C.c_int, [C.POINTER(C.c_int)]),
    "ptk_event_create": (C.c_int, [C.POINTER(_P)]),
    "ptk_event_destroy": (C.c_int, [_P]),
    "ptk_event_record": (C.c_int, [_P, _P]),
    "ptk_event_sync": (C.c_int, [_P]),
    "ptk_event_query": (C.c_int, [_P]),
    "ptk_stream_wait_event": (C.c_int, [_P, _P]),
    "ptk_event_elapsed_ms": (C.c_int, [_P, _P, C.POINTER(C.c_float)]),
    "ptk_pool_stats": (C.c_int, [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    "ptk_pool_trim_count": (C.c_longlong, []),
    "ptk_launch_count": (C.c_longlong, []),
    "ptk_launch_field_update": (C.c_int, [C.c_int, _P, _P, _P, C.POINTER(FdtdParams), _P, _P]),
    "ptk_launch_h_half_step": (C.c_int, [C.POINTER(_P), C.POINTER(_P), C.POINTER(FdtdParams), _P]),
    "ptk_launch_e_half_step": (C.c_int, [C.POINTER(_P), C.POINTER(_P), C.POINTER(_P),
                                         C.POINTER(FdtdParams), _P]),
    "ptk_launch_h_step_coef": (C.c_int, [C.POINTER(_P), C.POINTER(_P), _P, _P, C.POINTER(FdtdParams), _P]),
    "ptk_launch_e_step_coef": (C.c_int, [C.POINTER(_P), C.POINTER(_P), _P, _P, C.POINTER(FdtdParams), C.c_int,
                                         C.c_int, C.c_int, _P, C.c_int, _P, _P]),
    "ptk_capture_begin": (C.c_int, [_P]),
    "ptk_capture_end": (C.c_int, [_P, C.POINTER(_P)]),
    "ptk_graph_exec_launch": (C.c_int, [_P, _P, C.c_longlong]),
    "ptk_graph_exec_destroy": (C.c_int, [_P]),
    "ptk_solver_create": (C.c_int, [C.POINTER(FdtdParams), C.POINTER(_P)]),
    "ptk_solver_destroy": (C.c_int, [_P]),
    "ptk_solver_set_fields": (C.c_int, [_P, C.POINTER(_P), C.c_int, _P]),
    "ptk_solver_set_coefficients": (C.c_int, [_P, _P, _P, _P, _P, C.c_int, _P]),
    "ptk_solver_set_vacuum": (C.c_int, [_P, _P]),
    "ptk_solver_set_source": (C.c_int, [_P, C.c_int, C.c_int, C.c_int, _P, C.c_int, C.c_int, _P]),
    "ptk_solver_reset_clock": (C.c_int, [_P, _P]),
    "ptk_solver_set_tiles": (C.c_int, [_P, C.POINTER(TileConfig)]),
    "ptk_solver_get_tiles": (C.c_int, [_P, C.POINTER(TileConfig)]),
    "ptk_solver_use_material_index": (C.c_int, [_P, C.c_int, _P]),
    "ptk_solver_material_count": (C.c_int, [_P, C.POINTER(C.c_int)]),
    "ptk_solver_kernel": (C.c_int, [_P, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "ptk_solver_run": (C.c_int, [_P, C.c_int, _P]),
    "ptk_solver_get_fields": (C.c_int, [_P, C.POINTER(_P), C.c_int, _P]),
    "ptk_solver_bytes": (C.c_int, [_P, C.POINTER(C.c_size_t)]),
    "ptk_solver_last_launches": (C.c_int, [_P, C.POINTER(C.c_longlong)]),
    "ptk_fdtd_solve": (C.c_int, [C.POINTER(FdtdParams), C.POINTER(_P), _P, _P, _P, _P, C.c_int, C.c_int,
                                 C.c_int, _P, C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "ptk_fdtd_solve_static": (C.c_int, [C.POINTER(FdtdParams), C.POINTER(_P), _P, _P, _P, _P, C.c_int, C.c_int,
                                        C.c_int, _P, C.c_int, C.c_int, _P]),
    "ptk_fdtd_static_scratch_bytes": (C.c_size_t, []),
    "ptk_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(_P)]),
    "ptk_server_submit": (C.c_int, [_P, C.POINTER(ProblemDesc), C.c_double, C.POINTER(C.c_longlong)]),
    "ptk_server_run": (C.c_int, [_P, C.c_double]),
    "ptk_server_request": (C.c_int, [_P, C.c_longlong, C.POINTER(RequestInfo)]),
    "ptk_server_fetch": (C.c_int, [_P, C.c_longlong, C.POINTER(_P)]),
    "ptk_server_stats_get": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "ptk_server_destroy": (C.c_int, [_P]),
    "ptk_autotune_tiles":(C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(TileConfig), C.POINTER(C.c_float)]),
    "ptk_default_tiles": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(TileConfig)]),
    "ptk_selftest_wait_expiry": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_float)]),
    "ptk_problem_generate": (C.c_int, [C.POINTER(ProblemDesc), C.POINTER(FdtdParams), _P, _P, _P, _P,
                                       C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), _P]),
    "ptk_reference_params": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(FdtdParams)]),
    "ptk_fill_uniform": (C.c_int, [_P, C.c_size_t, C.c_float, C.c_uint64]),
}


def lib() -> C.CDLL:
    """The loaded native library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"native library {LIB_PATH} is missing: run "
                              "`python -c 'import __graft_entry__ as g; g.build()'` first "
                              "(ptask_gb300 has no CPU fallback)")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def check(rc: int, where: str) -> None:
    if rc != PTK_OK:
        raise PtkError(rc, where, lib().ptk_last_error().decode(errors="replace"))


def call(name: str, *args):
    rc = getattr(lib(), name)(*args)
    check(rc, name)
    return rc

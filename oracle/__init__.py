"""CPU oracle for the FDTD path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline / --impl reference) may import this
package; the product (ptask_gb300) never does.

  step_ref_f32   restatement of fdtd_cpu (ptaskUnitTest/graphfdtd.cpp:314-340), scalar vacuum
  step_ext_f32   per-cell coefficients + soft source (reduces bitwise to step_ref_f32 in vacuum)
  step_ext_f64   FP64 twin of step_ext_f32
  ref_fdtd_cpu   the reference's own fdtd_cpu compiled from its sources into oracle/_ref
                 (only where the reference tree was present at build time)
  problem_generate  the benchmark's seeded problem generator, restated here (bit-equal to
                 ptask_gb300's; pinned by tests) so that the CPU baseline loads nothing of the product
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_DIR = Path(__file__).resolve().parent
ORACLE_LIB = _DIR / "_build" / "liboracle.so"
REF_LIB = _DIR / "_ref" / "libref_fdtd.so"
REF_MAIN = _DIR / "_ref" / "ref_fdtd_main"


class Params(C.Structure):
    """Same layout as FDTD_PARAMS (graphfdtd.h:6-19)."""
    _fields_ = [("Nx", C.c_int), ("Ny", C.c_int), ("Nz", C.c_int),
                ("Cx", C.c_float), ("Cy", C.c_float), ("Cz", C.c_float),
                ("eps0", C.c_float), ("mu0", C.c_float), ("c0", C.c_float), ("Dt", C.c_float)]


class ProblemDesc(C.Structure):
    """Description of a seeded problem (same layout as ptk_problem_desc)."""
    _fields_ = [("Nx", C.c_int), ("Ny", C.c_int), ("Nz", C.c_int), ("n_boxes", C.c_int),
                ("eps_min", C.c_float), ("eps_max", C.c_float), ("box_min", C.c_int),
                ("box_max", C.c_int), ("courant", C.c_float), ("steps", C.c_int),
                ("source_mode", C.c_int), ("seed", C.c_uint64)]


def params_from(p) -> Params:
    """Copy any object with the FDTD_PARAMS attributes (e.g. ptask_gb300's FdtdParams)."""
    return Params(*(getattr(p, f) for f, _ in Params._fields_))


_o = None
_r = None


def _oracle():
    global _o
    if _o is None:
        if not ORACLE_LIB.exists():
            raise ImportError(f"{ORACLE_LIB} missing: build with ptask_gb300.build.build_oracle()")
        L = C.CDLL(str(ORACLE_LIB))
        V = C.c_void_p
        L.oracle_ref_f32.argtypes = [V] * 6 + [C.c_int, C.POINTER(Params)]
        L.oracle_ext_f32.argtypes = [V] * 10 + [C.c_int, C.POINTER(Params), C.c_int, C.c_int, C.c_int,
                                                V, C.c_int]
        L.oracle_ext_f64.argtypes = [C.POINTER(V), C.POINTER(V)] + [V] * 4 + [
            C.c_int, C.POINTER(Params), C.c_int, C.c_int, C.c_int, V, C.c_int]
        L.oracle_threads.restype = C.c_int
        L.oracle_problem_generate.argtypes = [C.POINTER(ProblemDesc), C.POINTER(Params)] + [V] * 4 + [
            C.POINTER(C.c_int)] * 3 + [V]
        _o = L
    return _o


def have_ref() -> bool:
    return REF_LIB.exists()


def _ref():
    global _r
    if _r is None:
        if not REF_LIB.exists():
            raise ImportError(f"{REF_LIB} missing (the reference tree was not available at build time)")
        L = C.CDLL(str(REF_LIB))
        V = C.c_void_p
        L.ref_fdtd_cpu.argtypes = [V] * 6 + [C.c_int, C.POINTER(Params)]
        L.ref_fdtd_cpu_multiple_inputs.argtypes = [V] * 6 + [C.c_int, C.c_int, C.POINTER(Params)]
        _r = L
    return _r


def _copies(fields):
    return [np.array(f, dtype=np.float32, copy=True, order="C") for f in fields]


def threads() -> int:
    return int(_oracle().oracle_threads())


def step_ref_f32(fields, steps: int, params) -> list[np.ndarray]:
    out = _copies(fields)
    rc = _oracle().oracle_ref_f32(*[a.ctypes.data for a in out], steps, C.byref(params_from(params)))
    assert rc == 0, rc
    return out


def step_ext_f32(fields, steps: int, params, Ca, Cb, Da, Db, src=(-1, -1, -1), wave=None):
    out = _copies(fields)
    coefs = [np.ascontiguousarray(c, np.float32) for c in (Ca, Cb, Da, Db)]
    w = np.ascontiguousarray(wave if wave is not None else np.zeros(0), np.float32)
    rc = _oracle().oracle_ext_f32(*[a.ctypes.data for a in out], *[c.ctypes.data for c in coefs], steps,
                                  C.byref(params_from(params)), src[0], src[1], src[2],
                                  w.ctypes.data if w.size else None, int(w.size))
    assert rc == 0, rc
    return out


def step_ext_f64(fields, steps: int, params, Ca, Cb, Da, Db, src=(-1, -1, -1), wave=None):
    ins = _copies(fields)
    outs = [np.empty(a.shape, np.float64) for a in ins]
    coefs = [np.ascontiguousarray(c, np.float32) for c in (Ca, Cb, Da, Db)]
    w = np.ascontiguousarray(wave if wave is not None else np.zeros(0), np.float32)
    V = C.c_void_p
    rc = _oracle().oracle_ext_f64((V * 6)(*[a.ctypes.data for a in ins]), (V * 6)(*[a.ctypes.data for a in outs]),
                                  *[c.ctypes.data for c in coefs], steps, C.byref(params_from(params)),
                                  src[0], src[1], src[2], w.ctypes.data if w.size else None, int(w.size))
    assert rc == 0, rc
    return outs


def ref_fdtd_cpu(fields, steps: int, params, blocks: int = 0) -> list[np.ndarray]:
    """The reference's own fdtd_cpu (blocks>0: fdtd_cpu_multiple_inputs with numBlocks=blocks)."""
    out = _copies(fields)
    P = C.byref(params_from(params))
    if blocks > 0:
        rc = _ref().ref_fdtd_cpu_multiple_inputs(*[a.ctypes.data for a in out], steps, blocks, P)
    else:
        rc = _ref().ref_fdtd_cpu(*[a.ctypes.data for a in out], steps, P)
    assert rc == 0, rc
    return out


FIELD_GROWS = ((1, 0, 0), (0, 1, 0), (0, 0, 1), (0, 1, 1), (1, 0, 1), (1, 1, 0))   # Hx..Ez: +1 on x, y, z


def zero_fields(nx: int, ny: int, nz: int) -> list[np.ndarray]:
    """Six zero fields in the reference's dense layout (C-ordered (d3, d2, d1), graphfdtd.cpp:68-86)."""
    return [np.zeros((nz + gz, ny + gy, nx + gx), np.float32) for gx, gy, gz in FIELD_GROWS]


class OracleProblem:
    """A generated problem: params (FDTD_PARAMS layout), per-cell coefficients, source, waveform."""

    def __init__(self, params, Ca, Cb, Da, Db, src, wave):
        self.params, self.Ca, self.Cb, self.Da, self.Db, self.src, self.wave = params, Ca, Cb, Da, Db, src, wave


def problem_generate(nx: int, ny: int, nz: int, *, n_boxes: int = 2, eps=(2.0, 6.0), box=(4, 16),
                     courant: float = 0.5, steps: int = 100, source_mode: int = 1, seed: int = 1) -> OracleProblem:
    """Same arguments and the same arrays as ptask_gb300.Problem.generate."""
    d = ProblemDesc(nx, ny, nz, n_boxes, eps[0], eps[1], box[0], box[1], courant, steps, source_mode, seed)
    p = Params()
    Ca, Cb, Da, Db = (np.empty((nz, ny, nx), np.float32) for _ in range(4))
    wave = np.zeros(max(steps, 1), np.float32)
    si, sj, sk = C.c_int(), C.c_int(), C.c_int()
    rc = _oracle().oracle_problem_generate(C.byref(d), C.byref(p), Ca.ctypes.data, Cb.ctypes.data, Da.ctypes.data,
                                           Db.ctypes.data, C.byref(si), C.byref(sj), C.byref(sk), wave.ctypes.data)
    assert rc == 0, rc
    return OracleProblem(p, Ca, Cb, Da, Db, (si.value, sj.value, sk.value), wave[:steps])


def normwise_error(got, ref) -> float:
    """max_i |g_i - r_i| / max_i |r_i| over one field (0 when both are zero)."""
    g = np.asarray(got, np.float64)
    r = np.asarray(ref, np.float64)
    den = float(np.max(np.abs(r))) if r.size else 0.0
    num = float(np.max(np.abs(g - r))) if r.size else 0.0
    if den == 0.0:
        return num
    return num / den

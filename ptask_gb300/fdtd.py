"""Python view of the FDTD path: problems, the device-resident solver, field helpers.

Fields are numpy float32 arrays in the reference's dense layout (ptaskUnitTest/Simple3DArray.h:33):
a field with extents (d1, d2, d3) is stored flat with index i + j*d1 + k*d1*d2, i.e. a C-ordered
array of shape (d3, d2, d1).  Field order is Hx, Hy, Hz, Ex, Ey, Ez throughout.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import PTK_DEVICE, PTK_HOST, FdtdParams, ProblemDesc, TileConfig, call, lib

FIELDS = ("Hx", "Hy", "Hz", "Ex", "Ey", "Ez")


def field_extents(f: int, nx: int, ny: int, nz: int) -> tuple[int, int, int]:
    """(d1, d2, d3) of field f, as the templates of graphfdtd.cpp:68-86."""
    return (nx + (1 if f in (0, 4, 5) else 0),
            ny + (1 if f in (1, 3, 5) else 0),
            nz + (1 if f in (2, 3, 4) else 0))


def field_shape(f: int, nx: int, ny: int, nz: int) -> tuple[int, int, int]:
    d1, d2, d3 = field_extents(f, nx, ny, nz)
    return (d3, d2, d1)


def zero_fields(nx: int, ny: int, nz: int) -> list[np.ndarray]:
    return [np.zeros(field_shape(f, nx, ny, nz), np.float32) for f in range(6)]


def random_fields(nx: int, ny: int, nz: int, seed: int, scale: float = 1e-4) -> list[np.ndarray]:
    """Seeded uniform [0, scale) fields (the reference draws rand()/(RAND_MAX*1e4), graphfdtd.cpp:117)."""
    out = []
    for f in range(6):
        a = np.empty(field_shape(f, nx, ny, nz), np.float32)
        call("ptk_fill_uniform", a.ctypes.data, a.size, C.c_float(scale), C.c_uint64(seed * 6 + f))
        out.append(a)
    return out


def reference_params(nx: int, ny: int, nz: int) -> FdtdParams:
    p = FdtdParams()
    call("ptk_reference_params", nx, ny, nz, C.byref(p))
    return p


@dataclass
class Problem:
    """A seeded FDTD problem: constants, per-cell coefficients, source position and waveform."""
    params: FdtdParams
    Ca: np.ndarray
    Cb: np.ndarray
    Da: np.ndarray
    Db: np.ndarray
    src: tuple[int, int, int]
    wave: np.ndarray

    @property
    def shape(self) -> tuple[int, int, int]:
        return (self.params.Nx, self.params.Ny, self.params.Nz)

    @property
    def has_source(self) -> bool:
        return self.src[0] >= 0

    @staticmethod
    def generate(nx: int, ny: int, nz: int, *, n_boxes: int = 2, eps: tuple[float, float] = (2.0, 6.0),
                 box: tuple[int, int] = (4, 16), courant: float = 0.5, steps: int = 100,
                 source_mode: int = 1, seed: int = 1) -> "Problem":
        d = ProblemDesc(nx, ny, nz, n_boxes, eps[0], eps[1], box[0], box[1], courant, steps,
                        source_mode, seed)
        p = FdtdParams()
        n = nx * ny * nz
        Ca, Cb, Da, Db = (np.empty((nz, ny, nx), np.float32) for _ in range(4))
        wave = np.zeros(max(steps, 1), np.float32)
        si, sj, sk = C.c_int(), C.c_int(), C.c_int()
        call("ptk_problem_generate", C.byref(d), C.byref(p), Ca.ctypes.data, Cb.ctypes.data,
             Da.ctypes.data, Db.ctypes.data, C.byref(si), C.byref(sj), C.byref(sk), wave.ctypes.data)
        assert Ca.size == n
        return Problem(p, Ca, Cb, Da, Db, (si.value, sj.value, sk.value), wave[:steps])

    @staticmethod
    def vacuum(params: FdtdParams) -> "Problem":
        """The reference's scalar-coefficient vacuum update expressed as per-cell arrays."""
        nx, ny, nz = params.Nx, params.Ny, params.Nz
        ce = np.float32(np.float32(params.Dt) / np.float32(params.eps0))
        ch = np.float32(np.float32(params.Dt) / np.float32(params.mu0))
        one = np.ones((nz, ny, nx), np.float32)
        return Problem(params, one.copy(), one * ce, one.copy(), one * ch, (-1, -1, -1),
                       np.zeros(0, np.float32))


def _ptr_array(arrs) -> "C.Array":
    return (C.c_void_p * len(arrs))(*[a if isinstance(a, int) else a.ctypes.data for a in arrs])


class Solver:
    """Device-resident FDTD instance (ptk_solver).  Mirrors one iterated FDTD graph instance."""

    def __init__(self, params: FdtdParams):
        lib()
        self.params = params
        self._h = C.c_void_p()
        call("ptk_solver_create", C.byref(params), C.byref(self._h))

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self) -> None:
        if self._h:
            call("ptk_solver_destroy", self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_fields(self, fields, stream=None) -> None:
        arrs = [np.ascontiguousarray(f, np.float32) for f in fields]
        self._keep = arrs
        call("ptk_solver_set_fields", self._h, _ptr_array(arrs), PTK_HOST, stream)
        call("ptk_stream_sync", stream)

    def set_fields_device(self, ptrs, stream=None) -> None:
        call("ptk_solver_set_fields", self._h, _ptr_array(ptrs), PTK_DEVICE, stream)

    def set_coefficients(self, Ca, Cb, Da, Db, stream=None) -> None:
        """Per-cell coefficient arrays (Nx*Ny*Nz floats each, reference layout)."""
        arrs = [np.ascontiguousarray(a, np.float32) for a in (Ca, Cb, Da, Db)]
        call("ptk_solver_set_coefficients", self._h, *[a.ctypes.data for a in arrs], PTK_HOST, stream)
        call("ptk_stream_sync", stream)

    def set_problem(self, prob: Problem, stream=None) -> None:
        arrs = [np.ascontiguousarray(a, np.float32) for a in (prob.Ca, prob.Cb, prob.Da, prob.Db)]
        call("ptk_solver_set_coefficients", self._h, *[a.ctypes.data for a in arrs], PTK_HOST, stream)
        if prob.has_source and prob.wave.size:
            w = np.ascontiguousarray(prob.wave, np.float32)
            call("ptk_solver_set_source", self._h, *prob.src, w.ctypes.data, w.size, PTK_HOST, stream)
        else:
            call("ptk_solver_set_source", self._h, 0, 0, 0, None, 0, PTK_HOST, stream)
        call("ptk_stream_sync", stream)

    def set_vacuum(self, stream=None) -> None:
        call("ptk_solver_set_vacuum", self._h, stream)

    def set_tiles(self, by: int, kc: int, vec: int = 0, stages: int = 0) -> None:
        """Fused-kernel tile shape: `by` rows, `kc` z-planes (0 = all), `vec` x cells per thread
        (1, 2, 4; 0 = chosen from Nx), `stages` > 0 selects the kernel whose operands are staged in
        shared memory by TMA tensor copies (that many planes in the ring, 2..6; 7 and 23 rows give
        64-wide tiles)."""
        call("ptk_solver_set_tiles", self._h, C.byref(TileConfig(by, kc, vec, stages)))

    def use_material_index(self, enable: bool = True, stream=None) -> None:
        """Read the coefficients through a one-byte material index (default) or the per-cell arrays."""
        call("ptk_solver_use_material_index", self._h, int(bool(enable)), stream)

    def material_count(self) -> int:
        n = C.c_int()
        call("ptk_solver_material_count", self._h, C.byref(n))
        return n.value

    def kernel(self) -> tuple[int, bool]:
        """(ring stages of the next run's step kernel, 0 = register kernel; reads the material index)"""
        st, m = C.c_int(), C.c_int()
        call("ptk_solver_kernel", self._h, C.byref(st), C.byref(m))
        return st.value, bool(m.value)

    def tiles(self) -> tuple[int, int, int, int]:
        t = TileConfig()
        call("ptk_solver_get_tiles", self._h, C.byref(t))
        return t.by, t.kc, t.vec, t.stages

    def reset_clock(self) -> None:
        call("ptk_solver_reset_clock", self._h, None)

    def run(self, steps: int, stream=None) -> None:
        call("ptk_solver_run", self._h, steps, stream)

    def last_launches(self) -> int:
        n = C.c_longlong()
        call("ptk_solver_last_launches", self._h, C.byref(n))
        return n.value

    def get_fields(self, stream=None) -> list[np.ndarray]:
        nx, ny, nz = self.params.Nx, self.params.Ny, self.params.Nz
        out = zero_fields(nx, ny, nz)
        call("ptk_solver_get_fields", self._h, _ptr_array(out), PTK_HOST, stream)
        return out

    def nbytes(self) -> int:
        n = C.c_size_t()
        call("ptk_solver_bytes", self._h, C.byref(n))
        return n.value


def solve(prob: Problem, fields, steps: int, tiles: tuple[int, int] | None = None) -> list[np.ndarray]:
    """Upload, run `steps` fused steps, download (synchronous)."""
    with Solver(prob.params) as s:
        if tiles:
            s.set_tiles(*tiles)
        s.set_fields(fields)
        s.set_problem(prob)
        s.run(steps)
        return s.get_fields()


def launch_count() -> int:
    return int(lib().ptk_launch_count())


def device_info() -> dict:
    name = C.create_string_buffer(256)
    sms = C.c_int()
    tot = C.c_size_t()
    free = C.c_size_t()
    call("ptk_device_info", name, 256, C.byref(sms), C.byref(tot), C.byref(free))
    return {"name": name.value.decode(), "sms": sms.value, "total": tot.value, "free": free.value}


__all__ = ["FIELDS", "Problem", "Solver", "solve", "field_extents", "field_shape", "zero_fields",
           "random_fields", "reference_params", "launch_count", "device_info", "PTK_HOST", "PTK_DEVICE"]


def tuned_tiles(nx: int, ny: int, nz: int) -> tuple[int, int, int, int]:
    """Fastest (rows, z depth, x cells per thread, staged planes) of the fused step kernel for this
    grid (autotuned on the device, cached per process)."""
    t = TileConfig()
    ms = C.c_float()
    call("ptk_autotune_tiles", nx, ny, nz, C.byref(t), C.byref(ms))
    return t.by, t.kc, t.vec, t.stages


def default_tiles(nx: int, ny: int, nz: int) -> tuple[int, int, int, int]:
    """Tile shape without timing: the autotuner's choice if this process tuned the grid, else the
    staged material-index kernel's default (11 rows, 4-plane ring, wave-filling depth)."""
    t = TileConfig()
    call("ptk_default_tiles", nx, ny, nz, C.byref(t))
    return t.by, t.kc, t.vec, t.stages

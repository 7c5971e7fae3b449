"""Device buffers, streams and events through the C ABI (no torch types on this path)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import call


class DeviceBuffer:
    """A block of HBM from the runtime's stream-ordered pool."""

    def __init__(self, nbytes: int, stream=None):
        self.nbytes = int(nbytes)
        self.ptr = C.c_void_p()
        call("ptk_mem_alloc", self.nbytes, stream, C.byref(self.ptr))

    @classmethod
    def from_array(cls, a: np.ndarray, stream=None) -> "DeviceBuffer":
        a = np.ascontiguousarray(a)
        b = cls(a.nbytes, stream)
        call("ptk_memcpy_h2d", b.ptr, a.ctypes.data, a.nbytes, stream)
        call("ptk_stream_sync", stream)
        return b

    def upload(self, a: np.ndarray, stream=None) -> None:
        a = np.ascontiguousarray(a)
        assert a.nbytes <= self.nbytes
        call("ptk_memcpy_h2d", self.ptr, a.ctypes.data, a.nbytes, stream)
        call("ptk_stream_sync", stream)

    def download(self, shape, dtype=np.float32, stream=None) -> np.ndarray:
        out = np.empty(shape, dtype)
        call("ptk_memcpy_d2h", out.ctypes.data, self.ptr, out.nbytes, stream)
        call("ptk_stream_sync", stream)
        return out

    @property
    def value(self) -> int:
        return int(self.ptr.value or 0)

    def free(self, stream=None) -> None:
        if self.ptr:
            call("ptk_mem_free", self.ptr, stream)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class HostBuffer:
    """Pinned host memory viewed as a numpy array."""

    def __init__(self, shape, dtype=np.float32):
        dtype = np.dtype(dtype)
        n = int(np.prod(shape)) * dtype.itemsize
        self.ptr = C.c_void_p()
        call("ptk_host_alloc", n, C.byref(self.ptr))
        buf = (C.c_char * max(n, 1)).from_address(self.ptr.value)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self) -> None:
        if self.ptr:
            self.array = None
            call("ptk_host_free", self.ptr)
            self.ptr = C.c_void_p()


class Stream:
    def __init__(self):
        self.handle = C.c_void_p()
        call("ptk_stream_create", C.byref(self.handle))

    def sync(self) -> None:
        call("ptk_stream_sync", self.handle)

    def close(self) -> None:
        if self.handle:
            call("ptk_stream_destroy", self.handle)
            self.handle = C.c_void_p()


class Event:
    def __init__(self):
        self.handle = C.c_void_p()
        call("ptk_event_create", C.byref(self.handle))

    def record(self, stream=None) -> None:
        call("ptk_event_record", self.handle, stream)

    def sync(self) -> None:
        call("ptk_event_sync", self.handle)

    def elapsed_ms(self, end: "Event") -> float:
        ms = C.c_float()
        call("ptk_event_elapsed_ms", self.handle, end.handle, C.byref(ms))
        return float(ms.value)

    def close(self) -> None:
        if self.handle:
            call("ptk_event_destroy", self.handle)
            self.handle = C.c_void_p()

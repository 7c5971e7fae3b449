"""ptask_gb300 -- GB300-native (sm_103a) runtime for the PTask FDTD task graph.

The compute path is libptask_gb300.so (hand-written CUDA kernels behind a C ABI, see
include/ptask_gb300.h); the PTask-compatible C++ runtime is libptask_rt.so (include/ptask/).
The native library is loaded on first use; every entry point raises ImportError if it has not been
built: there is no CPU fallback.
"""
from ._lib import LIB_PATH, PtkError, lib
from .fdtd import (FIELDS, Problem, Solver, device_info, field_extents, field_shape,
                   launch_count, random_fields, reference_params, solve, tuned_tiles, default_tiles, zero_fields)

__all__ = ["LIB_PATH", "PtkError", "lib", "FIELDS", "Problem", "Solver", "device_info",
           "field_extents", "field_shape", "launch_count", "random_fields", "reference_params",
           "solve", "tuned_tiles", "default_tiles", "zero_fields"]

"""Build recipe for the native parts of ptask_gb300 (no cmake, no setuptools).

Products (all in-tree, git-ignored):
  ptask_gb300/_build/libptask_gb300.so   CUDA kernels + C ABI (nvcc, sm_103a only)
  ptask_gb300/_build/libptask_rt.so      PTask-compatible C++ runtime (g++), links the above
  ptask_gb300/_build/bin/*               C++ programs of the runtime (graph drivers, tests)

Objects are rebuilt only when a source or header is newer; translation units compile in parallel.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "ptask_gb300"
CSRC = PKG / "csrc"
RTSRC = PKG / "runtime"
APPS = PKG / "apps"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"
# Root of the reference project's source tree (read only; only the oracle recipe and the drop-in
# compile test use it, and only where it exists).  One environment variable, shared with
# oracle/Makefile and tests/test_dropin.py.
REFERENCE = Path(os.environ.get("PTASK_REFERENCE", "/root/reference"))

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "--fmad=false", "-I", str(INCLUDE)]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
             "-I", str(INCLUDE)]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _newer(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _headers(*dirs: Path) -> list[Path]:
    out: list[Path] = []
    for d in dirs:
        if d.exists():
            out += list(d.rglob("*.h")) + list(d.rglob("*.cuh")) + list(d.rglob("*.hpp"))
    return out


def build_cuda_lib(verbose: bool = False) -> Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    BUILD.mkdir(parents=True, exist_ok=True)
    hdrs = _headers(CSRC, INCLUDE)
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.stem + (".cu.o" if src.suffix == ".cu" else ".cpp.o"))
        objs.append(obj)
        if _newer(obj, [src] + hdrs):
            if src.suffix == ".cu":
                cmd = [nvcc] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)]
            else:
                cmd = ["g++"] + CXX_FLAGS + ["-I", str(cuda / "include"), "-c", str(src), "-o", str(obj)]
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for f in [ex.submit(_run, c) for c in jobs]:
            f.result()
    lib = BUILD / "libptask_gb300.so"
    if jobs or _newer(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", str(lib)] + [str(o) for o in objs] +
             ["-lcudart", "-Xlinker", "-rpath,$ORIGIN"])
    if verbose:
        print(f"built {lib}")
    return lib


def build_runtime(verbose: bool = False) -> Path | None:
    """C++ PTask runtime (include/ptask/*.h) and its programs."""
    if not RTSRC.exists():
        return None
    BUILD.mkdir(parents=True, exist_ok=True)
    hdrs = _headers(RTSRC, INCLUDE)
    srcs = sorted(RTSRC.glob("*.cpp"))
    objs, jobs = [], []
    for src in srcs:
        obj = BUILD / ("rt_" + src.stem + ".o")
        objs.append(obj)
        if _newer(obj, [src] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-I", str(INCLUDE / "ptask"), "-pthread", "-fopenmp", "-c",
                         str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for f in [ex.submit(_run, c) for c in jobs]:
            f.result()
    lib = BUILD / "libptask_rt.so"
    core = BUILD / "libptask_gb300.so"
    if jobs or _newer(lib, objs + [core]):
        _run(["g++", "-shared", "-o", str(lib)] + [str(o) for o in objs] +
             ["-L", str(BUILD), "-lptask_gb300", "-pthread", "-fopenmp", "-ldl", "-Wl,-rpath,$ORIGIN"])
    bindir = BUILD / "bin"
    bindir.mkdir(exist_ok=True)
    jobs = []
    for app in sorted(APPS.glob("*.cpp")) if APPS.exists() else []:
        exe = bindir / app.stem
        if _newer(exe, [app, lib] + hdrs):
            jobs.append(["g++"] + CXX_FLAGS + ["-I", str(INCLUDE / "ptask"), "-pthread", str(app),
                         "-o", str(exe), "-L", str(BUILD), "-lptask_rt", "-lptask_gb300",
                         "-Wl,-rpath," + str(BUILD)])
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        for f in [ex.submit(_run, c) for c in jobs]:
            f.result()
    if verbose:
        print(f"built {lib}")
    return lib


def build_oracle(verbose: bool = False) -> None:
    """CPU checker: oracle/_build/liboracle.so; oracle/_ref from the reference when it is present."""
    odir = ROOT / "oracle"
    out = odir / "_build"
    out.mkdir(parents=True, exist_ok=True)
    lib = out / "liboracle.so"
    src = odir / "fdtd_oracle.c"
    if _newer(lib, [src]):
        _run(["gcc", "-O2", "-std=c11", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
              str(src), "-o", str(lib), "-lm"])
    if (REFERENCE / "ptaskUnitTest" / "graphfdtd.cpp").exists():
        _run(["make", "-s", "-C", str(odir), "ref", f"REF={REFERENCE / 'ptaskUnitTest'}"])
    if verbose:
        print(f"built {lib}")


def build_all(verbose: bool = False) -> None:
    build_cuda_lib(verbose)
    build_runtime(verbose)
    build_oracle(verbose)


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)

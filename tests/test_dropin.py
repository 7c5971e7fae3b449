"""The reference's own FDTD graph program builds unchanged against this runtime.

ptaskUnitTest/graphfdtd.cpp (the hot path's application code) is compiled from the reference tree,
without modification, against include/ptask (the ptaskapi.h surface) and linked with
libptask_rt.so + libptask_gb300.so.  g++ needs -fpermissive for the file's MSVC-isms (string literals
passed as char*).  The program is not run here (no GPU in this container, and the reference tree is
absent where the GPU tests run); tests/test_graph_gpu.py runs the same graph structure, built by
ptask_gb300/runtime/fdtd_graph.cpp through the same API calls, on the GPU.
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

REF = Path(os.environ.get("PTASK_REFERENCE", "/root/reference")) / "ptaskUnitTest"
BUILD = ROOT / "ptask_gb300" / "_build"


@pytest.mark.skipif(not (REF / "graphfdtd.cpp").exists(), reason="reference tree not present")
@pytest.mark.skipif(shutil.which("g++") is None, reason="no g++")
def test_reference_graphfdtd_compiles_and_links_unchanged(tmp_path):
    assert (BUILD / "libptask_rt.so").exists(), "build the runtime first"
    exe = tmp_path / "graphfdtd_ref"
    cmd = ["g++", "-std=c++17", "-fpermissive", "-w", "-O1",
           "-I", str(ROOT / "include" / "ptask"), "-I", str(ROOT / "include" / "ptask" / "win32"),
           "-I", str(ROOT / "include"), "-I", str(REF),
           str(REF / "graphfdtd.cpp"), str(ROOT / "tests" / "dropin" / "graphfdtd_harness.cpp"),
           "-o", str(exe), "-L", str(BUILD), "-lptask_rt", "-lptask_gb300", "-pthread",
           "-Wl,-rpath," + str(BUILD)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr[-4000:]
    assert exe.exists()

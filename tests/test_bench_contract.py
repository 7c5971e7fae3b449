"""The benchmark's output contract, checked on the CPU: `bench.py --impl reference` runs the CPU
implementation of the path (the oracle port of fdtd_cpu, graphfdtd.cpp:314-340) on the small
workload and prints one JSON line with the keys the contract names.  The reference arm loads the
oracle only (no part of the product library), and its `config` is the same object the GPU arm
prints for the workload.  The GPU arm's line is checked on a GB300 by running bench.py there."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

REQUIRED = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"}

# Runs bench.py's main() in-process, then reports which of the repository's modules and native
# libraries the process loaded.
PROBE = r"""
import json, runpy, sys
sys.argv = ["bench.py"] + sys.argv[1:]
try:
    runpy.run_path("bench.py", run_name="__main__")
except SystemExit as e:
    assert not e.code, e.code
maps = open("/proc/self/maps").read()
print("LOADED " + json.dumps({"ptask_gb300_module": any(m == "ptask_gb300" or m.startswith("ptask_gb300.")
                                                        for m in sys.modules),
                              "product_so": "libptask_gb300" in maps or "libptask_rt" in maps,
                              "oracle_so": "liboracle" in maps}))
"""


def run(*args):
    out = subprocess.run([sys.executable, "-c", PROBE, *args], capture_output=True, text=True, timeout=300,
                         cwd=str(ROOT))
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    loaded = json.loads([ln for ln in out.stdout.splitlines() if ln.startswith("LOADED ")][0][7:])
    return json.loads(lines[0]), loaded


def test_reference_arm_prints_one_contract_line():
    line, loaded = run("--impl", "reference", "--workload", "cpu32", "--steps", "2", "--warmup", "1")
    assert REQUIRED <= set(line), sorted(REQUIRED - set(line))
    assert line["impl"] == "reference" and line["metric"] == "FDTD Mcell-updates/s"
    assert line["unit"] == "Mcell-updates/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 2 and line["warmup"] == 1
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    assert f"{cb['cores']} host threads" in cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert line["config"]["grid"] == [32, 32, 32] and line["config"]["time_steps"] == 100
    # the reference arm runs the oracle and nothing of the product
    assert loaded == {"ptask_gb300_module": False, "product_so": False, "oracle_so": True}, loaded


def test_both_arms_print_the_same_config():
    sys.path.insert(0, str(ROOT))
    import bench
    line, _ = run("--impl", "reference", "--workload", "cpu32", "--steps", "1", "--warmup", "0")
    assert line["config"] == bench.workload_config(bench.WORKLOADS["cpu32"], 1)

"""The benchmark's output contract, checked on the CPU: `bench.py --impl reference` runs the CPU
implementation of the path (the oracle port of fdtd_cpu, graphfdtd.cpp:314-340) on the small
workload and prints one JSON line with the keys the contract names.  The GPU arm's line is checked
on a GB300 by the GPU suite's runs of bench.py."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

REQUIRED = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"}


def run(*args):
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True, text=True,
                         timeout=300, cwd=str(ROOT))
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    return json.loads(lines[0])


def test_reference_arm_prints_one_contract_line():
    line = run("--impl", "reference", "--workload", "cpu32", "--steps", "2", "--warmup", "1")
    assert REQUIRED <= set(line), sorted(REQUIRED - set(line))
    assert line["impl"] == "reference" and line["metric"] == "FDTD Mcell-updates/s"
    assert line["unit"] == "Mcell-updates/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["steps"] == 2 and line["warmup"] == 1
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert line["config"]["grid"] == [32, 32, 32] and line["config"]["time_steps"] == 100

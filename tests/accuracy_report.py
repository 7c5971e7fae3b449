"""Accuracy of every benchmark workload: GPU result against the FP32 oracle (bit for bit, and the
max normwise relative error the parity bar allows, 1e-5) and against the FP64 oracle.

For each workload the GPU path that the benchmark times is run on the same seeded problem as the
oracle: the solver with autotuned tiles for the plain and large grids, the continuous-batching
server for samples of the batched and served request sets.  The oracle (restatement of fdtd_cpu,
ptaskUnitTest/graphfdtd.cpp:314-340, with per-cell coefficients and the soft source) runs on all
host cores in FP32 and FP64.  Prints one JSON line per workload and a markdown table.

    python tests/accuracy_report.py [--only cpu32 plain256 large batched served] [--sample 8]

Needs a GPU and the built extension and oracle (__graft_entry__.build()).
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

import oracle  # noqa: E402
import ptask_gb300 as P  # noqa: E402


def group_error(got, ref) -> float:
    """Normwise error of the E fields and of the H fields as groups (max |g - r| over the group's
    three components over max |r| over the group), the larger of the two.  Unlike the per-field
    figure it stays meaningful when one component is zero up to rounding (by symmetry, or before
    the pulse reaches it), where any relative figure measures only rounding noise."""
    worst = 0.0
    for grp in ((0, 1, 2), (3, 4, 5)):
        num = max(float(np.max(np.abs(np.asarray(got[q], np.float64) - np.asarray(ref[q], np.float64))))
                  for q in grp)
        den = max(float(np.max(np.abs(np.asarray(ref[q], np.float64)))) for q in grp)
        worst = max(worst, num / den if den > 0 else (0.0 if num == 0 else float("inf")))
    return worst


def compare(name: str, got, prob, steps: int) -> dict:
    f = P.zero_fields(*prob.shape)
    t0 = time.perf_counter()
    r32 = oracle.step_ext_f32(f, steps, prob.params, prob.Ca, prob.Cb, prob.Da, prob.Db, prob.src, prob.wave)
    r64 = oracle.step_ext_f64(f, steps, prob.params, prob.Ca, prob.Cb, prob.Da, prob.Db, prob.src, prob.wave)
    dt = time.perf_counter() - t0
    return {
        "case": name,
        "bitexact_vs_fp32": all(np.array_equal(g, r) for g, r in zip(got, r32)),
        "err_vs_fp32": max(oracle.normwise_error(g, r) for g, r in zip(got, r32)),
        "err_vs_fp64": max(oracle.normwise_error(g, r) for g, r in zip(got, r64)),
        "fp32_oracle_vs_fp64": max(oracle.normwise_error(a, b) for a, b in zip(r32, r64)),
        "err_vs_fp64_eh": group_error(got, r64),
        "oracle_s": round(dt, 1),
    }


def plain(name: str, wl: dict) -> list[dict]:
    shape, steps = wl["shape"], wl["steps"]
    prob = P.Problem.generate(*shape, n_boxes=wl["boxes"], eps=wl["eps"], box=wl["box"], steps=steps,
                              source_mode=1, seed=2)
    with P.Solver(prob.params) as s:
        tiles = P.tuned_tiles(*shape)
        s.set_tiles(*tiles)
        s.set_fields(P.zero_fields(*shape))
        s.set_problem(prob)
        s.run(steps)
        got = s.get_fields()
    row = compare(f"{name} {shape[0]}x{shape[1]}x{shape[2]} x {steps}", got, prob, steps)
    row["gpu_path"] = f"solver, tiles {tiles}"
    return [row]


def served(name: str, reqs, sample: int) -> list[dict]:
    from ptask_gb300.serve import Server
    pick = [reqs[q] for q in np.linspace(0, len(reqs) - 1, min(sample, len(reqs))).astype(int)]
    rows = []
    with Server(keep_results=True) as s:
        tickets = [s.submit(r) for r in pick]
        s.run(time_scale=0)
        for t, r in zip(tickets, pick):
            prob = P.Problem.generate(r.nx, r.ny, r.nz, n_boxes=r.n_boxes, eps=r.eps, box=r.box, steps=r.steps,
                                      source_mode=r.source_mode, seed=r.seed)
            row = compare(f"{name} request {r.nx}x{r.ny}x{r.nz} x {r.steps}", s.fetch(t), prob, r.steps)
            row["gpu_path"] = f"server, {len(pick)} requests in one mix"
            rows.append(row)
    return rows


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--only", nargs="*", default=["cpu32", "plain256", "large", "batched", "served"])
    ap.add_argument("--sample", type=int, default=8, help="requests checked from the batched / served sets")
    args = ap.parse_args()
    import bench
    from ptask_gb300.serve import batched_instances, poisson_trace
    rows = []
    for name in args.only:
        n0 = len(rows)
        if name in bench.WORKLOADS:
            rows += plain(name, bench.WORKLOADS[name])
        elif name == "batched":
            rows += served(name, batched_instances(64, seed=4), args.sample)
        elif name == "served":
            rows += served(name, poisson_trace(1000, rate=200.0, seed=5), args.sample)
        for r in rows[n0:]:
            print(json.dumps(r), flush=True)
    print("\n| case | GPU path | bit-exact vs FP32 oracle | max normwise err vs FP32 | vs FP64, E/H groups | "
          "vs FP64, worst single field | FP32 oracle vs FP64 (worst field) |")
    print("|---|---|---|---|---|---|---|")
    for r in rows:
        print(f"| {r['case']} | {r['gpu_path']} | {'yes' if r['bitexact_vs_fp32'] else 'NO'} | "
              f"{r['err_vs_fp32']:.1e} | {r['err_vs_fp64_eh']:.2e} | {r['err_vs_fp64']:.2e} | "
              f"{r['fp32_oracle_vs_fp64']:.2e} |")
    bad = [r for r in rows if r["err_vs_fp32"] > 1e-5]
    return 1 if bad else 0


if __name__ == "__main__":
    raise SystemExit(main())

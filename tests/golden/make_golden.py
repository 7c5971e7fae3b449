"""Generate the golden FDTD fixtures from the reference's own CPU implementation.

Runs fdtd_cpu / fdtd_cpu_multiple_inputs of ptaskUnitTest/graphfdtd.cpp (314-391), compiled from the
reference tree into oracle/_ref by oracle/Makefile, on seeded inputs, and records:
  * the FDTD_PARAMS used (float32 values as hex strings, exact),
  * the seed and SHA-256 of every input field (inputs come from ptk_fill_uniform, seeded),
  * SHA-256 and float64 sum of every output field,
  * for the smallest cases, the full output arrays (golden_small.npz).
The reference has no golden vectors of its own (its check compares against fdtd_cpu on
time()-seeded data, graphfdtd.cpp:113,150-177); these fixtures pin the oracle where the reference
tree is absent.

Usage: python tests/golden/make_golden.py   (needs oracle/_ref, i.e. the reference tree at build time)
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
import ptask_gb300 as P  # noqa: E402

# (name, Nx, Ny, Nz, steps, numBlocks, seed); numBlocks > 0 uses fdtd_cpu_multiple_inputs.
CASES = [
    ("tiny_5x7x3_t3", 5, 7, 3, 3, 0, 11),
    ("odd_33x17x9_t5", 33, 17, 9, 5, 0, 12),
    ("regtest_64x64x4_i4_n4", 64, 64, 4, 4, 4, 13),   # mirrors ptaskUnitTest/regtest.sh:1114
    ("cube_32_t100", 32, 32, 32, 100, 0, 14),         # the 32^3 x 100-step size of the CPU config
    ("slab_130x9x6_t7", 130, 9, 6, 7, 0, 15),         # wider than one 128-cell tile in x
]
SMALL = {"tiny_5x7x3_t3", "odd_33x17x9_t5"}


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, np.float32).tobytes()).hexdigest()


def main() -> int:
    if not oracle.have_ref():
        print("oracle/_ref is not built (reference tree absent); cannot regenerate", file=sys.stderr)
        return 1
    out = {"generator": "tests/golden/make_golden.py", "source": "reference fdtd_cpu via oracle/_ref",
           "cases": []}
    small = {}
    for name, nx, ny, nz, steps, blocks, seed in CASES:
        p = P.reference_params(nx, ny, nz)
        fin = P.random_fields(nx, ny, nz, seed=seed)
        fout = oracle.ref_fdtd_cpu(fin, steps, p, blocks=blocks)
        out["cases"].append({
            "name": name, "Nx": nx, "Ny": ny, "Nz": nz, "steps": steps, "blocks": blocks, "seed": seed,
            "params": {f: (getattr(p, f) if f in ("Nx", "Ny", "Nz") else float(getattr(p, f)).hex())
                       for f, _ in p._fields_},
            "input_sha256": [sha(a) for a in fin],
            "output_sha256": [sha(a) for a in fout],
            "output_sum": [float(np.sum(a, dtype=np.float64)) for a in fout],
        })
        if name in SMALL:
            for q, a in enumerate(fout):
                small[f"{name}/{P.FIELDS[q]}"] = a
    (ROOT / "tests" / "golden" / "fdtd_golden.json").write_text(json.dumps(out, indent=1) + "\n")
    np.savez_compressed(ROOT / "tests" / "golden" / "golden_small.npz", **small)
    print(f"wrote {len(out['cases'])} cases")
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Screen synthetic tasks for the depth-4 fixtures (needs a GPU): scans the
batched workload's generator in a seeded order, keeps tasks with 17-32
tests and no program within kernel depth 3, and records the engine's
optimal depth within kernel depth 4 for each, so that
make_depth4_fixtures.py runs the oracle only on tasks whose outcome mix it
wants (one- and two-input tasks with an optimum of 4, and some without a
program within 4). The fixture values themselves come from the oracle; this
list only chooses tasks.

    python tests/golden/screen_depth4_candidates.py [OUT]   (default: depth4_candidates.json here)
"""
import json
import os
import random
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from pca_gb300 import taskgen  # noqa: E402
from pca_gb300.pcalib import Engine  # noqa: E402


def scan(n: int, seed: int = 2024):
    rng = random.Random(seed)
    out = []
    while len(out) < n:
        s, length = rng.randrange(1 << 40), rng.randrange(4, 9)
        spec, _ = taskgen.synthetic_task(s, length)
        if spec.num_tests >= 17:
            out.append((s, length, spec))
    return out


def main():
    cands = scan(3000)
    eng = Engine(0, 0)
    r3 = eng.solve_batch([c[2] for c in cands], max_depth=3, first_only=True, sol_cap=1)
    hard = [c for c, r in zip(cands, r3) if r.optimal_depth < 0]
    rows = []
    for i in range(0, len(hard), 64):
        part = hard[i:i + 64]
        r4 = eng.solve_batch([c[2] for c in part], max_depth=4, first_only=True, sol_cap=1)
        for (s, length, spec), r in zip(part, r4):
            rows.append({"seed": s, "length": length, "inputs": spec.num_inputs,
                         "tests": spec.num_tests, "gpu_optimal_depth": r.optimal_depth})
    eng.close()
    out = sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "depth4_candidates.json")
    json.dump(rows, open(out, "w"), indent=0)
    print(len(cands), "scanned,", len(hard), "without a program within depth 3:",
          sum(r["gpu_optimal_depth"] == 4 for r in rows), "with optimum 4")


if __name__ == "__main__":
    main()

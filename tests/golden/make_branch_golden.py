"""Record the reference solver's branch mode (CMP/BR, DIV/MOD; its default,
without --no-branch) as a fixture.

Runs the reference's own `enumerate <task> -d D` (compiled from the
reference sources by oracle/build_ref.sh into oracle/_ref/) on the fixture
tasks of ref_enumerate.json with D up to their branchless optimal depth (at
most 3), keeps the runs that finish within a time limit, and stores the
per-depth "candidates" / cumulative "OEP pruned" counters, the optimal
length and the printed programs in ref_enumerate_branch.json (task embedded).

    python tests/golden/make_branch_golden.py
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ENUM = os.path.join(ROOT, "oracle", "_ref", "enumerate")


def parse(out: str) -> dict:
    cands = [int(x) for x in re.findall(r"  candidates: (\d+) ", out)]
    pruned = [int(x) for x in re.findall(r"  OEP pruned: (\d+)\n", out)]
    sols = []
    for blk in re.findall(r"Solution #\d+ \(\d+ instructions\):\n((?:    [0-9A-F]{2}: .*\n)+)", out):
        sols.append([int(w, 16) for w in re.findall(r"    [0-9A-F]{2}: ([0-9A-F]{4})", blk)])
    m = re.search(r"Optimal solution length: (\d+) instructions \(kernel depth (\d+)\)", out)
    f = re.search(r"Found (\d+) distinct program", out)
    return {"candidates": cands, "pruned_cum": pruned, "programs": sols,
            "optimal_length": int(m.group(1)) if m else None,
            "optimal_depth": int(m.group(2)) if m else None,
            "found": int(f.group(1)) if f else 0}


def main(limit_s: float = 60.0):
    if not os.path.exists(ENUM):
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    ref = json.load(open(os.path.join(HERE, "ref_enumerate.json")))
    out = []
    for i, fx in enumerate(ref):
        k = fx["optimal_depth"] if fx["optimal_depth"] is not None else fx["max_depth"]
        depth = min(k, 3)
        with tempfile.TemporaryDirectory() as d:
            tp = os.path.join(d, "task.json")
            json.dump(fx["task"], open(tp, "w"))
            try:
                p = subprocess.run([ENUM, tp, "-d", str(depth)], capture_output=True, text=True,
                                   timeout=limit_s)
            except subprocess.TimeoutExpired:
                continue
        r = parse(p.stdout)
        r.update(index=i, max_depth=depth, exit=p.returncode, task=fx["task"])
        out.append(r)
    json.dump(out, open(os.path.join(HERE, "ref_enumerate_branch.json"), "w"))
    print(len(out), "of", len(ref), "tasks;",
          [(r["index"], r["optimal_depth"], len(r["programs"])) for r in out])


if __name__ == "__main__":
    sys.exit(main())

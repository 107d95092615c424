"""Run the CPU oracle (pinned to the reference by tests/test_oracle_golden.py)
in its exact modes on the golden tasks and record what the GPU tests compare
against, so the GPU suite does not spend minutes in single-threaded C:

  exact       key regs+flags, DFS first-wins: per-depth tried / cumulative
              pruned, per-level children and survivors at the final depth
  exact_live  key regs+flags+live: per-level children and survivors
  full        no pruning, uncapped: the canonical program set (tasks whose
              full set is cheap to enumerate on one core)

    python tests/golden/make_oracle_fixtures.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "tests"))

from conftest import spec_from_json  # noqa: E402
from oracle import oracle as O  # noqa: E402


def counters(r, upto):
    return {"optimal_depth": r.optimal_depth,
            "tried": [r.tried[k] for k in range(upto + 1)],
            "pruned_cum": [r.pruned_cum[k] for k in range(upto + 1)],
            "children": [r.children[k] for k in range(upto + 1)],
            "survivors": [r.survivors[k] for k in range(upto + 1)],
            "total_solutions": r.total_solutions}


def main():
    fx = json.load(open(os.path.join(HERE, "ref_enumerate.json")))
    out = []
    for i, f in enumerate(fx):
        spec = spec_from_json(f["task"])
        D = f["max_depth"]
        r, progs = O.enumerate_task(spec, D, O.EXACT, 1 << 16)
        last = r.optimal_depth if r.optimal_depth >= 0 else D
        e = {"index": i, "exact": counters(r, last), "exact_programs": progs[:200]}
        r2, _ = O.enumerate_task(spec, D, O.EXACT_LIVE, 0)
        e["exact_live"] = counters(r2, last)
        K = f["optimal_depth"]
        if K is not None and (K <= 2 or (K == 3 and spec.num_inputs == 1)):
            r3, full = O.enumerate_task(spec, D, O.NONE, 1 << 16)
            e["full"] = {"total": r3.total_solutions, "programs": full}
        out.append(e)
        print(i, f["source"], e["exact"]["optimal_depth"], e["exact"]["survivors"], flush=True)
    json.dump(out, open(os.path.join(HERE, "oracle_modes.json"), "w"))


if __name__ == "__main__":
    main()

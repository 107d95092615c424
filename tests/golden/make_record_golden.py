"""Record the reference's `enumerate --record` output as a fixture.

Runs the reference's own solver (compiled from the reference sources by
oracle/build_ref.sh into oracle/_ref/) with --record on fixture tasks where
its 32-bit pruner is exact (its per-depth counters equal the exact pruner's
in tests/golden/oracle_modes.json, so the states its recording pass visits
are the exact levels), and stores per run the SHA-256 and size of
states_<id>.bin and edges_<id>.bin, the first records verbatim (hex), and
the report's counts, in ref_record.json next to this script.

    python tests/golden/make_record_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ENUM = os.path.join(ROOT, "oracle", "_ref", "enumerate")


def main():
    if not os.path.exists(ENUM):
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    ref = json.load(open(os.path.join(HERE, "ref_enumerate.json")))
    modes = {m["index"]: m for m in json.load(open(os.path.join(HERE, "oracle_modes.json")))}
    picks = []
    for i, fx in enumerate(ref):
        K = fx["optimal_depth"]
        ex = modes[i]["exact"]
        if K is None or K > 2 or ex["optimal_depth"] != K:
            continue
        if fx["candidates"][:K + 1] != ex["tried"][:K + 1] or \
                fx["pruned_cum"][:K + 1] != ex["pruned_cum"][:K + 1]:
            continue
        picks.append(i)
    runs = []
    for n, i in enumerate(picks[:14]):
        fx = ref[i]
        for stride in ((8, 1) if n < 3 else (8,)):
            with tempfile.TemporaryDirectory() as d:
                tp = os.path.join(d, "task.json")
                json.dump(fx["task"], open(tp, "w"))
                out = os.path.join(d, "rec")
                os.makedirs(out)
                tid = 100 + i
                p = subprocess.run([ENUM, tp, "-d", str(fx["optimal_depth"]), "--record", out,
                                    "--task-id", str(tid), "--neg-stride", str(stride)],
                                   capture_output=True, text=True)
                st = open(os.path.join(out, f"states_{tid:06d}.bin"), "rb").read()
                ed = open(os.path.join(out, f"edges_{tid:06d}.bin"), "rb").read()
                m = re.search(r"states: (\d+) written \((\d+) positive, (\d+) negative\)", p.stdout)
                e = re.search(r"edges: (\d+) written", p.stdout)
                o = re.search(r"optimal state set: (\d+) states", p.stdout)
                runs.append(dict(index=i, task_id=tid, neg_stride=stride, exit=p.returncode,
                                 depth=fx["optimal_depth"],
                                 states_sha256=hashlib.sha256(st).hexdigest(), states_bytes=len(st),
                                 edges_sha256=hashlib.sha256(ed).hexdigest(), edges_bytes=len(ed),
                                 first_states_hex=st[:2 * 576].hex(), first_edges_hex=ed[:4 * 24].hex(),
                                 written=int(m.group(1)), positives=int(m.group(2)),
                                 negatives=int(m.group(3)), edges=int(e.group(1)),
                                 optimal_states=int(o.group(1))))
    json.dump(runs, open(os.path.join(HERE, "ref_record.json"), "w"), indent=1)
    print(len(runs), "runs on tasks", picks[:14])


if __name__ == "__main__":
    sys.exit(main())

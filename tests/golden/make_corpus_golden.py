"""Record the reference task generator's output as a fixture.

Runs the reference's `gen_tasks` (compiled from the reference sources by
oracle/build_ref.sh into oracle/_ref/) with a few argument sets and stores
every file it writes, verbatim, in ref_gen_tasks.json next to this script:
{"<args>": {"<file name>": "<file text>", ...}, ...}.

    python tests/golden/make_corpus_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
GEN = os.path.join(ROOT, "oracle", "_ref", "gen_tasks")

CONFIGS = [
    ["-n", "30", "-s", "42"],
    ["-n", "30", "-s", "7", "--min-len", "3", "--max-len", "8"],
    ["-n", "12", "-s", "3", "--verify"],
    ["-n", "12", "-s", "5", "--min-len", "8", "--max-len", "10"],
]


def main():
    if not os.path.exists(GEN):
        subprocess.run([os.path.join(ROOT, "oracle", "build_ref.sh")], check=True)
    out = {}
    for args in CONFIGS:
        with tempfile.TemporaryDirectory() as d:
            subprocess.run([GEN, d] + args, check=True, capture_output=True)
            out[" ".join(args)] = {f: open(os.path.join(d, f)).read() for f in sorted(os.listdir(d))}
    with open(os.path.join(HERE, "ref_gen_tasks.json"), "w") as f:
        json.dump(out, f, indent=0, sort_keys=True)
    print({k: len(v) for k, v in out.items()})


if __name__ == "__main__":
    sys.exit(main())

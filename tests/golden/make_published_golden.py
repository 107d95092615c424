"""Record the reference's task files with its published optimal program
lengths as a fixture (ref_published.json next to this script).

The lengths are the reference's own documented results of its solver in
branch mode (README.md:41-51 and the comments of Makefile:66-77): negate,
double, square 4; add 5; abs, relu 6; max 7; saturating_add 8; is_power2 7.
The task specs are read from the reference's tasks/*.json.

    python tests/golden/make_published_golden.py REFERENCE_ROOT   (or PCA_REFERENCE_ROOT set)
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PUBLISHED = {"negate": 4, "double": 4, "square": 4, "add": 5, "abs": 6, "relu": 6, "max": 7,
             "saturating_add": 8, "is_power2": 7}


def main(ref=None):
    ref = ref or os.environ.get("PCA_REFERENCE_ROOT", "")
    if not ref:
        sys.exit("usage: make_published_golden.py REFERENCE_ROOT (or set PCA_REFERENCE_ROOT)")
    out = []
    for name, length in PUBLISHED.items():
        task = json.load(open(os.path.join(ref, "tasks", name + ".json")))
        out.append({"name": name, "published_length": length, "task": task})
    json.dump(out, open(os.path.join(HERE, "ref_published.json"), "w"), indent=1)
    print(len(out), "tasks")


if __name__ == "__main__":
    sys.exit(main(*sys.argv[1:]))

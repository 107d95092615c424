"""Generate the golden fixtures from the reference itself.

Runs the reference's own CPU solver and libpca.so, compiled from the
reference sources by oracle/build_ref.sh into oracle/_ref/, and records
their outputs as JSON next to this script:

  ref_enumerate.json  `enumerate <task> -d D --no-branch` per task: the
                      per-depth "candidates" and cumulative "OEP pruned"
                      counters, the optimal length and the printed programs.
  ref_libpca.json     search_state_step / oep_hash64 / key_hash64 /
                      leaf_outputs / gen_candidates_branchless on random walks,
                      task_evaluate and pca_disasm, and
                      search_exhaustive_complete on manifest tasks (the cases
                      of python/test_exhaustive.py).

Task specs are embedded in the fixtures, so tests need no reference tree.

    python tests/golden/make_golden.py REFERENCE_ROOT   (or PCA_REFERENCE_ROOT set)
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import random
import re
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from pca_gb300.pcalib import SearchCtx, SearchState, TaskSpec  # noqa: E402
from pca_gb300 import taskgen  # noqa: E402

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PCA_REFERENCE_ROOT", "")
if not REF:
    sys.exit("usage: make_golden.py REFERENCE_ROOT (or set PCA_REFERENCE_ROOT)")
REF_BIN = os.path.join(REPO, "oracle", "_ref", "enumerate")
REF_LIB = os.path.join(REPO, "oracle", "_ref", "libpca.so")


def task_to_json(spec: TaskSpec) -> dict:
    n_in = spec.num_inputs
    return {
        "name": spec.name.decode(),
        "max_cycles": spec.max_cycles,
        "input_ports": [spec.input_ports[i] for i in range(n_in)],
        "output_ports": [spec.output_ports[0]],
        "tests": [{"in": [spec.tests[t].inputs[i] for i in range(n_in)],
                   "out": [spec.tests[t].outputs[0]]} for t in range(spec.num_tests)],
    }


def run_reference(path: str, depth: int) -> dict:
    out = subprocess.run([REF_BIN, path, "-d", str(depth), "--no-branch"], capture_output=True,
                         text=True, timeout=3600).stdout
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


def load_ref_lib():
    L = ctypes.CDLL(REF_LIB)
    P = ctypes.POINTER
    L.task_load.argtypes = [ctypes.c_char_p, P(TaskSpec)]
    L.search_ctx_init.argtypes = [P(SearchCtx), P(TaskSpec)]
    L.search_state_init_root.argtypes = [P(SearchCtx), P(SearchState)]
    L.search_state_step.argtypes = [P(SearchCtx), P(SearchState), ctypes.c_uint16, P(SearchState)]
    L.search_state_oep_hash64.argtypes = [P(SearchCtx), P(SearchState)]
    L.search_state_oep_hash64.restype = ctypes.c_uint64
    L.search_state_key_hash64.argtypes = [P(SearchCtx), P(SearchState)]
    L.search_state_key_hash64.restype = ctypes.c_uint64
    L.search_state_leaf_outputs.argtypes = [P(SearchCtx), P(SearchState)]
    L.search_state_leaf_outputs.restype = ctypes.c_uint8
    L.search_gen_candidates_branchless.argtypes = [P(ctypes.c_uint16), ctypes.c_int, P(SearchState)]
    L.search_exhaustive_complete.argtypes = [P(SearchCtx), P(SearchState), ctypes.c_int,
                                             P(ctypes.c_uint16), P(ctypes.c_int)]
    L.search_exhaustive_states_explored.restype = ctypes.c_uint64
    L.task_evaluate.argtypes = [P(TaskSpec), P(ctypes.c_uint16), ctypes.c_int]
    L.pca_disasm.argtypes = [ctypes.c_uint16, ctypes.c_char_p, ctypes.c_size_t]
    return L


def state_digest(s: SearchState) -> str:
    return hashlib.sha256(bytes(s)).hexdigest()[:32]


def main():
    os.makedirs(HERE, exist_ok=True)
    tasks = []  # (spec_path, depth)
    for name in ("negate", "double", "square", "add"):
        tasks.append((os.path.join(REF, "tasks", name + ".json"), 4))
    for name in ("abs", "relu", "sign", "clamp"):
        tasks.append((os.path.join(REF, "tasks", name + ".json"), 3))
    manifest = json.load(open(os.path.join(REF, "data", "manifest.json")))
    want = {(1, 1): 8, (1, 2): 10, (1, 3): 8, (2, 1): 8, (2, 2): 10, (2, 3): 2}
    got = {k: 0 for k in want}
    for t in manifest["tasks"]:
        if not t["path"].startswith("data/synthetic/"):
            continue
        k = (t["num_inputs"], t.get("optimal_depth"))
        if k in want and got[k] < want[k]:
            got[k] += 1
            tasks.append((os.path.join(REF, t["path"]), 3))
    tmp = tempfile.mkdtemp()
    neg = os.path.join(tmp, "negate16.json")
    json.dump(task_to_json(taskgen.negate_task(1)), open(neg, "w"))
    tasks.append((neg, 4))

    L = load_ref_lib()
    enum_fix = []
    for path, depth in tasks:
        spec = TaskSpec()
        assert L.task_load(path.encode(), ctypes.byref(spec)) == 0
        res = run_reference(path, depth)
        res["task"] = task_to_json(spec)
        res["max_depth"] = depth
        res["source"] = os.path.relpath(path, REF) if path.startswith(REF) else "generated:negate(seed=1)"
        enum_fix.append(res)
        print(res["source"], res["optimal_depth"], len(res["programs"]), res["candidates"], flush=True)
    json.dump(enum_fix, open(os.path.join(HERE, "ref_enumerate.json"), "w"))

    # libpca vectors: random walks (incl. DIV/MOD and non-branchless words)
    rng = random.Random(1234)
    walks = []
    for fx in enum_fix[8:20]:
        path = os.path.join(tmp, "w.json")
        json.dump(fx["task"], open(path, "w"))
        spec = TaskSpec()
        L.task_load(path.encode(), ctypes.byref(spec))
        ctx = SearchCtx()
        L.search_ctx_init(ctypes.byref(ctx), ctypes.byref(spec))
        for _ in range(6):
            s = SearchState()
            L.search_state_init_root(ctypes.byref(ctx), ctypes.byref(s))
            steps = []
            for _d in range(4):
                buf = (ctypes.c_uint16 * 4096)()
                n = L.search_gen_candidates_branchless(buf, 4096, ctypes.byref(s))
                cands = [buf[i] for i in range(n)]
                r = rng.random()
                if r < 0.15:
                    insn = (rng.choice([5, 6]) << 11) | (rng.randrange(1, 8) << 8) | \
                           (rng.randrange(8) << 5) | (rng.randrange(8) << 2)
                elif r < 0.2:
                    insn = rng.randrange(1 << 16)
                else:
                    insn = rng.choice(cands)
                d = SearchState()
                ok = L.search_state_step(ctypes.byref(ctx), ctypes.byref(s), insn, ctypes.byref(d))
                entry = {"insn": insn, "ok": ok,
                         "ncands": n, "cands_sha": hashlib.sha256(bytes(buf)[:2 * n]).hexdigest()[:32]}
                if ok:
                    entry.update({"state_sha": state_digest(d),
                                  "oep": str(L.search_state_oep_hash64(ctypes.byref(ctx), ctypes.byref(d))),
                                  "key": str(L.search_state_key_hash64(ctypes.byref(ctx), ctypes.byref(d))),
                                  "leaf": L.search_state_leaf_outputs(ctypes.byref(ctx), ctypes.byref(d))})
                    s = d
                steps.append(entry)
                if not ok:
                    break
            walks.append({"task": fx["task"], "steps": steps})

    # exhaustive completion (python/test_exhaustive.py:47-110)
    comp = []
    by_depth = {}
    for t in manifest["tasks"]:
        d = t.get("optimal_depth")
        if t.get("solved") and d in (1, 2, 3):
            by_depth.setdefault(d, []).append(t)
    for d in sorted(by_depth):
        for t in by_depth[d][:3]:
            spec = TaskSpec()
            L.task_load(os.path.join(REF, t["path"]).encode(), ctypes.byref(spec))
            ctx = SearchCtx()
            L.search_ctx_init(ctypes.byref(ctx), ctypes.byref(spec))
            root = SearchState()
            L.search_state_init_root(ctypes.byref(ctx), ctypes.byref(root))
            entry = {"task": task_to_json(spec), "manifest_depth": d, "runs": []}
            for start_insns, max_depth in (([], d), ([], d - 1)):
                insns = (ctypes.c_uint16 * 16)()
                n = ctypes.c_int(0)
                f = L.search_exhaustive_complete(ctypes.byref(ctx), ctypes.byref(root), max_depth,
                                                 insns, ctypes.byref(n))
                entry["runs"].append({"start": start_insns, "max_depth": max_depth, "found": f,
                                      "len": n.value, "insns": [insns[i] for i in range(n.value)],
                                      "explored": L.search_exhaustive_states_explored()})
            first = entry["runs"][0]
            if first["found"] and first["len"] >= 1 and d >= 2:
                mid = SearchState()
                L.search_state_step(ctypes.byref(ctx), ctypes.byref(root), first["insns"][0], ctypes.byref(mid))
                insns = (ctypes.c_uint16 * 16)()
                n = ctypes.c_int(0)
                f = L.search_exhaustive_complete(ctypes.byref(ctx), ctypes.byref(mid), d, insns, ctypes.byref(n))
                entry["runs"].append({"start": [first["insns"][0]], "max_depth": d, "found": f,
                                      "len": n.value, "insns": [insns[i] for i in range(n.value)],
                                      "explored": L.search_exhaustive_states_explored()})
            comp.append(entry)
    dis = {}
    for w in [rng.randrange(1 << 16) for _ in range(300)] + list(range(0, 1 << 16, 2048)):
        b = ctypes.create_string_buffer(64)
        L.pca_disasm(w, b, 64)
        dis[str(w)] = b.value.decode()
    json.dump({"walks": walks, "complete": comp, "disasm": dis},
              open(os.path.join(HERE, "ref_libpca.json"), "w"))
    print("walks", len(walks), "complete", len(comp))


if __name__ == "__main__":
    main()

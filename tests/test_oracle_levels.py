"""The oracle's level-synchronous form (oracle/oracle_levels.c) against its
depth-first form (oracle/pca_oracle.c), which tests/test_oracle_golden.py
pins to the reference's own outputs, on every golden task:

  * the optimal depth, and the kept states and generated children of every
    level below it, in both exact modes;
  * the first program of every final state among its solutions (depth-first
    order) is the depth-first oracle's program list with the last position
    pruned too: the same programs in the same order;
  * with nothing pruned, the full canonical program set.

The depth-4 fixtures (tests/golden/oracle_depth4.json) come from this form.
Their tasks are checked here at kernel depth 3 (no program, the same
levels 1..2 and counters), and against the depth-first oracle at depth 2."""
import ctypes

import pytest

from conftest import load_golden, spec_from_json
from oracle import oracle as O
from pca_gb300.pcalib import SearchCtx, SearchState

ENUM = load_golden("ref_enumerate.json")
MODES = {m["index"]: m for m in load_golden("oracle_modes.json")}


def final_key(spec, prog):
    L = O.lib()
    ctx = SearchCtx()
    L.orc_ctx_init(ctypes.byref(ctx), ctypes.byref(spec))
    s = SearchState()
    L.orc_init_root(ctypes.byref(ctx), ctypes.byref(s))
    for insn in prog[spec.num_inputs:-2]:
        c = SearchState()
        L.orc_step(ctypes.byref(ctx), ctypes.byref(s), insn, ctypes.byref(c))
        s = c
    return bytes(memoryview(s))[:32 * 16 + 32]


@pytest.mark.parametrize("i", range(len(ENUM)), ids=[f["source"] for f in ENUM])
def test_levels_equal_depth_first_oracle(i):
    fx = ENUM[i]
    spec = spec_from_json(fx["task"])
    D = fx["max_depth"]
    om = MODES[i]["exact"]
    r, progs = O.enumerate_split(spec, D, 16, O.EXACT, threads=4)
    K = r.optimal_depth
    assert K == om["optimal_depth"]
    S = K - 1 if K > 0 else (0 if K == 0 else D - 1)
    assert [r.survivors[d] for d in range(S + 1)] == om["survivors"][:S + 1]
    assert [r.children[d] for d in range(S + 1)] == om["children"][:S + 1]
    if K > 0:
        seen, firsts = set(), []
        for p in progs:
            k = final_key(spec, p)
            if k not in seen:
                seen.add(k)
                firsts.append(p)
        want = MODES[i]["exact_programs"]
        assert firsts[:len(want)] == want
        if len(want) < 200:  # the fixture keeps the first 200
            assert len(firsts) == len(want)
    lv = MODES[i]["exact_live"]
    r2, _ = O.enumerate_split(spec, D, 16, O.EXACT_LIVE, threads=4, sol_cap=1)
    assert r2.optimal_depth == lv["optimal_depth"]
    assert [r2.survivors[d] for d in range(S + 1)] == lv["survivors"][:S + 1]
    if "full" in MODES[i]:
        r0, p0 = O.enumerate_split(spec, D, 0, O.NONE, threads=4)
        assert r0.total_solutions == MODES[i]["full"]["total"]
        assert p0 == MODES[i]["full"]["programs"][:len(p0)]


DEPTH4 = load_golden("oracle_depth4.json")
D4 = [("is_power2", DEPTH4["is_power2"])] + [(f"syn{t['seed']}", t) for t in DEPTH4["tasks"]]


@pytest.mark.parametrize("case", D4, ids=[c[0] for c in D4])
def test_depth4_fixture_tasks_at_depth3(case):
    name, fx = case
    spec = spec_from_json(fx["task"])
    want = fx["exact_live"]
    r, _ = O.enumerate_split(spec, 3, 16, O.EXACT_LIVE, threads=4, sol_cap=1)
    assert r.optimal_depth == -1
    assert [r.survivors[d] for d in range(3)] == want["survivors"][:3]
    assert [r.tried[k] for k in range(4)] == want["tried"][:4]
    d, _ = O.enumerate_task(spec, 2, O.EXACT_LIVE, 0)
    assert d.optimal_depth == -1
    assert [d.survivors[k] for k in range(3)] == want["survivors"][:3]

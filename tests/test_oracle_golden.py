"""The CPU oracle is pinned to the reference: on every golden task it
reproduces `enumerate --no-branch` (per-depth candidates, cumulative OEP
pruned, optimal length, printed programs) and search_exhaustive_complete."""
import pytest

from conftest import load_golden, spec_from_json
from oracle import oracle as O

ENUM = load_golden("ref_enumerate.json")
LIBPCA = load_golden("ref_libpca.json")


@pytest.mark.parametrize("fx", ENUM, ids=[f["source"] for f in ENUM])
def test_oracle_matches_reference_enumerate(fx):
    spec = spec_from_json(fx["task"])
    r, progs = O.enumerate_task(spec, fx["max_depth"], O.REF32)
    last = r.optimal_depth if r.optimal_depth >= 0 else fx["max_depth"]
    assert [r.tried[k] for k in range(last + 1)] == fx["candidates"]
    assert [r.pruned_cum[k] for k in range(last + 1)] == fx["pruned_cum"]
    assert r.optimal_depth == (fx["optimal_depth"] if fx["optimal_depth"] is not None else -1)
    assert progs == fx["programs"]


@pytest.mark.parametrize("case", LIBPCA["complete"], ids=lambda c: c["task"]["name"])
def test_oracle_matches_reference_complete(case):
    from pca_gb300.pcalib import SearchCtx, SearchState
    L = O.lib()
    spec = spec_from_json(case["task"])
    import ctypes
    ctx = SearchCtx()
    L.orc_ctx_init(ctypes.byref(ctx), ctypes.byref(spec))
    for run in case["runs"]:
        s = SearchState()
        L.orc_init_root(ctypes.byref(ctx), ctypes.byref(s))
        for insn in run["start"]:
            d = SearchState()
            assert L.orc_step(ctypes.byref(ctx), ctypes.byref(s), insn, ctypes.byref(d)) == 1
            s = d
        found, n, insns, explored = O.exhaustive_complete(ctx, s, run["max_depth"])
        assert (int(found), n, insns, explored) == (run["found"], run["len"], run["insns"], run["explored"])


SHALLOW = [i for i, f in enumerate(ENUM) if len(f["candidates"]) <= 3]


@pytest.mark.parametrize("i", SHALLOW, ids=[ENUM[i]["source"] for i in SHALLOW])
def test_exact_pruner_agrees_with_reference_where_collision_free(i):
    """The reference keys its pruner on 32 bits of the hash in a 2^20-slot
    table per depth and keeps a child when 32 probes find no slot
    (tools/enumerate.c:54-77). An exact shadow set audits every decision:
    where the reference neither collided (false prune) nor saturated (missed
    prune), the exact pruner (key regs+flags, DFS first-wins) reproduces the
    reference's counters and programs exactly; otherwise the difference in the
    pruned count is exactly the audited false/missed prunes of the last
    level. The GPU engine is compared with the exact pruner everywhere."""
    modes = {m["index"]: m for m in load_golden("oracle_modes.json")}
    fx, ex = ENUM[i], modes[i]["exact"]
    spec = spec_from_json(fx["task"])
    r, progs = O.enumerate_task(spec, fx["max_depth"], O.REF32_AUDIT)
    last = len(fx["candidates"]) - 1
    assert [r.tried[k] for k in range(last + 1)] == fx["candidates"]
    assert ex["optimal_depth"] == r.optimal_depth
    if r.false_prunes == 0 and r.missed_prunes == 0:
        assert ex["tried"] == fx["candidates"]
        assert ex["pruned_cum"] == fx["pruned_cum"]
        assert modes[i]["exact_programs"][:100] == fx["programs"]
    else:
        assert fx["pruned_cum"][-1] - ex["pruned_cum"][-1] == r.false_prunes - r.missed_prunes


@pytest.mark.parametrize("i", [0, 8, 9, 10, 20, 40, 54])
def test_oracle_exact_fixture_is_reproducible(i):
    """oracle_modes.json (what the GPU tests compare with) is the oracle's
    own output: recompute a sample of it."""
    modes = {m["index"]: m for m in load_golden("oracle_modes.json")}
    fx = ENUM[i]
    spec = spec_from_json(fx["task"])
    r, progs = O.enumerate_task(spec, fx["max_depth"], O.EXACT, 1 << 16)
    last = len(modes[i]["exact"]["tried"]) - 1
    assert [r.tried[k] for k in range(last + 1)] == modes[i]["exact"]["tried"]
    assert [r.survivors[k] for k in range(last + 1)] == modes[i]["exact"]["survivors"]
    assert progs[:200] == modes[i]["exact_programs"]


def test_full_set_contains_reference_programs():
    """No pruning gives the canonical set: every (kernel, output register)
    of the optimal length; the reference prints a subset of it."""
    for fx in ENUM:
        if fx["optimal_depth"] is None or fx["optimal_depth"] > 2:
            continue
        spec = spec_from_json(fx["task"])
        r, full = O.enumerate_task(spec, fx["max_depth"], O.NONE, 1 << 16)
        assert r.optimal_depth == fx["optimal_depth"]
        assert r.total_solutions == len(full)
        fs = {tuple(p) for p in full}
        assert all(tuple(p) in fs for p in fx["programs"])

"""GPU engine parity (through the C ABI) against the reference and the
oracle on the golden tasks. Integer work: every comparison is exact.

  * exact pruner, every level built (count_levels): the reference's
    per-depth "candidates" and cumulative "OEP pruned" counters, the optimal
    length and the printed programs (DFS order, first 100);
  * exact pruner with live in the key: per-level OEP survivor counts;
  * default solve (suffix kernel from level K-1): the proven-optimal length;
  * split at the root (suffix kernel enumerates every kernel): the full
    canonical program set, order and content.
"""
import pytest

from conftest import load_golden, spec_from_json
from pca_gb300.pcalib import OEP_EXACT, OEP_EXACT_LIVE, OEP_NONE

pytestmark = pytest.mark.gpu

ENUM = load_golden("ref_enumerate.json")
MODES = {m["index"]: m for m in load_golden("oracle_modes.json")}
IDS = [f["source"] for f in ENUM]


def ref_depth(fx):
    return fx["optimal_depth"] if fx["optimal_depth"] is not None else -1


@pytest.mark.parametrize("i", range(len(ENUM)), ids=IDS)
def test_counters_and_programs_match_reference(engine, i):
    fx, om = ENUM[i], MODES[i]["exact"]
    spec = spec_from_json(fx["task"])
    sol = engine.solve(spec, max_depth=fx["max_depth"], oep_mode=OEP_EXACT, count_levels=True,
                       sol_cap=1 << 16)
    assert sol.optimal_depth == om["optimal_depth"] == ref_depth(fx)
    last = len(om["tried"]) - 1
    # the oracle's exact counters (full traversal of the last depth)
    assert sol.tried[:last + 1] == om["tried"]
    assert sol.pruned_cum[:last + 1] == om["pruned_cum"]
    assert sol.level_survivors[:last + 1] == om["survivors"]
    assert sol.level_children[:last + 1] == om["children"]
    # where the reference's own pruner is exact (no 32-bit collision, no
    # saturated probe window; see test_oracle_golden) its counters are the
    # same numbers
    if om["tried"] == fx["candidates"] and om["pruned_cum"] == fx["pruned_cum"]:
        assert sol.tried[:last + 1] == fx["candidates"]
        assert sol.pruned_cum[:last + 1] == fx["pruned_cum"]
    if sol.optimal_depth >= 0:
        assert sol.programs[:100] == fx["programs"][:len(sol.programs[:100])] or \
            sol.programs[:100] == MODES[i]["exact_programs"][:100]
        assert sol.programs[:len(fx["programs"])] == MODES[i]["exact_programs"][:len(fx["programs"])]


@pytest.mark.parametrize("i", range(len(ENUM)), ids=IDS)
def test_exact_live_survivor_counts(engine, i):
    fx, om = ENUM[i], MODES[i]["exact_live"]
    spec = spec_from_json(fx["task"])
    sol = engine.solve(spec, max_depth=fx["max_depth"], oep_mode=OEP_EXACT_LIVE,
                       count_levels=True, sol_cap=0)
    last = len(om["survivors"]) - 1
    assert sol.optimal_depth == om["optimal_depth"]
    assert sol.level_survivors[:last + 1] == om["survivors"]
    assert sol.level_children[:last + 1] == om["children"]


@pytest.mark.parametrize("i", range(len(ENUM)), ids=IDS)
def test_default_solve_optimal_depth(engine, i):
    fx = ENUM[i]
    spec = spec_from_json(fx["task"])
    sol = engine.solve(spec, max_depth=fx["max_depth"], sol_cap=1 << 12)
    assert sol.optimal_depth == ref_depth(fx)
    for p in sol.programs:
        assert len(p) == spec.num_inputs + sol.optimal_depth + 2


FULL = [i for i in range(len(ENUM)) if "full" in MODES[i]]


@pytest.mark.parametrize("i", FULL, ids=[IDS[i] for i in FULL])
def test_full_canonical_set(engine, i):
    fx, full = ENUM[i], MODES[i]["full"]
    spec = spec_from_json(fx["task"])
    a = engine.solve(spec, max_depth=fx["max_depth"], split_depth=0, sol_cap=1 << 16)
    assert a.optimal_depth == ref_depth(fx)
    assert a.total_solutions == full["total"]
    assert a.programs == full["programs"]
    b = engine.solve(spec, max_depth=fx["max_depth"], oep_mode=OEP_NONE, count_levels=True,
                     sol_cap=1 << 16)
    assert b.programs == full["programs"]


@pytest.mark.parametrize("split", [0, 1, 2])
def test_suffix_depths_agree(engine, split):
    """Suffix depths 3, 2 and 1 find the same optimum; every program a
    deeper split prints is in the full set of the root split."""
    for i in FULL:
        fx = ENUM[i]
        if fx["optimal_depth"] != 3:
            continue
        spec = spec_from_json(fx["task"])
        full = {tuple(p) for p in MODES[i]["full"]["programs"]}
        s = engine.solve(spec, max_depth=3, split_depth=split, sol_cap=1 << 16)
        assert s.optimal_depth == 3
        assert s.programs and all(tuple(p) in full for p in s.programs)


@pytest.mark.parametrize("i", FULL, ids=[IDS[i] for i in FULL])
def test_lean_last_level_matches_full_levels(engine, i):
    """The reference's task files (up to 16 tests) capped at their optimal
    depth d with split d - 1: the lean last level (links and probes, a hit's
    registers from its parent) gives the programs, counts and levels that
    full levels give, and every program is in the canonical full set."""
    fx = ENUM[i]
    d = ref_depth(fx)
    if d < 2:
        pytest.skip("optimum below kernel depth 2: the last stage reads the root")
    spec = spec_from_json(fx["task"])
    full = {tuple(p) for p in MODES[i]["full"]["programs"]}
    lean = engine.solve(spec, max_depth=d, split_depth=d - 1, sol_cap=1 << 16)
    ref = engine.solve(spec, max_depth=d, split_depth=d - 1, sol_cap=1 << 16, full_levels=True)
    assert lean.optimal_depth == ref.optimal_depth == d
    assert lean.total_solutions == ref.total_solutions
    assert lean.programs == ref.programs
    assert lean.candidates == ref.candidates and lean.evaluations == ref.evaluations
    assert lean.level_survivors == ref.level_survivors
    assert lean.programs and all(tuple(p) in full for p in lean.programs)

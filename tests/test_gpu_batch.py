"""Batched solving (pcagb_solve_batch): many tasks share every launch.
Each task's result inside a batch -- optimal depth, programs in DFS order,
the reference's counters -- equals its result alone and the oracle's; a
batch can mix test counts (16 and 32 tests) and input counts."""
import pytest

from conftest import load_golden, spec_from_json
from pca_gb300 import taskgen
from pca_gb300.pcalib import OEP_EXACT

pytestmark = pytest.mark.gpu

ENUM = load_golden("ref_enumerate.json")
MODES = {m["index"]: m for m in load_golden("oracle_modes.json")}


def ref_depth(fx):
    return fx["optimal_depth"] if fx["optimal_depth"] is not None else -1


def test_batch_equals_single_solves(engine):
    idx = list(range(len(ENUM)))
    tasks = [spec_from_json(ENUM[i]["task"]) for i in idx]
    batch = engine.solve_batch(tasks, max_depth=3, sol_cap=256)
    for i, sol in zip(idx, batch):
        single = engine.solve(tasks[idx.index(i)], max_depth=3, sol_cap=256)
        assert sol.optimal_depth == single.optimal_depth == ref_depth(ENUM[i])
        assert sol.programs == single.programs
        assert sol.total_solutions == single.total_solutions


SMALL = [i for i in range(len(ENUM)) if len(MODES[i]["exact"]["tried"]) <= 3
         or ENUM[i]["task"]["input_ports"] == [0]]


def test_batch_counters_match_oracle(engine):
    tasks = [spec_from_json(ENUM[i]["task"]) for i in SMALL]
    depth = max(ENUM[i]["max_depth"] for i in SMALL)
    batch = engine.solve_batch(tasks, max_depth=3, oep_mode=OEP_EXACT, count_levels=True,
                               sol_cap=1 << 12)
    for i, sol in zip(SMALL, batch):
        om = MODES[i]["exact"]
        last = len(om["tried"]) - 1
        assert sol.optimal_depth == om["optimal_depth"]
        assert sol.tried[:last + 1] == om["tried"], ENUM[i]["source"]
        assert sol.pruned_cum[:last + 1] == om["pruned_cum"], ENUM[i]["source"]
        assert sol.level_survivors[:last + 1] == om["survivors"]
        if sol.optimal_depth >= 0:
            assert sol.programs[:100] == MODES[i]["exact_programs"][:100]


def test_mixed_test_counts_and_depth_caps(engine):
    p2 = taskgen.is_power2_task(1)           # 32 tests, no program within depth 3
    neg = taskgen.negate_task(1)             # 16 tests, depth 1
    syn = [taskgen.synthetic_task(s, 3)[0] for s in range(6)]
    tasks = [p2, neg] + syn
    batch = engine.solve_batch(tasks, max_depth=3, sol_cap=512)
    for t, sol in zip(tasks, batch):
        single = engine.solve(t, max_depth=3, sol_cap=512)
        assert sol.optimal_depth == single.optimal_depth
        assert sol.programs == single.programs
    assert batch[0].optimal_depth == -1 and batch[1].optimal_depth == 1
    # a decided task's time is no later than the batch's end
    assert all(s.seconds <= max(x.seconds for x in batch) + 1e-9 for s in batch)


def test_synthetic_batch_programs_verify(engine):
    from pca_gb300.pcalib import PCALib
    lib = PCALib()
    tasks = taskgen.synthetic_batch(200, seed=5)
    batch = engine.solve_batch(tasks, max_depth=4, sol_cap=8)
    solved = 0
    for t, sol in zip(tasks, batch):
        if sol.optimal_depth >= 0:
            solved += 1
            for p in sol.programs:
                assert lib.evaluate(t, p) == t.num_tests
                assert len(p) == t.num_inputs + sol.optimal_depth + 2
    assert solved > 0

"""The benchmarked configuration against the oracle, through the C ABI: up
to 32 tests, kernel depth 4, levels 1..3 deduplicated by the exact pruner
(key regs+flags+live, the bench's mode, and regs+flags), the last
instruction enumerated by the suffix kernel (split depth 3), every solving
program returned. Fixtures: tests/golden/oracle_depth4.json, made by the
oracle's level-synchronous restatement (tests/golden/make_depth4_fixtures.py).

  * is_power2, 32 tests (the headline step): per-level children and
    survivors, the per-depth counters, and no program within kernel depth 4;
  * synthetic tasks with 17-32 tests and one or two inputs: the optimal
    depth, the number of solving programs, the first 64 in depth-first order
    and a digest of all of them, levels and counters (also with the search
    capped at the optimal depth, whose split level is then built lean, and
    with full levels); the depth-first first
    program under the automatic split, alone and in a batch; under the
    regs+flags key, the levels and the first program (one-input tasks)."""
import hashlib
import struct

import pytest

from conftest import load_golden, spec_from_json
from pca_gb300.pcalib import OEP_EXACT, OEP_EXACT_LIVE

pytestmark = pytest.mark.gpu

D4 = load_golden("oracle_depth4.json")
TASKS = D4["tasks"]
IDS = [f"seed{t['seed']}_in{len(t['task']['input_ports'])}_t{len(t['task']['tests'])}"
       for t in TASKS]


def digest(progs):
    h = hashlib.sha256()
    for p in progs:
        h.update(struct.pack("<16H", *(list(p) + [0] * (16 - len(p)))))
    return h.hexdigest()


def check_levels(sol, want):
    S = len(want["survivors"]) - 1
    K = len(want["tried"]) - 1
    assert sol.level_survivors[:S + 1] == want["survivors"]
    assert sol.level_children[:S + 1] == want["children"]
    assert sol.tried[:K + 1] == want["tried"]
    assert sol.pruned_cum[:K + 1] == want["pruned_cum"]


@pytest.mark.parametrize("shape,full", [(1, False), (32, False), (32, True)],
                         ids=["warp_per_prefix", "lane_per_prefix_lean", "lane_per_prefix_full"])
@pytest.mark.parametrize("mode,key", [(OEP_EXACT_LIVE, "exact_live"), (OEP_EXACT, "exact")])
def test_is_power2_headline_step(engine, mode, key, shape, full):
    """A warp per prefix reads full levels; a lane per prefix reads the last
    level lean (the default) or full (full_levels)."""
    fx = D4["is_power2"]
    want = fx[key]
    spec = spec_from_json(fx["task"])
    sol = engine.solve(spec, max_depth=4, split_depth=3, oep_mode=mode, sol_cap=1 << 12,
                       suffix_chunk=shape, full_levels=full)
    assert sol.optimal_depth == want["optimal_depth"] == -1
    assert sol.total_solutions == 0 and sol.programs == []
    check_levels(sol, want)


@pytest.mark.parametrize("shape", [1, 32], ids=["warp_per_prefix", "lane_per_prefix"])
@pytest.mark.parametrize("i", range(len(TASKS)), ids=IDS)
def test_synthetic_depth4_full_set(engine, i, shape):
    """Every solving program of the benchmarked configuration's last
    position, scanned a warp per prefix or a lane per prefix (suffix_chunk
    1 / 32), against the oracle's full set."""
    fx = TASKS[i]
    want = fx["exact_live"]
    spec = spec_from_json(fx["task"])
    cap = max(want["total_solutions"], 1)
    sol = engine.solve(spec, max_depth=4, split_depth=3, oep_mode=OEP_EXACT_LIVE, sol_cap=cap,
                       suffix_chunk=shape)
    assert sol.optimal_depth == want["optimal_depth"]
    assert sol.total_solutions == want["total_solutions"]
    assert sol.programs[:64] == want["programs"]
    assert digest(sol.programs) == want["digest"]
    check_levels(sol, want)


@pytest.mark.parametrize("full", [False, True], ids=["lean_last_level", "full_levels"])
@pytest.mark.parametrize("i", range(len(TASKS)), ids=IDS)
def test_synthetic_full_set_capped_at_optimal_depth(engine, i, full):
    """The search capped at each task's optimal depth d (split d - 1, the
    oracle's split there): the last depth's split level is built lean (links
    and probes only; a hit's registers recomputed from its parent) unless
    full_levels is set, and every solving program, the levels and the
    counters equal the oracle's."""
    fx = TASKS[i]
    want = fx["exact_live"]
    d = want["optimal_depth"]
    if d < 2:
        pytest.skip("optimum below kernel depth 2: the last stage reads the root")
    spec = spec_from_json(fx["task"])
    cap = max(want["total_solutions"], 1)
    sol = engine.solve(spec, max_depth=d, split_depth=d - 1, oep_mode=OEP_EXACT_LIVE, sol_cap=cap,
                       full_levels=full)
    assert sol.optimal_depth == d
    assert sol.total_solutions == want["total_solutions"]
    assert sol.programs[:64] == want["programs"]
    assert digest(sol.programs) == want["digest"]
    check_levels(sol, want)


@pytest.mark.parametrize("i", range(len(TASKS)), ids=IDS)
def test_synthetic_depth4_first_program(engine, i):
    fx = TASKS[i]
    want = fx["exact_live"]
    spec = spec_from_json(fx["task"])
    sol = engine.solve(spec, max_depth=4, first_only=True, sol_cap=1)
    assert sol.optimal_depth == want["optimal_depth"]
    assert sol.programs == want["programs"][:1]
    if "exact_first" in fx:
        ex = engine.solve(spec, max_depth=4, split_depth=3, oep_mode=OEP_EXACT, first_only=True,
                          sol_cap=1)
        assert ex.optimal_depth == want["optimal_depth"]
        assert ex.programs == fx["exact_first"]
        assert ex.level_survivors[:4] == fx["exact_survivors"]


def test_batch_first_programs(engine):
    """All fixture tasks in one batch (one and two inputs, 17-32 tests):
    each task's optimal depth and depth-first first program as alone."""
    specs = [spec_from_json(fx["task"]) for fx in TASKS]
    batch = engine.solve_batch(specs, max_depth=4, first_only=True, sol_cap=1)
    for fx, sol in zip(TASKS, batch):
        want = fx["exact_live"]
        assert sol.optimal_depth == want["optimal_depth"]
        assert sol.programs[:1] == want["programs"][:1]


def test_batch_full_sets_one_input(engine):
    """One-input tasks and is_power2 in one batch at split 3: every task's
    full solving set and its levels as the oracle's."""
    picked = [fx for fx in TASKS if len(fx["task"]["input_ports"]) == 1][:4]
    specs = [spec_from_json(D4["is_power2"]["task"])] + [spec_from_json(fx["task"])
                                                          for fx in picked]
    cap = max(fx["exact_live"]["total_solutions"] for fx in picked) + 1
    batch = engine.solve_batch(specs, max_depth=4, split_depth=3, sol_cap=cap)
    assert batch[0].optimal_depth == -1
    for fx, sol in zip(picked, batch[1:]):
        want = fx["exact_live"]
        assert sol.optimal_depth == want["optimal_depth"]
        assert sol.total_solutions == want["total_solutions"]
        assert digest(sol.programs) == want["digest"]
        S = len(want["survivors"]) - 1
        assert sol.level_survivors[:S + 1] == want["survivors"]


@pytest.mark.parametrize("split", [1, 2])
def test_depth4_middle_shapes_agree(engine, split):
    """The depth-4 stage from level 2 (two suffix instructions) and from
    level 1 (three): a warp per (prefix, chunk of middles) and a lane per
    innermost middle find the same full set, and the first-only answer is
    the oracle's first program."""
    for fx in [f for f in TASKS if f["exact_live"]["optimal_depth"] == 4][:6]:
        want = fx["exact_live"]
        spec = spec_from_json(fx["task"])
        runs = [engine.solve(spec, max_depth=4, split_depth=split, oep_mode=OEP_EXACT_LIVE,
                             sol_cap=1 << 16, suffix_chunk=ck) for ck in (16, 1024)]
        assert runs[0].optimal_depth == runs[1].optimal_depth == 4
        assert runs[0].total_solutions == runs[1].total_solutions
        assert runs[0].programs == runs[1].programs
        first = engine.solve(spec, max_depth=4, split_depth=split, first_only=True, sol_cap=1,
                             suffix_chunk=1024)
        assert first.programs == want["programs"][:1]

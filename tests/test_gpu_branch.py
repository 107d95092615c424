"""Branch mode (the reference solver's default: CMP, forward BR, DIV, MOD)
on the GPU against the reference's own runs (tests/golden/
make_branch_golden.py): the same optimal length, the same printed programs
in the same order, and the same per-depth "candidates" and cumulative "OEP
pruned" counters (its walk stops at the 100th solution of the optimal depth,
and so do the counters here). The reference keys its pruner on 32 bits in a
table of 2^20 slots per depth; on tasks whose levels outgrow the table it
misses prunes, keeps duplicate states and prints other programs, so
counters and programs are compared where its levels stay small, the optimal
length everywhere (with every program here checked by the VM). On depths
up to 2 every result also equals the CPU restatement of the walk with the
exact pruner (oracle.enumerate_branch), which with the reference's 32-bit
keys reproduces the reference's own numbers (tests/test_oracle_branch.py);
where the two pruners differ, the reference merged distinct states."""
import json
import os
import subprocess

import pytest

from conftest import load_golden, spec_from_json

pytestmark = pytest.mark.gpu

BRANCH = load_golden("ref_enumerate_branch.json")


def small(fx):
    # levels well inside the reference's 2^20-slot tables
    return max(fx["candidates"] or [0]) < 200000


@pytest.mark.parametrize("fx", BRANCH, ids=lambda f: f"task{f['index']}")
def test_branch_mode_matches_reference(engine, fx):
    task = spec_from_json(fx["task"])
    sol = engine.solve_branch(task, max_depth=fx["max_depth"], sol_cap=100)
    want = fx["optimal_depth"] if fx["optimal_depth"] is not None else -1
    assert sol.optimal_depth == want
    if want < 0:
        return
    if fx["max_depth"] <= 2:
        # the exact pruner's walk, restated on the CPU: equal everywhere
        from oracle import oracle as O
        r, progs = O.enumerate_branch(task, fx["max_depth"], O.EXACT)
        assert r.optimal_depth == sol.optimal_depth
        assert sol.programs == progs
        assert sol.tried == [r.tried[k] for k in range(want + 1)]
        assert sol.pruned_cum == [r.pruned_cum[k] for k in range(want + 1)]
        if sol.tried == fx["candidates"]:
            assert sol.pruned_cum == fx["pruned_cum"] and sol.programs == fx["programs"]
        else:
            # the reference's 32-bit keys merged distinct states (its
            # restatement with those keys reproduces it)
            assert sum(fx["candidates"]) < sum(sol.tried)
    elif small(fx):
        assert sol.programs == fx["programs"]
        assert sol.tried == fx["candidates"]
        assert sol.pruned_cum == fx["pruned_cum"]
    else:
        # the reference's saturated tables keep duplicate states, so it
        # prints other representatives; every program here solves the task
        from pca_gb300.pcalib import PCALib
        lib = PCALib()
        assert sol.programs
        for prog in sol.programs:
            assert len(prog) == fx["optimal_length"]
            assert lib.evaluate(task, prog) == task.num_tests


def test_branch_cli_report(tmp_path):
    from pca_gb300.build import LIBDIR
    fx = next(f for f in BRANCH if f["optimal_depth"] == 2 and small(f))
    tp = tmp_path / "task.json"
    tp.write_text(json.dumps(fx["task"]))
    p = subprocess.run([os.path.join(LIBDIR, "enumerate"), str(tp), "-d", str(fx["max_depth"])],
                       capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert "branches on, OEP on" in p.stdout
    assert f"Optimal solution length: {fx['optimal_length']} instructions" in p.stdout
    assert f"Found {fx['found']} distinct program(s)" in p.stdout
    for k, c in enumerate(fx["candidates"]):
        assert f"  candidates: {c}  " in p.stdout


@pytest.mark.parametrize("fx", [f for f in BRANCH if f["optimal_depth"] in (1, 2)][::3],
                         ids=lambda f: f"task{f['index']}")
def test_unbuilt_last_level_gives_same_programs(engine, fx):
    """Without building the last level (solving children found directly, the
    pruner's choice replayed by a second pass), the optimal length and the
    printed programs are the same."""
    task = spec_from_json(fx["task"])
    full = engine.solve_branch(task, max_depth=fx["max_depth"])
    direct = engine.solve_branch(task, max_depth=fx["max_depth"], last_level_max_children=0)
    assert direct.optimal_depth == full.optimal_depth
    assert direct.programs == full.programs
    assert direct.split_used == full.optimal_depth - 1


PUBLISHED = load_golden("ref_published.json")


@pytest.mark.parametrize("t", PUBLISHED, ids=lambda t: t["name"])
def test_published_branch_mode_lengths(engine, t):
    """The reference's documented optimal lengths of its own task files in
    branch mode (negate/double/square 4, add 5, abs/relu 6, max 7, is_power2
    7, saturating_add 8), found and proven here (every shorter depth searched
    completely); the programs pass the VM."""
    from pca_gb300.pcalib import PCALib
    task = spec_from_json(t["task"])
    K = t["published_length"] - task.num_inputs - 2
    sol = engine.solve_branch(task, max_depth=K)
    assert sol.optimal_depth == K
    lib = PCALib()
    assert sol.programs
    for prog in sol.programs:
        assert len(prog) == t["published_length"]
        assert lib.evaluate(task, prog) == task.num_tests


@pytest.mark.parametrize("t", PUBLISHED, ids=lambda t: t["name"])
def test_first_only_branch_mode_same_first_programs(engine, t):
    """The hybrid solver's stopping rule (the optimal depth ends at the
    first launch of parents with a solution, every shorter depth searched
    completely) finds the same optimal length, and its programs are the
    full search's first programs in depth-first order."""
    task = spec_from_json(t["task"])
    K = t["published_length"] - task.num_inputs - 2
    full = engine.solve_branch(task, max_depth=K)
    first = engine.solve_branch(task, max_depth=K, first_only=True)
    assert first.optimal_depth == full.optimal_depth == K
    assert first.programs and first.programs == full.programs[:len(first.programs)]
    assert first.split_used == K - 1


@pytest.mark.parametrize("fx", [f for f in BRANCH if f["optimal_depth"] in (1, 2)][::3],
                         ids=lambda f: f"task{f['index']}")
def test_first_only_branch_mode_on_recorded_runs(engine, fx):
    """On the recorded reference runs: the same optimal length (or none
    within the depth), and the first programs of the full search."""
    task = spec_from_json(fx["task"])
    full = engine.solve_branch(task, max_depth=fx["max_depth"])
    first = engine.solve_branch(task, max_depth=fx["max_depth"], first_only=True)
    assert first.optimal_depth == full.optimal_depth
    assert first.programs == full.programs[:len(first.programs)]

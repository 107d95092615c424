"""The CPU restatement of the reference's branch mode (oracle.enumerate_branch,
REF32 pruner) reproduces the reference's own runs (recorded by
tests/golden/make_branch_golden.py) on every fixture task up to kernel depth
2: optimal length, per-depth "candidates" and "OEP pruned", and the printed
programs in order."""
import pytest

from conftest import load_golden, spec_from_json
from oracle import oracle as O

BRANCH = [f for f in load_golden("ref_enumerate_branch.json") if f["max_depth"] <= 2]


@pytest.mark.parametrize("fx", BRANCH, ids=lambda f: f"task{f['index']}")
def test_restatement_matches_reference(fx):
    task = spec_from_json(fx["task"])
    r, progs = O.enumerate_branch(task, fx["max_depth"], O.REF32)
    want = fx["optimal_depth"] if fx["optimal_depth"] is not None else -1
    assert r.optimal_depth == want
    last = want if want >= 0 else fx["max_depth"]
    assert [r.tried[k] for k in range(last + 1)] == fx["candidates"]
    assert [r.pruned_cum[k] for k in range(last + 1)] == fx["pruned_cum"]
    assert progs == fx["programs"]


def test_exact_pruner_differs_only_by_collisions():
    # tasks where the reference's 32-bit keys merged distinct states: the
    # exact pruner keeps them (more candidates, fewer prunes), same programs
    seen = 0
    for fx in BRANCH:
        if fx["optimal_depth"] != 2:
            continue
        task = spec_from_json(fx["task"])
        r, progs = O.enumerate_branch(task, 2, O.EXACT)
        assert r.optimal_depth == 2
        if [r.tried[k] for k in range(3)] != fx["candidates"]:
            seen += 1
            assert r.tried[2] > fx["candidates"][2]
            assert r.pruned_cum[2] < fx["pruned_cum"][2]
    assert seen >= 1  # the fixtures hold such tasks

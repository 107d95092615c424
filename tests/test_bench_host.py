"""Host logic of bench.py's proofs past depth 4 (continue_open_tasks), over a
stand-in engine: the open tasks are solved again to the deeper cap, cheapest
first (one input before two, fewer tests first), every task started is
finished, none is started once the time budget is spent, and the counts add
up."""
import os
import sys
import time
from argparse import Namespace
from types import SimpleNamespace

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


class FakeEngine:
    calls = []

    def __init__(self, device, budget):
        self.closed = False

    def solve(self, task, max_depth, first_only, sol_cap):
        FakeEngine.calls.append((task.name, max_depth))
        time.sleep(task.cost)
        k = task.answer
        cands = [0] * 5 + [7] * (max_depth - 4 if k < 0 else k - 4)
        return SimpleNamespace(optimal_depth=k, candidates=cands)

    def close(self):
        self.closed = True


def _task(name, n_in, n_tests, answer, cost=0.0):
    return SimpleNamespace(name=name, num_inputs=n_in, num_tests=n_tests, answer=answer, cost=cost)


def test_open_tasks_continue_cheapest_first_within_the_budget(monkeypatch):
    import bench
    import pca_gb300.pcalib as pcalib
    monkeypatch.setattr(pcalib, "Engine", FakeEngine)
    FakeEngine.calls = []
    tasks = [_task("b", 2, 16, -1, 0.3), _task("a", 1, 32, 5), _task("c", 1, 16, -1),
             _task("d", 2, 32, 5, 0.3)]
    args = Namespace(hbm_gb=0.0, beyond_depth=5, beyond_budget_s=0.2)
    out = bench.continue_open_tasks(tasks, args)
    # one input first (fewer tests first), then two; the budget is spent
    # during "b", so "d" is never started
    assert [c[0] for c in FakeEngine.calls] == ["c", "a", "b"]
    assert all(c[1] == 5 for c in FakeEngine.calls)
    assert out["tasks_open_after_depth_4"] == 4 and out["started"] == 3
    assert out["proven_optimal_at_depth"] == {"5": 1}
    assert out["no_program_up_to_depth"] == 2 and out["not_started_time_bound"] == 1
    assert out["one_input"]["tasks"] == 2 and out["two_inputs"]["tasks"] == 1
    assert out["candidates_decided"] == 3 * 7


def test_no_open_tasks(monkeypatch):
    import bench
    import pca_gb300.pcalib as pcalib
    monkeypatch.setattr(pcalib, "Engine", FakeEngine)
    out = bench.continue_open_tasks([], Namespace(hbm_gb=0.0, beyond_depth=5,
                                                  beyond_budget_s=1.0))
    assert out["started"] == 0 and out["not_started_time_bound"] == 0

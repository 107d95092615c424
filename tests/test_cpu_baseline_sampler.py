"""The CPU baseline's sampler (oracle.sample_throughput, the reference
algorithm timed by bench.py's cpu_baseline leg and reference arm): worker
threads take (level-1, level-2) candidate pairs in DFS order and run the
reference DFS below each; the candidate count is the reference's "tried"
count of what was visited (every generated child, plus every output
register tried at a leaf). Where the whole space fits in the budget the
count is exact and does not depend on the thread count."""
from oracle import oracle as O
from pca_gb300 import taskgen


def _rd(insn: int) -> int:
    return (insn >> 8) & 7


def test_depth_one_and_two_counts_are_exact():
    task = taskgen.negate_task(1)
    root_live = 0b10                       # one input, in r1
    c0 = O.gen_candidates(root_live)
    n1, secs, sols = O.sample_throughput(task, 1, 2, 30.0)
    assert n1 == len(c0) and secs >= 0
    want2 = len(c0) + sum(len(O.gen_candidates(root_live | 1 << _rd(c))) for c in c0)
    got = set()
    for threads in (1, 3):
        n2, _, sols2 = O.sample_throughput(task, 2, threads, 30.0)
        # each leaf output register tried is one more candidate; at depth 2
        # every such register holds the target on all tests, so each verifies
        assert sols2 > 0 and n2 == want2 + sols2
        got.add((n2, sols2))
    assert len(got) == 1


def test_budget_bounds_the_sample():
    task = taskgen.is_power2_task(1)
    n, secs, _ = O.sample_throughput(task, 4, 2, 0.2)
    assert 0 < n and secs < 5.0

"""The split-depth autotuner changes the work, never the answer: a
first-only solve returns the proven optimal depth and the DFS-first optimal
program, identical whichever level the last stage starts from -- the
autotuner's pick or any forced split."""
import pytest

from pca_gb300 import taskgen

pytestmark = pytest.mark.gpu


def test_first_program_independent_of_split(engine):
    tasks = taskgen.synthetic_batch(120, seed=17)
    sols = engine.solve_batch(tasks, max_depth=4, sol_cap=1)
    picked = [t for t, s in zip(tasks, sols) if s.optimal_depth >= 2][:20]
    assert picked
    for t in picked:
        auto = engine.solve(t, max_depth=4, first_only=True, sol_cap=1)
        for split in (0, 1, 2, 3):
            forced = engine.solve(t, max_depth=4, first_only=True, sol_cap=1, split_depth=split)
            assert forced.optimal_depth == auto.optimal_depth
            assert forced.programs == auto.programs


def test_batch_first_only_matches_single(engine):
    tasks = taskgen.synthetic_batch(60, seed=23)
    batch = engine.solve_batch(tasks, max_depth=4, sol_cap=1, first_only=True)
    for t, b in zip(tasks, batch):
        single = engine.solve(t, max_depth=4, first_only=True, sol_cap=1)
        assert (b.optimal_depth, b.programs) == (single.optimal_depth, single.programs)

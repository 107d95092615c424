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


def test_launch_choices_change_no_answer(engine):
    """The autotuner's other choices -- tests checked per lane before the
    warp-wide check, middle chunk of the deeper suffix kernels, a warp or a
    lane per prefix at the last position, chunked first-only stages --
    forced to every value: the same optimal depth and the same DFS-first
    program, from splits that run suffix depths 1-3."""
    tasks = taskgen.synthetic_batch(120, seed=29)
    sols = engine.solve_batch(tasks, max_depth=4, sol_cap=1, first_only=True)
    picked = [t for t, s in zip(tasks, sols) if s.optimal_depth >= 3][:8]
    picked += [t for t, s in zip(tasks, sols) if s.optimal_depth < 0][:2]
    assert picked
    for t in picked:
        auto = engine.solve(t, max_depth=4, first_only=True, sol_cap=1)
        for split in (1, 2, 3):
            for ft in (1, 2, 3):
                for ck in (1, 5, 16, 64, 1024):
                    if split == 3 and ck not in (1, 64, 1024):
                        continue   # suffix depth 1: a warp (1) or a lane (>= 32) per prefix
                    f = engine.solve(t, max_depth=4, first_only=True, sol_cap=1, split_depth=split,
                                     first_tests=ft, suffix_chunk=ck)
                    assert (f.optimal_depth, f.programs) == (auto.optimal_depth, auto.programs)
        for launch in (-1, 1, 7, 4096):
            f = engine.solve(t, max_depth=4, first_only=True, sol_cap=1, stage_launch=launch)
            assert (f.optimal_depth, f.programs) == (auto.optimal_depth, auto.programs)


def test_launch_choices_keep_full_sets(engine):
    """Every solving program, not only the first: the full set at the
    optimal depth is the same under each tests-per-lane and chunk choice."""
    tasks = taskgen.synthetic_batch(60, seed=31)
    sols = engine.solve_batch(tasks, max_depth=3, sol_cap=1, first_only=True)
    picked = [t for t, s in zip(tasks, sols) if s.optimal_depth >= 2][:5]
    for t in picked:
        base = engine.solve(t, max_depth=3, split_depth=0, sol_cap=1 << 14)
        for ft in (1, 2, 3):
            for ck in (1, 3, 16, 1024):
                s = engine.solve(t, max_depth=3, split_depth=0, sol_cap=1 << 14, first_tests=ft,
                                 suffix_chunk=ck)
                assert s.optimal_depth == base.optimal_depth
                assert s.total_solutions == base.total_solutions
                assert s.programs == base.programs
        # the last position from level 2: a warp or a lane per prefix
        w = engine.solve(t, max_depth=3, split_depth=2, sol_cap=1 << 14, suffix_chunk=1)
        for ft in (1, 2, 3):
            ln = engine.solve(t, max_depth=3, split_depth=2, sol_cap=1 << 14, first_tests=ft,
                              suffix_chunk=32)
            assert (ln.optimal_depth, ln.total_solutions, ln.programs) == \
                (w.optimal_depth, w.total_solutions, w.programs)
            # the lane kernel sums the evaluation count itself; the warp
            # kernel's is a separate pass over the same prefixes
            assert ln.evaluations_run == w.evaluations_run


def test_tuner_measures_every_choice():
    """On stages large enough to time, the tuner tries each tests-per-lane
    choice twice before settling on the cheapest, then each shape of the
    last position (a warp or a lane per prefix): after eleven is_power2
    depth-4 solves (their depth-4 stage, suffix depth 1, is large enough)
    every choice has two measured costs, and the answers never change. The
    solves build full levels: a lean last level (the default) has no
    register block for a warp per prefix, so its stage always runs a lane per
    prefix and explores tests per lane only. A fresh engine on the device
    starts from the costs earlier engines measured, so the check is on the
    counts having grown to at least one."""
    from pca_gb300.pcalib import Engine
    t = taskgen.is_power2_task(1)
    eng = Engine(0, 8 << 30)
    try:
        outs = [eng.solve(t, max_depth=4, split_depth=3, sol_cap=1, full_levels=True)
                for _ in range(11)]
        lean = eng.solve(t, max_depth=4, split_depth=3, sol_cap=1)
        tun = eng.tuning()
    finally:
        eng.close()
    assert all(o.optimal_depth == -1 for o in outs + [lean])
    assert lean.candidates == outs[0].candidates
    assert tun["t_child_lean_ms"] > 0
    assert all(tun["first_tests_n"][1][ft] >= 2 for ft in (1, 2, 3))
    assert all(tun["first_tests_ms"][1][ft] > 0 for ft in (1, 2, 3))
    assert all(tun["chunk_n"][1][c] >= 2 and tun["chunk_ms"][1][c] > 0 for c in (0, 1))
    assert tun["chunk_choices"][1][:2] == [1, 32]
    assert tun["t_eval_ms"][1] > 0 and tun["launch_rt_ms"] > 0

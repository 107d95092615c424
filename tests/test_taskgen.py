"""Seeded workload generators: shapes and value distributions."""
from pca_gb300 import taskgen


def test_negate_task():
    t = taskgen.negate_task(1)
    xs = [t.tests[i].inputs[0] for i in range(t.num_tests)]
    assert t.num_tests == 16 and t.num_inputs == 1
    assert {0, 1, 0xFFFF, 0x7FFF, 0x8000} <= set(xs)
    assert all(t.tests[i].outputs[0] == (-xs[i]) & 0xFFFF for i in range(16))


def test_is_power2_task():
    t = taskgen.is_power2_task(1)
    xs = [t.tests[i].inputs[0] for i in range(t.num_tests)]
    outs = [t.tests[i].outputs[0] for i in range(t.num_tests)]
    assert t.num_tests == 32
    assert sum(outs) == 13 and 0 in xs and 0x8000 in xs
    for x, o in zip(xs, outs):
        assert o == (1 if x and not x & (x - 1) else 0)


def test_synthetic_tasks_are_consistent():
    for seed in range(50):
        task, prog = taskgen.synthetic_task(seed, 3 + seed % 6)
        assert 16 <= task.num_tests <= 32 and 1 <= task.num_inputs <= 2
        for i in range(task.num_tests):
            ins = [task.tests[i].inputs[k] for k in range(task.num_inputs)]
            assert taskgen.run_program(prog, ins)[prog[-1][1]] == task.tests[i].outputs[0]


def test_batches_deterministic():
    a = taskgen.synthetic_batch(20, seed=3)
    b = taskgen.synthetic_batch(20, seed=3)
    assert [bytes(x) for x in a] == [bytes(x) for x in b]
    s = taskgen.poisson_stream(100)
    assert all(s[i][0] < s[i + 1][0] for i in range(99))

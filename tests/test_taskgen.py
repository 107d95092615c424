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


def test_served_stream_rate_and_length_mix():
    s = taskgen.poisson_stream(4000, rate=50.0, seed=5)
    gaps = [b[0] - a[0] for a, b in zip(s, s[1:])]
    assert abs(sum(gaps) / len(gaps) - 1 / 50.0) < 0.1 / 50.0
    lengths = [int(t.name.decode().rsplit("len", 1)[1]) for _, t in s]
    want = {4: 0.30, 5: 0.30, 6: 0.25, 7: 0.10, 8: 0.05}
    for L, p in want.items():
        assert abs(lengths.count(L) / len(lengths) - p) < 0.03, (L, lengths.count(L))
    assert set(lengths) == set(want)


def test_batched_lengths_and_shapes():
    tasks = taskgen.synthetic_batch(600, seed=9)
    lengths = [int(t.name.decode().rsplit("len", 1)[1]) for t in tasks]
    assert set(lengths) == set(range(3, 9))
    assert all(abs(lengths.count(L) / 600 - 1 / 6) < 0.06 for L in range(3, 9))
    assert {t.num_inputs for t in tasks} == {1, 2}
    assert min(t.num_tests for t in tasks) == 16 and max(t.num_tests for t in tasks) == 32
    assert {int(t.name.decode().rsplit("len", 1)[1]) for t in taskgen.deep_tasks(60)} == {8, 9, 10}


def test_program_generator_distribution():
    import random
    rng = random.Random(0)
    ops, regs, small, imms = {}, set(), 0, 0
    for _ in range(3000):
        for op, rd, rs, rt, imm in taskgen.random_program(rng, 1):
            ops[op] = ops.get(op, 0) + 1
            regs |= {rd, rs, rt} if op not in ("LDI", "ADDI") else {rd}
            if op in ("LDI", "ADDI"):
                imms += 1
                small += imm < 16
    assert set(ops) == set(taskgen.BRANCHLESS_OPS)
    assert all(abs(c / 3000 - 1 / 11) < 0.03 for c in ops.values())
    assert regs == set(range(1, 8))
    assert 0.45 < small / imms < 0.6   # half small immediates, plus uniform ones below 16

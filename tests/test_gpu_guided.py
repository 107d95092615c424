"""The learned part's contract with the exhaustive engine.

* Labels come from the solver: every positive state really finishes
  optimally in its labelled number of steps (checked by an exact GPU
  completion from that state).
* Ordering never changes what is proven: an ordered solve (value network,
  random, DFS) reports the task's optimal depth, and its programs are correct
  and belong to the plain solve's program set at the same split.
* The trained network gains over the plain (DFS) order on held-out tasks:
  fewer prefixes of the optimal depth are visited before the first correct
  program.
"""
import random

import pytest

from pca_gb300 import taskgen
from pca_gb300.pcalib import PCALib

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def pick(engine, seed, n, depths):
    tasks = taskgen.synthetic_batch(n, seed=seed)
    sols = engine.solve_batch(tasks, max_depth=4, sol_cap=1)
    return [t for t, s in zip(tasks, sols) if s.optimal_depth in depths]


def test_positive_labels_are_exact(engine):
    from pca_gb300.guided import label_task
    lib = PCALib()
    rng = random.Random(3)
    tasks = pick(engine, 31, 300, (2, 3))[:8]
    assert tasks
    checked = 0
    for task in tasks:
        sol = engine.solve(task, max_depth=4, sol_cap=256)
        states, depth, label, remaining = label_task(lib, task, sol.programs, sol.optimal_depth, rng, 2)
        ctx = lib.init_ctx(task)
        for s, d, y, r in zip(states, depth, label, remaining):
            if y < 0.5:
                continue
            found, n, insns, _ = engine.complete(ctx, s, d + r)
            assert found and n == r
            checked += 1
    assert checked > 0


@pytest.mark.parametrize("order", ["dfs", "random", "value", "value_sampled",
                                   "value_sampled_long_stage"])
def test_ordered_solve_is_exact(engine, order):
    from pca_gb300.guided import RandomOrder, ValueOrder
    from pca_gb300.valuenet import ValueNet
    lib = PCALib()
    fn = {"dfs": lambda v: None, "random": RandomOrder(5),
          "value": ValueOrder(ValueNet(seed=1), min_states=1, gain=0.0),
          "value_sampled": ValueOrder(ValueNet(seed=1), min_states=1, gain=0.0, sample=512,
                                      full_gain=None),
          # every stage counts as long: the whole level is ranked though a
          # sample size is set
          "value_sampled_long_stage": ValueOrder(ValueNet(seed=1), min_states=1, gain=0.0,
                                                 sample=512, full_gain=0.0)}[order]
    for task in pick(engine, 41, 300, (3, 4))[:6]:
        plain = engine.solve(task, max_depth=4, split_depth=2, sol_cap=1 << 14)
        got = engine.solve_ordered(task, fn, chunk=64, max_depth=4, split_depth=2, sol_cap=1 << 14)
        assert got.optimal_depth == plain.optimal_depth
        assert got.programs and set(map(tuple, got.programs)) <= set(map(tuple, plain.programs))
        for p in got.programs:
            assert lib.evaluate(task, p) == task.num_tests
        assert 0 < got.prefixes_to_first <= got.prefixes_at_optimal


@pytest.mark.parametrize("order", ["dfs", "value"])
def test_ordered_solve_auto_split_is_exact(engine, order):
    """With an automatic split the engine runs a stage it expects to be
    cheap plain (keeping its DFS-first solution) and orders the others;
    either way the optimal depth and correct programs of the plain set come
    back."""
    from pca_gb300.guided import ValueOrder
    from pca_gb300.valuenet import ValueNet
    lib = PCALib()
    fn = {"dfs": lambda v: None, "value": ValueOrder(ValueNet(seed=1), min_states=1, gain=0.0)}[order]
    tasks = pick(engine, 41, 300, (3, 4))[:6] + pick(engine, 202, 800, (4,))[:2]
    for task in tasks:
        plain = engine.solve(task, max_depth=4, split_depth=2, sol_cap=1 << 14)
        got = engine.solve_ordered(task, fn, chunk=64, max_depth=4, split_depth=-1, sol_cap=1 << 14)
        assert got.optimal_depth == plain.optimal_depth
        assert got.programs and set(map(tuple, got.programs)) <= set(map(tuple, plain.programs))
        for p in got.programs:
            assert lib.evaluate(task, p) == task.num_tests


def test_trained_network_beats_dfs_order(engine):
    from pca_gb300.guided import ValueOrder, build_dataset, train
    from pca_gb300.valuenet import ValueNet
    ds, used = build_dataset(engine, taskgen.synthetic_batch(1500, seed=101), max_depth=4, seed=1)
    assert used > 50
    net = ValueNet(seed=0, lr=1e-3, pos_weight=8.0)
    losses = train(net, ds, epochs=6)
    assert losses[-1] < losses[0]
    vo = ValueOrder(net, min_states=1, gain=0.0)
    frac_dfs, frac_val = [], []
    for task in pick(engine, 202, 800, (3, 4))[:24]:
        a = engine.solve_ordered(task, lambda v: None, chunk=256, max_depth=4, split_depth=2)
        b = engine.solve_ordered(task, vo, chunk=256, max_depth=4, split_depth=2)
        assert a.optimal_depth == b.optimal_depth
        frac_dfs.append(a.prefixes_to_first / a.prefixes_at_optimal)
        frac_val.append(b.prefixes_to_first / b.prefixes_at_optimal)
    assert sum(frac_val) < 0.5 * sum(frac_dfs)


def _orders_task(engine):
    return pick(engine, 41, 300, (3, 4))[0]


@pytest.mark.parametrize("kind", ["duplicate", "out_of_range", "short", "float", "raises"])
def test_bad_orders_are_refused(engine, kind):
    """An order that is not a permutation of the level (it would skip
    prefixes and leave a depth unproven, or index outside the level) is
    refused before any kernel reads it; an exception in the callback comes
    back to the caller. The engine stays usable afterwards."""
    from pca_gb300.pcalib import EngineError
    task = _orders_task(engine)

    class Boom(Exception):
        pass

    def fn(view):
        n = view.n
        if kind == "raises":
            raise Boom()
        if kind == "short":
            # n - 1 entries; the word after them (inside the same allocation,
            # so an allocation-granular range check cannot see the shortfall)
            # repeats entry 0, so reading n entries finds a duplicate
            buf = torch.arange(n + 1, dtype=torch.int32, device="cuda")
            buf[max(n - 1, 0)] = 0
            return buf[:max(n - 1, 0)]
        if kind == "float":
            return torch.arange(n, dtype=torch.float32, device="cuda")
        o = torch.arange(n, dtype=torch.int32, device="cuda")
        if n >= 2 and kind == "duplicate":
            o[1] = 0
        if kind == "out_of_range":
            o[-1] = n
        return o

    expect = Boom if kind == "raises" else EngineError
    with pytest.raises(expect):
        engine.solve_ordered(task, fn, chunk=64, max_depth=4, split_depth=2)
    plain = engine.solve(task, max_depth=4, split_depth=2, sol_cap=1)
    again = engine.solve_ordered(task, lambda v: None, chunk=64, max_depth=4, split_depth=2)
    assert again.optimal_depth == plain.optimal_depth


def test_host_pointer_order_is_refused(engine):
    """Through the raw C ABI: a callback that hands back host memory is
    refused (the engine checks the pointer's memory type and range before
    launching anything on it)."""
    import ctypes

    import numpy as np

    from pca_gb300.pcalib import ORDER_CB, SolveOpts, SolveResult
    task = _orders_task(engine)
    lib = engine.lib
    host = np.arange(1 << 16, dtype=np.uint32)
    cb = ORDER_CB(lambda vp, _u: host.ctypes.data)
    o = SolveOpts()
    lib.pcagb_default_opts(ctypes.byref(o))
    o.max_depth, o.split_depth = 4, 2
    r = SolveResult()
    progs = (ctypes.c_uint16 * 16)()
    lens = (ctypes.c_int * 1)()
    rc = lib.pcagb_solve_ordered(engine.h, ctypes.byref(task), ctypes.byref(o), cb, None, 64,
                                 ctypes.byref(r), progs, lens, 1)
    assert rc != 0
    assert b"not device memory" in lib.pcagb_last_error()
    assert engine.solve(task, max_depth=4, split_depth=2, sol_cap=1).optimal_depth >= 0

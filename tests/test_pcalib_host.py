"""The ctypes engine wrapper's host logic over a stand-in for libpcagb
(pca_gb300.pcalib.Engine takes the library object): results are converted
per task, and an exception raised in a Python callback -- on_done of a
batch, the order callback of an ordered solve -- never crosses the C
boundary: the engine sees a normal return (DFS order for an order
callback) and the exception is raised once the call returns."""
import ctypes

import pytest

from pca_gb300 import taskgen
from pca_gb300.pcalib import Engine, EngineError, LevelView


class FakeLib:
    def __init__(self):
        self.order_returns = []
        self.destroyed = False

    def pcagb_engine_create(self, device, budget, out):
        out._obj.value = 0x1000
        return 0

    def pcagb_engine_destroy(self, h):
        self.destroyed = True

    def pcagb_default_opts(self, o):
        pass

    def pcagb_last_error(self):
        return b"stand-in error"

    def pcagb_solve_batch_cb(self, h, arr, n, o, res, progs, lens, cap, cb, user):
        for i in range(n):       # task i: one stored program [100 + i, 7]
            res[i].optimal_depth = i % 3
            res[i].stored = 1
            res[i].candidates[0] = 10 * i
            lens[i * cap] = 2
            progs[i * cap * 16] = 100 + i
            progs[i * cap * 16 + 1] = 7
            cb(i, ctypes.pointer(res[i]), None)
        return 0

    def pcagb_solve_ordered(self, h, task, o, cb, user, chunk, r, progs, lens, cap):
        view = LevelView(n=5, tp=32, depth=2)
        self.order_returns.append(cb(ctypes.pointer(view), None))
        r._obj.optimal_depth = 3
        return 0


def _engine():
    lib = FakeLib()
    return Engine(0, 0, lib=lib), lib


def test_batch_results_are_converted_per_task():
    eng, lib = _engine()
    seen = []
    sols = eng.solve_batch([taskgen.negate_task(s) for s in range(4)], max_depth=4, sol_cap=2,
                           on_done=lambda i, sol: seen.append((i, sol.programs)))
    assert [s.optimal_depth for s in sols] == [0, 1, 2, 0]
    assert [s.programs for s in sols] == [[[100 + i, 7]] for i in range(4)]
    assert seen == [(i, [[100 + i, 7]]) for i in range(4)]
    assert [s.candidates[0] for s in sols] == [0, 10, 20, 30]
    eng.close()
    assert lib.destroyed


def test_on_done_exception_is_raised_after_the_batch():
    eng, _ = _engine()
    calls = []

    def on_done(i, sol):
        calls.append(i)
        if i == 1:
            raise ValueError("delivery failed")

    with pytest.raises(ValueError, match="delivery failed"):
        eng.solve_batch([taskgen.negate_task(s) for s in range(3)], on_done=on_done)
    assert calls == [0, 1, 2]   # the engine went on with the batch


def test_order_callback_exception_means_dfs_order_then_raise():
    eng, lib = _engine()

    def bad_order(view):
        assert view.n == 5 and view.depth == 2
        raise RuntimeError("ranking failed")

    with pytest.raises(RuntimeError, match="ranking failed"):
        eng.solve_ordered(taskgen.negate_task(1), bad_order)
    assert lib.order_returns == [None]


def test_order_callback_must_return_a_device_permutation_tensor():
    import torch
    eng, lib = _engine()
    with pytest.raises(EngineError, match="int32 CUDA tensor"):
        eng.solve_ordered(taskgen.negate_task(1), lambda view: torch.arange(view.n))
    assert lib.order_returns == [None]
    sol = eng.solve_ordered(taskgen.negate_task(1), lambda view: None)
    assert sol.optimal_depth == 3 and lib.order_returns == [None, None]


def test_order_object_starts_every_solve_afresh():
    """An order object with per-level state (ValueOrder keys scored levels
    by device address, size and depth) is told before each ordered solve,
    so a level of a later solve at a freed level's address is scored anew."""
    eng, _ = _engine()
    events = []

    class Order:
        def new_solve(self):
            events.append("new_solve")

        def __call__(self, view):
            events.append("order")
            return None

    order = Order()
    task = taskgen.negate_task(1)
    eng.solve_ordered(task, order)
    eng.solve_ordered(task, order)
    assert events == ["new_solve", "order", "new_solve", "order"]

"""The serving loop's host logic, on the CPU, over engines that stand in for
the GPU solver (pca_gb300.serve with engine_factory): requests that arrive
while a slot is busy join the next batch, every request gets its own task's
answer as soon as that task is decided, the serial baseline takes one task
at a time, and an engine error reaches the requests it leaves open without
stopping the server."""
import time
from dataclasses import dataclass

from pca_gb300.serve import SerialServer, Server, latency_summary, replay


@dataclass
class FakeSolution:
    optimal_depth: int
    candidates: tuple


def answer(task) -> FakeSolution:
    return FakeSolution(optimal_depth=task % 5, candidates=(task, 1))


class FakeEngine:
    """solve_batch sleeps `delay` seconds per call, then decides its tasks in
    reverse order; a task equal to `fail_on` makes the call raise after the
    tasks decided before it."""

    def __init__(self, delay=0.05, fail_on=None):
        self.delay = delay
        self.fail_on = fail_on
        self.calls = []
        self.closed = False

    def solve_batch(self, tasks, max_depth, oep_mode, sol_cap, on_done, first_only,
                    shared_gpu=False):
        assert first_only
        self.calls.append(list(tasks))
        time.sleep(self.delay)
        for i in reversed(range(len(tasks))):
            if tasks[i] == self.fail_on:
                raise RuntimeError(f"engine error on task {tasks[i]}")
            on_done(i, answer(tasks[i]))

    def close(self):
        self.closed = True


def test_requests_arriving_while_busy_join_the_next_batch():
    engines = []

    def factory():
        engines.append(FakeEngine(delay=0.2))
        return engines[-1]

    srv = Server(slots=1, max_batch=8, engine_factory=factory)
    first = srv.submit(0, 100)
    time.sleep(0.05)            # the first batch is on the (fake) device
    rest = [srv.submit(i, 100 + i) for i in range(1, 11)]
    for r in [first] + rest:
        assert r.done.wait(10)
    srv.close()
    assert engines[0].closed
    # batch 1: the lone request; then the queue drained in arrival order, at
    # most max_batch per batch
    assert srv.batches == [1, 8, 2]
    assert engines[0].calls == [[100], list(range(101, 109)), [109, 110]]
    for r in [first] + rest:
        assert r.solution == answer(r.task) and r.error is None
        assert r.latency >= 0


def test_answers_are_per_task_in_a_mixed_trace():
    srv = Server(slots=3, max_batch=16, engine_factory=lambda: FakeEngine(delay=0.02))
    trace = [(0.002 * i, 7 * i + 3) for i in range(60)]
    reqs = replay(srv, trace)
    srv.close()
    assert [r.task for r in reqs] == [t for _, t in trace]
    assert all(r.solution == answer(r.task) for r in reqs)
    assert sum(srv.batches) == 60 and max(srv.batches) > 1
    s = latency_summary(reqs)
    assert s["requests"] == 60 and s["failed"] == 0
    assert s["proven_optimal"] == 60
    assert s["candidates"] == sum(t + 1 for _, t in trace)
    assert s["p50_s"] <= s["p99_s"] <= s["max_s"]


def test_serial_baseline_takes_one_task_at_a_time():
    srv = SerialServer(engine_factory=lambda: FakeEngine(delay=0.01))
    reqs = replay(srv, [(0.0, t) for t in range(12)])
    srv.close()
    assert srv.batches == [1] * 12
    assert [r.solution for r in reqs] == [answer(t) for t in range(12)]


def test_engine_error_reaches_open_requests_and_the_server_goes_on():
    srv = Server(slots=1, max_batch=4, engine_factory=lambda: FakeEngine(delay=0.1, fail_on=2))
    hold = srv.submit(0, 50)        # occupies the slot while the next four queue
    time.sleep(0.03)
    batch = [srv.submit(i, t) for i, t in enumerate((1, 2, 3, 4), start=1)]
    for r in [hold] + batch:
        assert r.done.wait(10)
    later = srv.submit(9, 6)        # the worker is still serving
    assert later.done.wait(10)
    srv.close()
    by_task = {r.task: r for r in batch}
    # reverse order: 4 and 3 were decided before the error on 2
    assert by_task[4].solution == answer(4) and by_task[3].solution == answer(3)
    for t in (2, 1):
        assert by_task[t].solution is None
        assert isinstance(by_task[t].error, RuntimeError)
    assert hold.solution == answer(50)
    assert later.solution == answer(6) and later.error is None
    s = latency_summary([hold] + batch + [later])
    assert s["failed"] == 2 and s["proven_optimal"] == 4


def test_close_stops_every_worker():
    srv = Server(slots=3, engine_factory=lambda: FakeEngine(delay=0.0))
    reqs = replay(srv, [(0.0, t) for t in range(5)])
    srv.close()
    assert all(not t.is_alive() for t in srv.threads)
    assert all(r.done.is_set() for r in reqs)


def test_close_answers_queued_requests_and_refuses_new_ones():
    srv = Server(slots=1, max_batch=2, engine_factory=lambda: FakeEngine(delay=0.05))
    reqs = [srv.submit(i, i) for i in range(7)]   # queued behind a busy slot
    srv.close()
    assert all(r.done.is_set() and r.solution == answer(r.task) for r in reqs)
    assert sum(srv.batches) == 7 and max(srv.batches) <= 2
    try:
        srv.submit(99, 1)
    except RuntimeError:
        pass
    else:
        raise AssertionError("a closed server took a request")


def test_close_leaves_a_busy_worker_to_free_its_engine_after_its_solve():
    import warnings

    eng = FakeEngine(delay=1.0)
    srv = Server(slots=1, engine_factory=lambda: eng)
    r = srv.submit(0, 3)
    time.sleep(0.05)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        srv.close(timeout=0.1)
    assert not eng.closed and any(issubclass(x.category, RuntimeWarning) for x in w)
    assert r.done.wait(5) and r.solution == answer(3)
    srv.threads[0].join(5)
    assert eng.closed, "the worker did not free its engine when its solve ended"

"""Serving: continuous batching over several engine slots. Requests arrive
while others run, join the next free slot's batch, and each answer -- the
proven optimal depth and its programs -- is the same as the task's answer
alone."""
import time

import pytest

from pca_gb300 import taskgen
from pca_gb300.serve import SerialServer, Server, latency_summary, replay

pytestmark = pytest.mark.gpu


def trace(n=48, rate=5000.0):
    # short tasks (source length 3-5) so the test stays quick
    return [(t, task) for t, task in taskgen.poisson_stream(n, rate=rate, seed=21)]


def test_served_results_equal_single_solves(engine):
    tr = trace()
    srv = Server(slots=3, max_batch=64, max_depth=3, hbm_fraction=0.3)
    try:
        reqs = replay(srv, tr)
    finally:
        srv.close()
    # a burst: requests arriving while the slots are busy share batches
    assert len(srv.batches) < len(tr), "requests were not batched"
    for r, (_, task) in zip(reqs, tr):
        alone = engine.solve(task, max_depth=3, sol_cap=16, first_only=True)
        assert r.solution.optimal_depth == alone.optimal_depth
        assert r.solution.programs == alone.programs
        assert r.latency >= 0
    s = latency_summary(reqs)
    assert s["requests"] == len(tr) and s["p50_s"] <= s["p99_s"]


def test_serial_server_matches_too(engine):
    tr = trace(12, 100.0)
    srv = SerialServer(max_depth=3, hbm_fraction=0.2)
    try:
        reqs = replay(srv, tr)
    finally:
        srv.close()
    assert all(b == 1 for b in srv.batches)
    for r, (_, task) in zip(reqs, tr):
        assert r.solution.optimal_depth == engine.solve(task, max_depth=3).optimal_depth


def test_native_server_results_equal_single_solves(engine):
    """The native server (admission by free HBM, concurrent solves on their
    own streams, queued requests batched): every answer equals the task's
    answer alone."""
    from pca_gb300.serve import NativeServer
    tr = trace(64, 3000.0)
    srv = NativeServer(workers=4, max_batch=16, max_depth=3, pool_bytes=8 << 30,
                       arena_bytes=512 << 20)
    try:
        reqs = replay(srv, tr)
        st = srv.stats()
    finally:
        srv.close()
    assert st["finished"] == len(tr) and st["admitted"] == len(tr)
    assert st["batches"] < len(tr), "no queued requests were batched"
    for r, (_, task) in zip(reqs, tr):
        assert r.error is None
        alone = engine.solve(task, max_depth=3, sol_cap=16, first_only=True)
        assert r.solution.optimal_depth == alone.optimal_depth
        assert r.solution.programs == alone.programs


def test_request_admitted_while_a_long_solve_runs(engine):
    """A request submitted while another solve is running is admitted and
    answered before that solve finishes, with the same answer as alone."""
    from pca_gb300.serve import NativeServer
    long_task = taskgen.is_power2_task(1)        # no program up to kernel depth 5: ~1 s
    shorts = [task for _, task in trace(8, 100.0)]
    srv = NativeServer(workers=3, max_batch=1, max_depth=3, pool_bytes=24 << 30,
                       arena_bytes=8 << 30)
    try:
        big = srv.submit(0, long_task, max_depth=5)
        time.sleep(0.2)                           # the long solve is on the GPU
        small = [srv.submit(i + 1, t) for i, t in enumerate(shorts)]
        for r in small:
            assert r.done.wait(120)
        big.done.wait(300)
    finally:
        srv.close()
    assert big.error is None and big.solution.optimal_depth == -1
    for r, t in zip(small, shorts):
        assert r.error is None
        # both on the server's clock
        assert 0 <= r.admitted < big.finished and r.finished < big.finished
        alone = engine.solve(t, max_depth=3, sol_cap=16, first_only=True)
        assert (r.solution.optimal_depth, r.solution.programs) == (alone.optimal_depth,
                                                                   alone.programs)


def test_admission_waits_for_free_memory():
    """A pool that holds two arenas runs at most two solves at once although
    four workers are idle; every request is still answered."""
    from pca_gb300.serve import NativeServer
    tr = trace(24, 2000.0)
    srv = NativeServer(workers=4, max_batch=1, max_depth=3, pool_bytes=2 * (256 << 20),
                       arena_bytes=256 << 20)
    try:
        reqs = replay(srv, tr)
        st = srv.stats()
    finally:
        srv.close()
    assert all(r.error is None for r in reqs)
    assert st["max_running_solves"] <= 2
    assert st["pool_peak"] <= 2 * (256 << 20)

"""Serving: continuous batching over several engine slots. Requests arrive
while others run, join the next free slot's batch, and each answer -- the
proven optimal depth and its programs -- is the same as the task's answer
alone."""
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

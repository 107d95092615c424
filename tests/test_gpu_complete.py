"""GPU-backed search_exhaustive_complete through the libpca ABI, on the
cases of the reference's python/test_exhaustive.py: shortest completion
length, no completion below the optimum, partial-state completion, no state
leaking between calls, and replay of the returned path."""
import pytest

from conftest import load_golden, spec_from_json
from pca_gb300.pcalib import PCALib

pytestmark = pytest.mark.gpu

CASES = load_golden("ref_libpca.json")["complete"]


def replay_solves(L, ctx, state, insns):
    cur = state
    for insn in insns:
        cur = L.step(ctx, cur, insn)
        if cur is None:
            return False
    return bool(L.leaf_check(ctx, cur))


@pytest.mark.parametrize("case", CASES, ids=lambda c: c["task"]["name"])
def test_complete_matches_reference(case):
    L = PCALib()
    spec = spec_from_json(case["task"])
    ctx = L.init_ctx(spec)
    for run in case["runs"]:
        s = L.init_root(ctx)
        for insn in run["start"]:
            s = L.step(ctx, s, insn)
        found, n, insns = L.exhaustive_complete(ctx, s, run["max_depth"])
        assert int(found) == run["found"]
        assert n == run["len"]
        if found:
            assert replay_solves(L, ctx, s, insns)
            assert insns == run["insns"]


def test_no_leak_between_calls():
    L = PCALib()
    spec0 = spec_from_json(CASES[-1]["task"])
    ctx0 = L.init_ctx(spec0)
    first = L.exhaustive_complete(ctx0, L.init_root(ctx0), CASES[-1]["manifest_depth"])
    for case in CASES:
        spec = spec_from_json(case["task"])
        ctx = L.init_ctx(spec)
        L.exhaustive_complete(ctx, L.init_root(ctx), case["manifest_depth"])
    again = L.exhaustive_complete(ctx0, L.init_root(ctx0), CASES[-1]["manifest_depth"])
    assert again == first

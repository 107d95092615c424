"""The oracle against the reference's own `enumerate --no-branch`, run live
on tasks that are not in the golden fixtures (oracle/_ref, built from the
reference's sources; skipped where it is absent): per-depth candidates,
cumulative OEP-pruned counts, the optimal depth and the printed programs
agree on fresh seeded tasks of one and two inputs, in branchless mode and
in the reference's branch mode."""
import importlib.util
import json
import os

import pytest

from conftest import GOLDEN, REPO
from oracle import oracle as O
from pca_gb300 import taskgen

REF_BIN = os.path.join(REPO, "oracle", "_ref", "enumerate")


def _golden_tools():
    spec = importlib.util.spec_from_file_location("make_golden",
                                                  os.path.join(GOLDEN, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


# optimal kernel depth 2 (one and two inputs), 3, and none up to depth 3
@pytest.mark.parametrize("seed,length", [(1001, 4), (1057, 3), (1006, 4), (1036, 4), (1022, 4),
                                         (1001, 3)])
def test_oracle_matches_live_reference(tmp_path, seed, length):
    if not os.path.exists(REF_BIN):
        pytest.skip("the reference's enumerate is not built here")
    tools = _golden_tools()
    task, _ = taskgen.synthetic_task(seed, length)
    path = tmp_path / "task.json"
    path.write_text(json.dumps(tools.task_to_json(task), indent=2))
    depth = 3
    want = tools.run_reference(str(path), depth)
    got, progs = O.enumerate_task(task, depth, O.REF32)
    last = got.optimal_depth if got.optimal_depth >= 0 else depth
    assert [got.tried[k] for k in range(last + 1)] == want["candidates"]
    assert [got.pruned_cum[k] for k in range(last + 1)] == want["pruned_cum"]
    assert got.optimal_depth == (want["optimal_depth"] if want["optimal_depth"] is not None
                                 else -1)
    assert progs == want["programs"]


@pytest.mark.parametrize("seed,length", [(1001, 4), (1057, 3), (1006, 4), (1036, 4)])
def test_branch_restatement_matches_live_reference(tmp_path, seed, length):
    """The same for the reference's branch mode (its default: CMP, forward
    BR, DIV and MOD) to kernel depth 2."""
    import subprocess
    if not os.path.exists(REF_BIN):
        pytest.skip("the reference's enumerate is not built here")
    tools = _golden_tools()
    task, _ = taskgen.synthetic_task(seed, length)
    path = tmp_path / "task.json"
    path.write_text(json.dumps(tools.task_to_json(task), indent=2))
    out = subprocess.run([REF_BIN, str(path), "-d", "2"], capture_output=True, text=True,
                         timeout=600).stdout
    want = _parse(out)
    got, progs = O.enumerate_branch(task, 2, O.REF32)
    want_depth = want["optimal_depth"] if want["optimal_depth"] is not None else -1
    assert got.optimal_depth == want_depth
    last = want_depth if want_depth >= 0 else 2
    assert [got.tried[k] for k in range(last + 1)] == want["candidates"]
    assert [got.pruned_cum[k] for k in range(last + 1)] == want["pruned_cum"]
    assert progs == want["programs"]


def _parse(out: str) -> dict:
    spec = importlib.util.spec_from_file_location(
        "make_branch_golden", os.path.join(GOLDEN, "make_branch_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.parse(out)

"""`enumerate --record` from the GPU levels (pcagb_record) against the
reference's own recording pass: the states and edges files are identical
byte for byte (SHA-256 of each, recorded from the reference binary by
tests/golden/make_record_golden.py on tasks where its 32-bit pruner is
exact), and so are the counts in the report."""
import hashlib
import json
import os
import subprocess

import pytest

from conftest import load_golden, spec_from_json

pytestmark = pytest.mark.gpu

RUNS = load_golden("ref_record.json")
ENUM = load_golden("ref_enumerate.json")


@pytest.mark.parametrize("run", RUNS, ids=lambda r: f"task{r['index']}_stride{r['neg_stride']}")
def test_record_files_equal_reference(engine, run, tmp_path):
    task = spec_from_json(ENUM[run["index"]]["task"])
    st = engine.record(task, str(tmp_path), max_depth=run["depth"], task_id=run["task_id"],
                       neg_stride=run["neg_stride"])
    assert st["optimal_depth"] == run["depth"]
    assert (st["states_written"], st["positives"], st["negatives"], st["edges_written"],
            st["optimal_states"]) == (run["written"], run["positives"], run["negatives"],
                                      run["edges"], run["optimal_states"])
    states = open(tmp_path / f"states_{run['task_id']:06d}.bin", "rb").read()
    edges = open(tmp_path / f"edges_{run['task_id']:06d}.bin", "rb").read()
    assert states[:2 * 576].hex() == run["first_states_hex"]
    assert edges[:4 * 24].hex() == run["first_edges_hex"]
    assert len(states) == run["states_bytes"] and len(edges) == run["edges_bytes"]
    assert hashlib.sha256(states).hexdigest() == run["states_sha256"]
    assert hashlib.sha256(edges).hexdigest() == run["edges_sha256"]


def test_record_nothing_without_a_program(engine, tmp_path):
    task = spec_from_json(ENUM[RUNS[-1]["index"]]["task"])
    depth = RUNS[-1]["depth"]
    st = engine.record(task, str(tmp_path), max_depth=depth - 1, task_id=7)
    assert st["optimal_depth"] == -1 and st["states_written"] == 0
    assert not os.listdir(tmp_path)


def test_cli_record_report(tmp_path):
    from pca_gb300.build import LIBDIR
    run = next(r for r in RUNS if r["depth"] == 2)
    tp = tmp_path / "task.json"
    tp.write_text(json.dumps(ENUM[run["index"]]["task"]))
    out = tmp_path / "rec"
    out.mkdir()
    p = subprocess.run([os.path.join(LIBDIR, "enumerate"), str(tp), "-d", str(run["depth"]),
                        "--record", str(out), "--task-id", str(run["task_id"]), "--neg-stride",
                        str(run["neg_stride"])], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr
    assert f"states: {run['written']} written ({run['positives']} positive, " \
           f"{run['negatives']} negative)" in p.stdout
    assert f"edges: {run['edges']} written" in p.stdout
    assert f"optimal state set: {run['optimal_states']} states across {run['depth'] + 1} depths" \
        in p.stdout
    states = (out / f"states_{run['task_id']:06d}.bin").read_bytes()
    assert hashlib.sha256(states).hexdigest() == run["states_sha256"]

"""The `enumerate` and `gpu_hybrid` command lines (drop-ins for the
reference's tools/enumerate.c and gpu/hybrid.cu programs): argument
grammar, report lines and exit codes. GPU runs are marked; argument
handling that stops before the engine runs on the CPU."""
import json
import os
import re
import subprocess

import pytest

from conftest import REPO, load_golden

LIB = os.path.join(REPO, "pca_gb300", "_lib")
ENUM = load_golden("ref_enumerate.json")
MODES = {m["index"]: m for m in load_golden("oracle_modes.json")}


def write_task(tmp_path, fx):
    p = tmp_path / "task.json"
    p.write_text(json.dumps(fx["task"], indent=2))
    return str(p)


def run(args):
    return subprocess.run(args, capture_output=True, text=True, timeout=600)


def test_branch_mode_without_pruner_is_refused(tmp_path):
    r = run([os.path.join(LIB, "enumerate"), write_task(tmp_path, ENUM[0]), "-d", "2", "--no-oep"])
    assert r.returncode == 2
    assert "branch mode" in r.stderr


def test_usage(tmp_path):
    assert run([os.path.join(LIB, "enumerate")]).returncode == 1
    assert run([os.path.join(LIB, "gpu_hybrid")]).returncode == 1


def parse_enumerate(out):
    cands = [int(x) for x in re.findall(r"  candidates: (\d+) ", out)]
    pruned = [int(x) for x in re.findall(r"  OEP pruned: (\d+)\n", out)]
    sols = [[int(w, 16) for w in re.findall(r"    [0-9A-F]{2}: ([0-9A-F]{4})", blk)]
            for blk in re.findall(r"Solution #\d+ \(\d+ instructions\):\n((?:    [0-9A-F]{2}: .*\n)+)", out)]
    m = re.search(r"Optimal solution length: (\d+) instructions \(kernel depth (\d+)\)", out)
    return cands, pruned, sols, (int(m.group(2)) if m else None)


PICK = [0, 3, 9, 17, 26, 33, 47, 54]


@pytest.mark.gpu
@pytest.mark.parametrize("i", PICK, ids=[ENUM[i]["source"] for i in PICK])
def test_enumerate_cli_matches_reference(tmp_path, i):
    fx, om = ENUM[i], MODES[i]["exact"]
    r = run([os.path.join(LIB, "enumerate"), write_task(tmp_path, fx), "-d", str(fx["max_depth"]),
             "--no-branch", "--count"])
    assert r.returncode == (0 if fx["optimal_depth"] is not None else 1), r.stderr
    cands, pruned, sols, k = parse_enumerate(r.stdout)
    assert k == fx["optimal_depth"]
    assert cands == om["tried"] and pruned == om["pruned_cum"]
    if om["tried"] == fx["candidates"] and om["pruned_cum"] == fx["pruned_cum"]:
        assert cands == fx["candidates"]
    assert sols == MODES[i]["exact_programs"][:100]
    # the fast path prints the same programs
    r2 = run([os.path.join(LIB, "enumerate"), write_task(tmp_path, fx), "-d", str(fx["max_depth"]),
              "--no-branch"])
    assert parse_enumerate(r2.stdout)[2:] == (sols, k)


@pytest.mark.gpu
@pytest.mark.parametrize("i", PICK, ids=[ENUM[i]["source"] for i in PICK])
def test_gpu_hybrid_cli(tmp_path, i):
    fx = ENUM[i]
    r = run([os.path.join(LIB, "gpu_hybrid"), write_task(tmp_path, fx), str(fx["max_depth"]), "32"])
    assert r.returncode == (0 if fx["optimal_depth"] is not None else 1), r.stderr
    if fx["optimal_depth"] is None:
        return
    m = re.search(r"Optimal solution length: (\d+) instructions \(kernel depth (\d+)\)", r.stdout)
    assert int(m.group(2)) == fx["optimal_depth"]
    verdicts = re.findall(r"cpu_verify=(\d+)/(\d+) (OK|FAIL)", r.stdout)
    assert verdicts and all(v[2] == "OK" and v[0] == v[1] for v in verdicts)
    assert len(verdicts) <= 32

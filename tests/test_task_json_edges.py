"""Task JSON edge cases through task_load, against the reference's own
libpca.so built from its sources (oracle/_ref, present where the reference
tree is; skipped elsewhere): the return code and every byte of the loaded
task_spec_t agree on empty, oversized, out-of-range, malformed and
reordered inputs."""
import ctypes
import json
import os

import pytest

from conftest import REPO
from pca_gb300.pcalib import PCALib, TaskSpec

REF_LIB = os.path.join(REPO, "oracle", "_ref", "libpca.so")

CASES = {
    "plain": {"name": "t", "input_ports": [0], "output_ports": [0],
              "tests": [{"in": [1], "out": [2]}, {"in": [3], "out": [4]}]},
    "two_inputs": {"name": "two", "max_cycles": 50, "input_ports": [0, 1], "output_ports": [0],
                   "tests": [{"in": [1, 2], "out": [3]}]},
    "no_tests": {"name": "empty", "input_ports": [0], "output_ports": [0], "tests": []},
    "forty_tests": {"name": "big", "input_ports": [0], "output_ports": [0],
                    "tests": [{"in": [i], "out": [2 * i]} for i in range(40)]},
    "wide_values": {"name": "wide", "input_ports": [0], "output_ports": [0],
                    "tests": [{"in": [65536 + 5], "out": [70000]}, {"in": [65535], "out": [0]}]},
    "negative_values": {"name": "neg", "input_ports": [0], "output_ports": [0],
                        "tests": [{"in": [-1], "out": [-32768]}, {"in": [-2], "out": [2]}]},
    "keys_reordered": {"tests": [{"out": [9], "in": [8]}], "output_ports": [0],
                       "input_ports": [0], "name": "reord", "max_cycles": 7},
    "long_name": {"name": "n" * 200, "input_ports": [0], "output_ports": [0],
                  "tests": [{"in": [1], "out": [1]}]},
    "extra_keys": {"name": "x", "comment": "ignored", "input_ports": [0], "output_ports": [0],
                   "tests": [{"in": [1], "out": [1], "note": 3}]},
}
RAW = {
    "not_json": "this is not json",
    "empty_file": "",
    "truncated": '{"name": "t", "input_ports": [0], "output_ports": [0], "tests": [{"in": [1], ',
}


@pytest.fixture(scope="module")
def ref_lib():
    if not os.path.exists(REF_LIB):
        pytest.skip("the reference's libpca.so is not built here")
    lib = ctypes.CDLL(REF_LIB)
    lib.task_load.argtypes = [ctypes.c_char_p, ctypes.POINTER(TaskSpec)]
    lib.task_load.restype = ctypes.c_int
    return lib


def _load_both(ref_lib, path):
    mine = PCALib().lib
    a, b = TaskSpec(), TaskSpec()
    ctypes.memset(ctypes.byref(a), 0, ctypes.sizeof(a))
    ctypes.memset(ctypes.byref(b), 0, ctypes.sizeof(b))
    ra = mine.task_load(str(path).encode(), ctypes.byref(a))
    rb = ref_lib.task_load(str(path).encode(), ctypes.byref(b))
    return ra, rb, bytes(a), bytes(b)


@pytest.mark.parametrize("name", sorted(CASES))
def test_task_load_matches_reference(ref_lib, tmp_path, name):
    p = tmp_path / f"{name}.json"
    p.write_text(json.dumps(CASES[name], indent=2))
    ra, rb, a, b = _load_both(ref_lib, p)
    assert ra == rb
    if ra == 0:
        assert a == b


@pytest.mark.parametrize("name", sorted(RAW))
def test_malformed_files_fail_alike(ref_lib, tmp_path, name):
    p = tmp_path / f"{name}.json"
    p.write_text(RAW[name])
    ra, rb, a, b = _load_both(ref_lib, p)
    assert ra == rb
    if ra == 0:
        assert a == b


def test_missing_file_fails_alike(ref_lib, tmp_path):
    ra, rb, _, _ = _load_both(ref_lib, tmp_path / "absent.json")
    assert ra == rb != 0

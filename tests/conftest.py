"""Shared test setup: the `gpu` marker, the native builds, golden fixtures.

Tests marked `gpu` need a CUDA device and call the engine through the C ABI
(libpcagb.so); the others run on the CPU: the oracle against the golden
fixtures, the host-side ABI functions, and the library's exported symbols.
"""
import json
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)
GOLDEN = os.path.join(REPO, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session", autouse=True)
def native_builds():
    from pca_gb300.build import build_engine
    from oracle.build import build_oracle
    build_engine()
    build_oracle()


def load_golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def spec_from_json(d):
    from pca_gb300.pcalib import TaskSpec
    s = TaskSpec()
    s.name = d["name"].encode()[:63]
    s.max_cycles = d["max_cycles"]
    s.num_inputs = len(d["input_ports"])
    for i, p in enumerate(d["input_ports"]):
        s.input_ports[i] = p
    s.num_outputs = len(d["output_ports"])
    for i, p in enumerate(d["output_ports"]):
        s.output_ports[i] = p
    for t, tc in enumerate(d["tests"][:32]):
        for i, v in enumerate(tc["in"]):
            s.tests[t].inputs[i] = v & 0xFFFF
        for i, v in enumerate(tc["out"]):
            s.tests[t].outputs[i] = v & 0xFFFF
    s.num_tests = min(len(d["tests"]), 32)
    return s


@pytest.fixture(scope="session")
def engine():
    from pca_gb300.pcalib import Engine
    e = Engine(0, 48 << 30)
    yield e
    e.close()

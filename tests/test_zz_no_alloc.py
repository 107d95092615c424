"""pcagb_solve_small_noalloc: the solve for callers that cannot call
cudaMalloc (their device memory belongs to another allocator, or they must
not risk an allocation's synchronisation). It keeps its scratch in a static
device array instead of an engine's arena.

Called through the C ABI and checked against pcagb_solve with split depth 0
(the same full canonical program set, compared exactly as sorted lists) on
two calls in a row and on interleaved tasks, so leftovers in the shared
scratch would show; sizes beyond its limit are rejected; a repeated call
changes the device's free memory by nothing. This file sorts last so a run
that stops at the first failure has run every other test first."""
import ctypes

import pytest

from conftest import load_golden, spec_from_json
from pca_gb300 import taskgen
from pca_gb300.pcalib import Engine, load_library

pytestmark = pytest.mark.gpu

CAP = 1 << 15


def noalloc(lib, task, max_depth):
    progs = (ctypes.c_uint16 * (16 * CAP))()
    lens = (ctypes.c_int * CAP)()
    opt = ctypes.c_int(-9)
    total = ctypes.c_uint64(0)
    rc = lib.pcagb_solve_small_noalloc(ctypes.byref(task), max_depth, None, ctypes.byref(opt),
                                       ctypes.byref(total), progs, lens, CAP)
    if rc < 0:
        raise RuntimeError(lib.pcagb_noalloc_last_error().decode())
    n = min(total.value, CAP)
    return rc, opt.value, total.value, sorted([progs[i * 16 + j] for j in range(lens[i])]
                                              for i in range(n))


def cases():
    enum = load_golden("ref_enumerate.json")
    out = [("negate16", taskgen.negate_task(1), 3)]
    picked = {1: 0, 2: 0, 3: 0}
    for fx in enum:
        k = fx["optimal_depth"]
        spec = spec_from_json(fx["task"])
        if k in picked and picked[k] < 2 and (k < 3 or spec.num_inputs == 1):
            picked[k] += 1
            out.append((fx["source"], spec, 3))
    out.append(("abs-none", spec_from_json(enum[4]["task"]), 2))
    return out


CASES = cases()


@pytest.fixture(scope="module")
def lib():
    return load_library()


@pytest.fixture(scope="module")
def expected():
    eng = Engine(0, 4 << 30)
    exp = {}
    for name, task, depth in CASES:
        s = eng.solve(task, max_depth=depth, split_depth=0, sol_cap=CAP)
        exp[name] = (s.optimal_depth, s.total_solutions, sorted(s.programs))
    eng.close()
    return exp


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_matches_pcagb_solve_on_two_calls(lib, expected, case):
    name, task, depth = case
    want = expected[name]
    for _ in range(2):
        rc, opt, total, progs = noalloc(lib, task, depth)
        assert rc == (1 if want[0] >= 0 else 0)
        assert (opt, total, progs) == want


def test_interleaved_tasks_leave_nothing_behind(lib, expected):
    order = [CASES[1], CASES[-1], CASES[1], CASES[3], CASES[0], CASES[3]]
    for name, task, depth in order:
        _, opt, total, progs = noalloc(lib, task, depth)
        assert (opt, total, progs) == expected[name]


def test_rejects_depth_beyond_limit(lib):
    task = taskgen.negate_task(1)
    opt = ctypes.c_int(0)
    total = ctypes.c_uint64(0)
    rc = lib.pcagb_solve_small_noalloc(ctypes.byref(task), 4, None, ctypes.byref(opt),
                                       ctypes.byref(total), None, None, 0)
    assert rc == -1
    assert b"no-allocation limit" in lib.pcagb_noalloc_last_error()


def test_repeated_call_allocates_no_device_memory(lib):
    torch = pytest.importorskip("torch")
    name, task, depth = CASES[-2]
    noalloc(lib, task, depth)  # loads the kernels
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    noalloc(lib, task, depth)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0


FRESH_PROCESS = r"""
import ctypes, sys
sys.path.insert(0, sys.argv[1])
from pca_gb300 import taskgen
from pca_gb300.pcalib import device_memory, load_library
lib = load_library()

def call(task, depth):
    opt, total = ctypes.c_int(-9), ctypes.c_uint64(0)
    rc = lib.pcagb_solve_small_noalloc(ctypes.byref(task), depth, None, ctypes.byref(opt),
                                       ctypes.byref(total), None, None, 0)
    assert rc >= 0, lib.pcagb_noalloc_last_error().decode()
    return opt.value

assert call(taskgen.negate_task(1), 3) == 1       # first call: only the depth-1 kernel runs
free0, _ = device_memory(0, lib)
assert call(taskgen.is_power2_task(1), 3) == -1   # depths 1, 2 and 3 all run
free1, _ = device_memory(0, lib)
print(free0, free1)
"""


def test_first_shallow_call_then_deeper_call_allocates_nothing():
    """In a fresh process whose first call is decided at kernel depth 1, a
    later call that runs the depth-2 and depth-3 kernels for the first time
    still takes no device memory: the set-up loaded every kernel."""
    import os
    import subprocess
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", FRESH_PROCESS, repo], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    free0, free1 = map(int, r.stdout.split()[-2:])
    assert free1 == free0

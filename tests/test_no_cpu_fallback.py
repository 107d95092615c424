"""No entry point falls back to the CPU: on a machine without a CUDA device
the engine refuses to start (PCAGB_ENODEV, with a message), the solver
command lines exit with an error, and the GPU-backed
search_exhaustive_complete returns that error instead of searching on the
host. Skipped where a device is present."""
import ctypes

import pytest

from pca_gb300 import taskgen
from pca_gb300.pcalib import Engine, EngineError, SearchCtx, SearchState, load_library

PCAGB_ENODEV = -5


@pytest.fixture(scope="module")
def lib():
    L = load_library()
    free, total = ctypes.c_size_t(0), ctypes.c_size_t(0)
    if L.pcagb_device_memory(0, ctypes.byref(free), ctypes.byref(total)) == 0:
        pytest.skip("a CUDA device is present")
    return L


def test_engine_refuses_without_a_device(lib):
    h = ctypes.c_void_p()
    assert lib.pcagb_engine_create(0, 0, ctypes.byref(h)) == PCAGB_ENODEV
    assert not h.value
    assert b"no CUDA device" in lib.pcagb_last_error()
    with pytest.raises(EngineError, match="no CUDA device"):
        Engine(0, 0, lib=lib)


def test_exhaustive_completion_does_not_search_on_the_host(lib):
    task = taskgen.negate_task(1)
    ctx, root = SearchCtx(), SearchState()
    assert lib.search_ctx_init(ctypes.byref(ctx), ctypes.byref(task)) == 0
    lib.search_state_init_root(ctypes.byref(ctx), ctypes.byref(root))
    insns = (ctypes.c_uint16 * 16)()
    n = ctypes.c_int(-1)
    rc = lib.search_exhaustive_complete(ctypes.byref(ctx), ctypes.byref(root), 3, insns,
                                        ctypes.byref(n))
    assert rc == PCAGB_ENODEV and n.value == 0
    assert lib.search_exhaustive_states_explored() == 0


def test_solver_command_lines_refuse_without_a_device(lib, tmp_path):
    import json
    import os
    import subprocess

    from conftest import REPO, load_golden
    fx = load_golden("ref_enumerate.json")[0]
    path = tmp_path / "task.json"
    path.write_text(json.dumps(fx["task"]))
    bindir = os.path.join(REPO, "pca_gb300", "_lib")
    for args in (["enumerate", str(path), "-d", "2"], ["gpu_hybrid", str(path), "2"]):
        r = subprocess.run([os.path.join(bindir, args[0])] + args[1:], capture_output=True,
                           text=True, timeout=60)
        assert r.returncode == 1 and "no CUDA device" in r.stderr, (args[0], r.stderr)
        assert "Optimal solution length" not in r.stdout

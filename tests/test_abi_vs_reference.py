"""The libpca half of libpcagb.so against the reference's own libpca.so built
from its sources (oracle/_ref; skipped where the reference tree is absent):
search_state_step on every one of the 65,536 instruction words from states
reached by random walks (legal or not, the written state byte for byte),
the two FNV-1a hashes and the leaf outputs of the states it produces, and
the branchless generator for all 128 liveness masks."""
import ctypes
import os
import random

import pytest

from conftest import REPO
from pca_gb300 import taskgen
from pca_gb300.pcalib import PCALib, SearchCtx, SearchState

REF_LIB = os.path.join(REPO, "oracle", "_ref", "libpca.so")


@pytest.fixture(scope="module")
def ref():
    if not os.path.exists(REF_LIB):
        pytest.skip("the reference's libpca.so is not built here")
    L = ctypes.CDLL(REF_LIB)
    P = ctypes.POINTER
    L.search_ctx_init.argtypes = [P(SearchCtx), ctypes.c_void_p]
    L.search_ctx_init.restype = ctypes.c_int
    L.search_state_init_root.argtypes = [P(SearchCtx), P(SearchState)]
    L.search_state_init_root.restype = None
    L.search_state_step.argtypes = [P(SearchCtx), P(SearchState), ctypes.c_uint16, P(SearchState)]
    L.search_state_step.restype = ctypes.c_int
    for name in ("search_state_oep_hash64", "search_state_key_hash64"):
        getattr(L, name).argtypes = [P(SearchCtx), P(SearchState)]
        getattr(L, name).restype = ctypes.c_uint64
    L.search_state_leaf_outputs.argtypes = [P(SearchCtx), P(SearchState)]
    L.search_state_leaf_outputs.restype = ctypes.c_uint8
    L.search_gen_candidates_branchless.argtypes = [P(ctypes.c_uint16), ctypes.c_int, P(SearchState)]
    L.search_gen_candidates_branchless.restype = ctypes.c_int
    return L


def _walk(lib, ctx, steps, rng):
    s = lib.init_root(ctx)
    for _ in range(steps):
        s = lib.step(ctx, s, rng.choice(lib.gen_candidates(s)))
    return s


@pytest.mark.parametrize("task_kind,steps", [("negate", 0), ("negate", 2), ("two_input", 1),
                                             ("two_input", 3)])
def test_step_on_every_instruction_word(ref, task_kind, steps):
    mine = PCALib()
    if task_kind == "negate":
        task = taskgen.negate_task(3)
    else:
        task, _ = taskgen.synthetic_task(50, 4)
    assert task_kind == "negate" or task.num_inputs == 2
    ctx = mine.init_ctx(task)
    s = _walk(mine, ctx, steps, random.Random(steps))
    a, b = SearchState(), SearchState()
    size = ctypes.sizeof(SearchState)
    legal = 0
    for insn in range(1 << 16):
        ctypes.memset(ctypes.byref(a), 0, size)
        ctypes.memset(ctypes.byref(b), 0, size)
        ra = mine.lib.search_state_step(ctypes.byref(ctx), ctypes.byref(s), insn, ctypes.byref(a))
        rb = ref.search_state_step(ctypes.byref(ctx), ctypes.byref(s), insn, ctypes.byref(b))
        assert ra == rb, hex(insn)
        if ra != 1:
            continue
        legal += 1
        assert bytes(a) == bytes(b), hex(insn)
        if insn % 61 == 0:
            for name in ("search_state_oep_hash64", "search_state_key_hash64",
                         "search_state_leaf_outputs"):
                assert getattr(mine.lib, name)(ctypes.byref(ctx), ctypes.byref(a)) == \
                    getattr(ref, name)(ctypes.byref(ctx), ctypes.byref(b)), (name, hex(insn))
    assert legal > 1000


def test_generator_for_every_liveness_mask(ref):
    mine = PCALib()
    s = SearchState()
    buf_a = (ctypes.c_uint16 * 4096)()
    buf_b = (ctypes.c_uint16 * 4096)()
    for m in range(128):
        s.live = m << 1
        na = mine.lib.search_gen_candidates_branchless(buf_a, 4096, ctypes.byref(s))
        nb = ref.search_gen_candidates_branchless(buf_b, 4096, ctypes.byref(s))
        assert na == nb and list(buf_a[:na]) == list(buf_b[:nb]), m
    # a short buffer: the count and the prefix written agree
    s.live = 0xFE
    na = mine.lib.search_gen_candidates_branchless(buf_a, 100, ctypes.byref(s))
    nb = ref.search_gen_candidates_branchless(buf_b, 100, ctypes.byref(s))
    assert na == nb and list(buf_a[:min(na, 100)]) == list(buf_b[:min(nb, 100)])


def test_disassembler_on_every_instruction_word(ref):
    mine = PCALib().lib
    ref.pca_disasm.argtypes = [ctypes.c_uint16, ctypes.c_char_p, ctypes.c_size_t]
    ref.pca_disasm.restype = None
    a = ctypes.create_string_buffer(96)
    b = ctypes.create_string_buffer(96)
    for insn in range(1 << 16):
        mine.pca_disasm(insn, a, 96)
        ref.pca_disasm(insn, b, 96)
        assert a.value == b.value, hex(insn)


def test_task_evaluate_on_random_programs(ref):
    from conftest import load_golden, spec_from_json
    mine = PCALib().lib
    ref.task_evaluate.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint16), ctypes.c_int]
    ref.task_evaluate.restype = ctypes.c_int
    rng = random.Random(7)
    specs = [spec_from_json(f["task"]) for f in load_golden("ref_enumerate.json")[:10]]
    for spec in specs:
        for _ in range(300):
            n = rng.randrange(1, 14)
            words = [rng.randrange(1 << 16) for _ in range(n)]
            prog = (ctypes.c_uint16 * n)(*words)
            ra = mine.task_evaluate(ctypes.byref(spec), prog, n)
            rb = ref.task_evaluate(ctypes.byref(spec), prog, n)
            assert ra == rb, (spec.name, [hex(w) for w in words])


def test_exports_cover_the_reference_library(ref):
    import shutil
    import subprocess
    from pca_gb300.pcalib import EXPORTS, load_library
    if not shutil.which("nm"):
        pytest.skip("nm is not installed")
    out = subprocess.run(["nm", "-D", "--defined-only", REF_LIB], capture_output=True, text=True,
                         check=True).stdout
    ref_funcs = {line.split()[-1] for line in out.splitlines() if " T " in line}
    lib = load_library()
    assert all(hasattr(lib, name) for name in ref_funcs - {"pca_assemble", "pca_dump"})
    # the two left out serve the reference's emulator command line only
    assert ref_funcs - set(EXPORTS) == {"pca_assemble", "pca_dump"}


def test_serialize_and_dump_of_walked_states(ref, tmp_path):
    mine = PCALib()
    libc = ctypes.CDLL(None)
    libc.fopen.restype = ctypes.c_void_p
    libc.fopen.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
    libc.fclose.argtypes = [ctypes.c_void_p]
    P = ctypes.POINTER
    rec_size = 576
    for lib in (mine.lib, ref):
        lib.search_state_serialize.argtypes = [P(SearchCtx), P(SearchState), ctypes.c_uint32,
                                               ctypes.c_uint16, ctypes.c_uint8, ctypes.c_uint8,
                                               ctypes.c_int8, ctypes.c_void_p]
        lib.search_state_serialize.restype = None
        lib.search_state_dump.argtypes = [P(SearchCtx), P(SearchState), ctypes.c_void_p]
        lib.search_state_dump.restype = None
    rng = random.Random(3)
    task, _ = taskgen.synthetic_task(1006, 4)
    ctx = mine.init_ctx(task)
    for walk in range(12):
        s = _walk(mine, ctx, walk % 5, rng)
        args = (rng.randrange(1 << 32), rng.randrange(1 << 16), rng.randrange(8), rng.randrange(2),
                rng.randrange(-1, 6))
        outs = []
        for lib in (mine.lib, ref):
            buf = ctypes.create_string_buffer(rec_size)
            lib.search_state_serialize(ctypes.byref(ctx), ctypes.byref(s), *args, buf)
            outs.append(buf.raw)
        assert outs[0] == outs[1], walk
        texts = []
        for k, lib in enumerate((mine.lib, ref)):
            path = str(tmp_path / f"dump{k}.txt").encode()
            fp = libc.fopen(path, b"w")
            lib.search_state_dump(ctypes.byref(ctx), ctypes.byref(s), fp)
            libc.fclose(fp)
            texts.append(open(path, "rb").read())
        assert texts[0] == texts[1] and texts[0], walk


def _stdout_of(fn):
    """What fn() writes to the process's file descriptor 1."""
    import os
    import tempfile
    libc = ctypes.CDLL(None)
    libc.fflush(None)
    with tempfile.TemporaryFile() as f:
        saved = os.dup(1)
        os.dup2(f.fileno(), 1)
        try:
            fn()
            libc.fflush(None)
        finally:
            os.dup2(saved, 1)
            os.close(saved)
        f.seek(0)
        return f.read()


def test_printed_task_and_program_listing(ref):
    from conftest import load_golden, spec_from_json
    mine = PCALib().lib
    ref.task_print.argtypes = [ctypes.c_void_p]
    ref.pca_disasm_prog.argtypes = [ctypes.POINTER(ctypes.c_uint16), ctypes.c_int]
    rng = random.Random(5)
    for f in load_golden("ref_enumerate.json")[:8]:
        spec = spec_from_json(f["task"])
        a = _stdout_of(lambda: mine.task_print(ctypes.byref(spec)))
        b = _stdout_of(lambda: ref.task_print(ctypes.byref(spec)))
        assert a == b and a
        words = [rng.randrange(1 << 16) for _ in range(rng.randrange(1, 20))]
        prog = (ctypes.c_uint16 * len(words))(*words)
        a = _stdout_of(lambda: mine.pca_disasm_prog(prog, len(words)))
        b = _stdout_of(lambda: ref.pca_disasm_prog(prog, len(words)))
        assert a == b and a


def test_vm_runs_random_programs_alike(ref):
    mine = PCALib().lib
    for lib in (mine, ref):
        lib.pca_init.argtypes = [ctypes.c_void_p]
        lib.pca_load.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint16), ctypes.c_size_t]
        lib.pca_step.argtypes = [ctypes.c_void_p]
        lib.pca_run.argtypes = [ctypes.c_void_p, ctypes.c_uint64]
        lib.pca_run.restype = ctypes.c_int
    rng = random.Random(11)
    size = 8192   # larger than pca_vm_t; the tail stays zero in both
    for _ in range(400):
        words = [rng.randrange(1 << 16) for _ in range(rng.randrange(1, 40))]
        prog = (ctypes.c_uint16 * len(words))(*words)
        max_cycles = rng.randrange(1, 300)
        vms = []
        for lib in (mine, ref):
            vm = ctypes.create_string_buffer(size)
            lib.pca_init(vm)
            lib.pca_load(vm, prog, len(words))
            lib.pca_step(vm)
            rc = lib.pca_run(vm, max_cycles)
            vms.append((rc, vm.raw))
        assert vms[0] == vms[1], [hex(w) for w in words]

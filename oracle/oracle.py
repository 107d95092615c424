"""ctypes bindings of the CPU oracle (oracle/_build/liborc.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, as the checker. The struct layouts are the
reference's (tasks/spec.h:20-34, src/search_state.h:20-35), identical to the
product's, so the same ctypes structures serve both.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liborc.so")

MAX_TESTS = 32
MAXD = 17


class OrcResult(ctypes.Structure):
    _fields_ = [("optimal_depth", ctypes.c_int),
                ("tried", ctypes.c_uint64 * MAXD),
                ("pruned_cum", ctypes.c_uint64 * MAXD),
                ("sols_at", ctypes.c_int * MAXD),
                ("survivors", ctypes.c_uint64 * MAXD),
                ("children", ctypes.c_uint64 * MAXD),
                ("num_solutions", ctypes.c_int),
                ("total_solutions", ctypes.c_uint64),
                ("false_prunes", ctypes.c_uint64),
                ("missed_prunes", ctypes.c_uint64)]


NONE, REF32, EXACT, EXACT_LIVE, REF32_AUDIT = 0, 1, 2, 3, 4

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            from oracle.build import build_oracle  # noqa: WPS433 (lazy build)
            build_oracle()
        from pca_gb300.pcalib import TaskSpec, SearchCtx, SearchState
        L = ctypes.CDLL(LIB)
        P = ctypes.POINTER
        L.orc_enumerate.argtypes = [P(TaskSpec), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    P(ctypes.c_uint16), P(ctypes.c_int), P(OrcResult)]
        L.orc_enumerate.restype = ctypes.c_int
        L.orc_enumerate_split.argtypes = [P(TaskSpec), ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, P(ctypes.c_uint16),
                                          P(ctypes.c_int), P(OrcResult)]
        L.orc_enumerate_split.restype = ctypes.c_int
        L.orc_enumerate_branch.argtypes = [P(TaskSpec), ctypes.c_int, ctypes.c_int,
                                           P(ctypes.c_uint16), P(ctypes.c_int), P(OrcResult)]
        L.orc_enumerate_branch.restype = ctypes.c_int
        L.orc_enumerate_sample.argtypes = [P(TaskSpec), ctypes.c_int, ctypes.c_int,
                                           ctypes.c_double, P(ctypes.c_double), P(ctypes.c_uint64)]
        L.orc_enumerate_sample.restype = ctypes.c_uint64
        L.orc_task_load.argtypes = [ctypes.c_char_p, P(TaskSpec)]
        L.orc_task_evaluate.argtypes = [P(TaskSpec), P(ctypes.c_uint16), ctypes.c_int]
        L.orc_ctx_init.argtypes = [P(SearchCtx), P(TaskSpec)]
        L.orc_init_root.argtypes = [P(SearchCtx), P(SearchState)]
        L.orc_init_root.restype = None
        L.orc_step.argtypes = [P(SearchCtx), P(SearchState), ctypes.c_uint16, P(SearchState)]
        L.orc_oep_hash64.argtypes = [P(SearchCtx), P(SearchState)]
        L.orc_oep_hash64.restype = ctypes.c_uint64
        L.orc_key_hash64.argtypes = [P(SearchCtx), P(SearchState)]
        L.orc_key_hash64.restype = ctypes.c_uint64
        L.orc_leaf_outputs.argtypes = [P(SearchCtx), P(SearchState)]
        L.orc_leaf_outputs.restype = ctypes.c_uint8
        L.orc_gen_candidates.argtypes = [P(ctypes.c_uint16), ctypes.c_int, ctypes.c_uint8]
        L.orc_exhaustive_complete.argtypes = [P(SearchCtx), P(SearchState), ctypes.c_int,
                                              P(ctypes.c_uint16), P(ctypes.c_int),
                                              P(ctypes.c_uint64)]
        _lib = L
    return _lib


def enumerate_task(task, max_depth: int, mode: int = REF32, sol_cap: int = -1):
    """Iterative deepening of the reference's branchless enumerator.

    sol_cap < 0 reproduces the reference's cap of 100 programs and its early
    stop; sol_cap >= 0 traverses the optimal depth fully and stores up to
    sol_cap programs. Returns (OrcResult, [programs])."""
    L = lib()
    n = 100 if sol_cap < 0 else max(sol_cap, 1)
    progs = (ctypes.c_uint16 * (16 * n))()
    lens = (ctypes.c_int * n)()
    r = OrcResult()
    if L.orc_enumerate(ctypes.byref(task), max_depth, mode, sol_cap, progs, lens,
                       ctypes.byref(r)) != 0:
        raise RuntimeError("oracle rejected the task")
    out = [[progs[i * 16 + j] for j in range(lens[i])] for i in range(r.num_solutions)]
    return r, out


def enumerate_split(task, max_depth: int, split: int, mode: int = EXACT_LIVE,
                    threads: int = 0, sol_cap: int = 1 << 16):
    """Level-synchronous form of the IDDFS (oracle_levels.c): positions
    1..min(K-1, split) deduplicated under `mode`, the rest enumerated without
    pruning; every solving program at the first K with one is counted and the
    first sol_cap are returned in depth-first order. threads = 0: every host
    core. Returns (OrcResult, [programs])."""
    L = lib()
    n = max(sol_cap, 1)
    progs = (ctypes.c_uint16 * (16 * n))()
    lens = (ctypes.c_int * n)()
    r = OrcResult()
    nthreads = threads or (os.cpu_count() or 1)
    if L.orc_enumerate_split(ctypes.byref(task), max_depth, split, mode, nthreads, sol_cap,
                             progs, lens, ctypes.byref(r)) != 0:
        raise RuntimeError("oracle rejected the task or ran out of host memory")
    out = [[progs[i * 16 + j] for j in range(lens[i])] for i in range(r.num_solutions)]
    return r, out


def enumerate_branch(task, max_depth: int, mode: int = REF32):
    """Iterative deepening of the reference's branch mode (CMP, forward BR,
    DIV, MOD) with its walk stopping at the 100th solution; mode REF32 (the
    reference's 32-bit pruner) or EXACT. Returns (OrcResult, [programs])."""
    L = lib()
    progs = (ctypes.c_uint16 * (16 * 100))()
    lens = (ctypes.c_int * 100)()
    r = OrcResult()
    if L.orc_enumerate_branch(ctypes.byref(task), max_depth, mode, progs, lens,
                              ctypes.byref(r)) != 0:
        raise RuntimeError("oracle rejected the task")
    out = [[progs[i * 16 + j] for j in range(lens[i])] for i in range(r.num_solutions)]
    return r, out


def sample_throughput(task, depth: int, nthreads: int, budget_s: float):
    """Reference-algorithm candidates counted over a time-bounded sample;
    returns (candidates, seconds, solutions)."""
    secs = ctypes.c_double(0)
    sols = ctypes.c_uint64(0)
    n = lib().orc_enumerate_sample(ctypes.byref(task), depth, nthreads, budget_s,
                                   ctypes.byref(secs), ctypes.byref(sols))
    return n, secs.value, sols.value


def exhaustive_complete(ctx, state, max_depth: int):
    insns = (ctypes.c_uint16 * 16)()
    n = ctypes.c_int(0)
    explored = ctypes.c_uint64(0)
    found = lib().orc_exhaustive_complete(ctypes.byref(ctx), ctypes.byref(state), max_depth,
                                          insns, ctypes.byref(n), ctypes.byref(explored))
    return bool(found), n.value, [insns[i] for i in range(n.value)], explored.value


def gen_candidates(live: int):
    buf = (ctypes.c_uint16 * 4096)()
    n = lib().orc_gen_candidates(buf, 4096, live)
    return [buf[i] for i in range(n)]

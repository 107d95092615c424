"""ctypes mirror of libpcagb.so.

`PCALib` has the reference's interface (python/search_eval.py:74-185): same
struct layouts (python/search_eval.py:32-69), same method names, same
return conventions, so reference-style callers switch by changing the
library path. `Engine` wraps the GPU solver entry points (pcagb_*).

The library must have been built (python -m pca_gb300.build); nothing here
falls back to a CPU implementation.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

MAX_TESTS = 32
PCA_NUM_REGS = 8
MAX_IO_PORTS = 8
MAX_CANDIDATES = 4096
MAXD = 17

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libpcagb.so")


class TestCase(ctypes.Structure):
    _fields_ = [("inputs", ctypes.c_uint16 * MAX_IO_PORTS),
                ("outputs", ctypes.c_uint16 * MAX_IO_PORTS)]


class TaskSpec(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 64),
                ("max_cycles", ctypes.c_uint64),
                ("input_ports", ctypes.c_uint8 * MAX_IO_PORTS),
                ("num_inputs", ctypes.c_int),
                ("output_ports", ctypes.c_uint8 * MAX_IO_PORTS),
                ("num_outputs", ctypes.c_int),
                ("tests", TestCase * MAX_TESTS),
                ("num_tests", ctypes.c_int)]


class SearchCtx(ctypes.Structure):
    _fields_ = [("task", TaskSpec),
                ("num_tests", ctypes.c_uint8),
                ("num_inputs", ctypes.c_uint8),
                ("num_outputs", ctypes.c_uint8),
                ("input_regs", ctypes.c_uint8 * MAX_IO_PORTS),
                ("output_port", ctypes.c_uint8)]


class SearchState(ctypes.Structure):
    _fields_ = [("regs", (ctypes.c_uint16 * PCA_NUM_REGS) * MAX_TESTS),
                ("flags", ctypes.c_uint8 * MAX_TESTS),
                ("live", ctypes.c_uint8),
                ("depth", ctypes.c_uint8)]


class SolveOpts(ctypes.Structure):
    _fields_ = [("max_depth", ctypes.c_int),
                ("min_depth", ctypes.c_int),
                ("split_depth", ctypes.c_int),
                ("oep_mode", ctypes.c_int),
                ("count_levels", ctypes.c_int),
                ("first_only", ctypes.c_int),
                ("first_tests", ctypes.c_int),
                ("suffix_chunk", ctypes.c_int),
                ("stage_launch", ctypes.c_int),
                ("shared_gpu", ctypes.c_int),
                ("full_levels", ctypes.c_int),
                ("reserved", ctypes.c_int * 1)]


class SolveResult(ctypes.Structure):
    _fields_ = [("optimal_depth", ctypes.c_int),
                ("stored", ctypes.c_int),
                ("total_solutions", ctypes.c_uint64),
                ("candidates", ctypes.c_uint64 * MAXD),
                ("evaluations", ctypes.c_uint64 * MAXD),
                ("tried", ctypes.c_uint64 * MAXD),
                ("pruned_cum", ctypes.c_uint64 * MAXD),
                ("level_children", ctypes.c_uint64 * MAXD),
                ("level_survivors", ctypes.c_uint64 * MAXD),
                ("seconds", ctypes.c_double),
                ("gpu_ms_expand", ctypes.c_double),
                ("gpu_ms_suffix", ctypes.c_double),
                ("gpu_ms_insert", ctypes.c_double),
                ("kernel_launches", ctypes.c_uint64),
                ("insert_launches", ctypes.c_uint64),
                ("suffix_launches", ctypes.c_uint64),
                ("h2d_bytes", ctypes.c_uint64),
                ("d2h_bytes", ctypes.c_uint64),
                ("insert_children", ctypes.c_uint64),
                ("split_used", ctypes.c_int),
                ("reserved0", ctypes.c_int),
                ("prefixes_at_optimal", ctypes.c_uint64),
                ("prefixes_to_first", ctypes.c_uint64),
                ("ms_to_first", ctypes.c_double),
                ("evaluations_run", ctypes.c_uint64),
                ("gpu_ms_lanes", ctypes.c_double * MAXD)]


class Tuning(ctypes.Structure):
    _fields_ = [("t_eval_ms", ctypes.c_double * 4),
                ("t_child_ms", ctypes.c_double),
                ("t_build_fixed_ms", ctypes.c_double),
                ("dedup_ratio", ctypes.c_double),
                ("first_tests_ms", (ctypes.c_double * 4) * 4),
                ("first_tests_n", (ctypes.c_int * 4) * 4),
                ("chunk_ms", (ctypes.c_double * 4) * 4),
                ("chunk_n", (ctypes.c_int * 4) * 4),
                ("chunk_choices", (ctypes.c_uint32 * 4) * 4),
                ("launch_rt_ms", ctypes.c_double),
                ("t_child_lean_ms", ctypes.c_double)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int),
                ("pool_bytes", ctypes.c_size_t),
                ("arena_bytes", ctypes.c_size_t),
                ("workers", ctypes.c_int),
                ("max_batch", ctypes.c_int),
                ("sol_cap", ctypes.c_int),
                ("opts", SolveOpts)]


class ServerStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "queued", "running_solves", "max_running_solves", "admitted", "finished", "batches",
        "pool_bytes", "pool_used", "pool_peak", "pool_largest_free")]


class LevelView(ctypes.Structure):
    _fields_ = [("regs", ctypes.c_void_p), ("flags", ctypes.c_void_p), ("live", ctypes.c_void_p),
                ("task", ctypes.c_void_p), ("n", ctypes.c_uint64), ("tp", ctypes.c_int),
                ("depth", ctypes.c_int), ("target_depth", ctypes.c_int), ("ntasks", ctypes.c_int),
                ("task_io", ctypes.c_void_p), ("task_T", ctypes.c_void_p),
                ("stream", ctypes.c_void_p), ("est_stage_ms", ctypes.c_double)]


ORDER_CB = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.POINTER(LevelView), ctypes.c_void_p)


class RecordStats(ctypes.Structure):
    _fields_ = [("optimal_depth", ctypes.c_int), ("optimal_states", ctypes.c_int),
                ("states_written", ctypes.c_uint64), ("positives", ctypes.c_uint64),
                ("negatives", ctypes.c_uint64), ("edges_written", ctypes.c_uint64),
                ("visited", ctypes.c_uint64)]


OEP_NONE, OEP_EXACT, OEP_EXACT_LIVE = 0, 1, 2

DONE_CB = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.POINTER(SolveResult), ctypes.c_void_p)

# every function declared in include/pca_gb300.h
EXPORTS = [
    "pca_init", "pca_load", "pca_step", "pca_run", "pca_disasm", "pca_disasm_prog",
    "task_load", "task_evaluate", "task_print",
    "search_ctx_init", "search_state_init_root", "search_state_step",
    "search_state_oep_hash64", "search_state_key_hash64", "search_state_leaf_outputs",
    "search_state_serialize", "search_gen_candidates_branchless",
    "search_exhaustive_complete", "search_exhaustive_states_explored", "search_state_dump",
    "pcagb_last_error", "pcagb_default_opts", "pcagb_engine_create", "pcagb_engine_destroy",
    "pcagb_solve", "pcagb_solve_batch", "pcagb_solve_batch_cb", "pcagb_solve_ordered",
    "pcagb_complete", "pcagb_record", "pcagb_solve_branch", "pcagb_solve_branch_ex",
    "pcagb_solve_branch_first", "pcagb_branch_last_error",
    "pcagb_num_candidates",
    "pcagb_engine_stream", "pcagb_tuning", "pcagb_device_memory",
    "pcagb_server_default_config", "pcagb_server_create", "pcagb_server_submit",
    "pcagb_server_next", "pcagb_server_collect", "pcagb_server_stats", "pcagb_server_destroy",
    "pcagb_server_last_error",
    "pcagb_solve_small_noalloc", "pcagb_noalloc_last_error",
]


def load_library(path: str = LIB_PATH) -> ctypes.CDLL:
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with `python -m pca_gb300.build`")
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER
    sig = {
        "task_load": ([ctypes.c_char_p, P(TaskSpec)], ctypes.c_int),
        "task_evaluate": ([P(TaskSpec), P(ctypes.c_uint16), ctypes.c_int], ctypes.c_int),
        "search_ctx_init": ([P(SearchCtx), P(TaskSpec)], ctypes.c_int),
        "search_state_init_root": ([P(SearchCtx), P(SearchState)], None),
        "search_state_step": ([P(SearchCtx), P(SearchState), ctypes.c_uint16, P(SearchState)],
                              ctypes.c_int),
        "search_state_oep_hash64": ([P(SearchCtx), P(SearchState)], ctypes.c_uint64),
        "search_state_key_hash64": ([P(SearchCtx), P(SearchState)], ctypes.c_uint64),
        "search_state_leaf_outputs": ([P(SearchCtx), P(SearchState)], ctypes.c_uint8),
        "search_gen_candidates_branchless": ([P(ctypes.c_uint16), ctypes.c_int, P(SearchState)],
                                             ctypes.c_int),
        "search_exhaustive_complete": ([P(SearchCtx), P(SearchState), ctypes.c_int,
                                        P(ctypes.c_uint16), P(ctypes.c_int)], ctypes.c_int),
        "search_exhaustive_states_explored": ([], ctypes.c_uint64),
        "pca_disasm": ([ctypes.c_uint16, ctypes.c_char_p, ctypes.c_size_t], None),
        "pcagb_last_error": ([], ctypes.c_char_p),
        "pcagb_default_opts": ([P(SolveOpts)], None),
        "pcagb_engine_create": ([ctypes.c_int, ctypes.c_size_t, P(ctypes.c_void_p)], ctypes.c_int),
        "pcagb_engine_destroy": ([ctypes.c_void_p], None),
        "pcagb_solve": ([ctypes.c_void_p, P(TaskSpec), P(SolveOpts), P(SolveResult),
                         P(ctypes.c_uint16), P(ctypes.c_int), ctypes.c_int], ctypes.c_int),
        "pcagb_solve_batch": ([ctypes.c_void_p, P(TaskSpec), ctypes.c_int, P(SolveOpts),
                               P(SolveResult), P(ctypes.c_uint16), P(ctypes.c_int), ctypes.c_int],
                              ctypes.c_int),
        "pcagb_solve_batch_cb": ([ctypes.c_void_p, P(TaskSpec), ctypes.c_int, P(SolveOpts),
                                  P(SolveResult), P(ctypes.c_uint16), P(ctypes.c_int),
                                  ctypes.c_int, DONE_CB, ctypes.c_void_p], ctypes.c_int),
        "pcagb_solve_ordered": ([ctypes.c_void_p, P(TaskSpec), P(SolveOpts), ORDER_CB,
                                 ctypes.c_void_p, ctypes.c_uint64, P(SolveResult),
                                 P(ctypes.c_uint16), P(ctypes.c_int), ctypes.c_int], ctypes.c_int),
        "pcagb_complete": ([ctypes.c_void_p, P(SearchCtx), P(SearchState), ctypes.c_int,
                            P(ctypes.c_uint16), P(ctypes.c_int), P(ctypes.c_uint64)], ctypes.c_int),
        "pcagb_record": ([ctypes.c_void_p, P(TaskSpec), ctypes.c_int, ctypes.c_uint32, ctypes.c_int,
                          ctypes.c_char_p, P(RecordStats)], ctypes.c_int),
        "pcagb_solve_branch": ([ctypes.c_void_p, P(TaskSpec), ctypes.c_int, P(SolveResult),
                                P(ctypes.c_uint16), P(ctypes.c_int), ctypes.c_int], ctypes.c_int),
        "pcagb_solve_branch_ex": ([ctypes.c_void_p, P(TaskSpec), ctypes.c_int, ctypes.c_uint64,
                                   P(SolveResult), P(ctypes.c_uint16), P(ctypes.c_int), ctypes.c_int],
                                  ctypes.c_int),
        "pcagb_solve_branch_first": ([ctypes.c_void_p, P(TaskSpec), ctypes.c_int, P(SolveResult),
                                      P(ctypes.c_uint16), P(ctypes.c_int), ctypes.c_int],
                                     ctypes.c_int),
        "pcagb_branch_last_error": ([], ctypes.c_char_p),
        "pcagb_num_candidates": ([ctypes.c_uint8], ctypes.c_int),
        "pcagb_engine_stream": ([ctypes.c_void_p], ctypes.c_void_p),
        "pcagb_tuning": ([ctypes.c_void_p, P(Tuning)], ctypes.c_int),
        "pcagb_device_memory": ([ctypes.c_int, P(ctypes.c_size_t), P(ctypes.c_size_t)],
                                ctypes.c_int),
        "pcagb_server_default_config": ([P(ServerConfig)], None),
        "pcagb_server_create": ([P(ServerConfig), P(ctypes.c_void_p)], ctypes.c_int),
        "pcagb_server_submit": ([ctypes.c_void_p, P(TaskSpec), ctypes.c_int, P(ctypes.c_uint64)],
                                ctypes.c_int),
        "pcagb_server_next": ([ctypes.c_void_p, ctypes.c_double, P(ctypes.c_uint64)],
                              ctypes.c_int),
        "pcagb_server_collect": ([ctypes.c_void_p, ctypes.c_uint64, P(SolveResult),
                                  P(ctypes.c_uint16), P(ctypes.c_int), ctypes.c_int,
                                  P(ctypes.c_double)], ctypes.c_int),
        "pcagb_server_stats": ([ctypes.c_void_p, P(ServerStats)], ctypes.c_int),
        "pcagb_server_destroy": ([ctypes.c_void_p], None),
        "pcagb_server_last_error": ([], ctypes.c_char_p),
        "pcagb_solve_small_noalloc": ([P(TaskSpec), ctypes.c_int, ctypes.c_void_p,
                                       P(ctypes.c_int), P(ctypes.c_uint64), P(ctypes.c_uint16),
                                       P(ctypes.c_int), ctypes.c_int], ctypes.c_int),
        "pcagb_noalloc_last_error": ([], ctypes.c_char_p),
    }
    for name, (args, res) in sig.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    return lib


class PCALib:
    """The reference's PCALib interface over libpcagb.so."""

    def __init__(self, lib_path: str = LIB_PATH):
        self.lib = load_library(lib_path)

    def load_task(self, path):
        spec = TaskSpec()
        if self.lib.task_load(path.encode(), ctypes.byref(spec)) != 0:
            raise RuntimeError(f"Failed to load task: {path}")
        return spec

    def init_ctx(self, spec):
        ctx = SearchCtx()
        if self.lib.search_ctx_init(ctypes.byref(ctx), ctypes.byref(spec)) != 0:
            raise RuntimeError("Failed to init search context")
        return ctx

    def init_root(self, ctx):
        root = SearchState()
        self.lib.search_state_init_root(ctypes.byref(ctx), ctypes.byref(root))
        return root

    def step(self, ctx, src, insn):
        dst = SearchState()
        ok = self.lib.search_state_step(ctypes.byref(ctx), ctypes.byref(src), insn,
                                        ctypes.byref(dst))
        return dst if ok else None

    def oep_hash(self, ctx, state):
        return self.lib.search_state_oep_hash64(ctypes.byref(ctx), ctypes.byref(state))

    def key_hash(self, ctx, state):
        return self.lib.search_state_key_hash64(ctypes.byref(ctx), ctypes.byref(state))

    def leaf_check(self, ctx, state):
        return self.lib.search_state_leaf_outputs(ctypes.byref(ctx), ctypes.byref(state))

    def gen_candidates(self, state):
        buf = (ctypes.c_uint16 * MAX_CANDIDATES)()
        n = self.lib.search_gen_candidates_branchless(buf, MAX_CANDIDATES, ctypes.byref(state))
        return [buf[i] for i in range(n)]

    def exhaustive_complete(self, ctx, state, max_depth):
        """IDDFS completion from state to max_depth on the GPU.
        Returns (found, sol_len, [insns])."""
        insns = (ctypes.c_uint16 * 16)()
        sol_len = ctypes.c_int(0)
        found = self.lib.search_exhaustive_complete(ctypes.byref(ctx), ctypes.byref(state),
                                                    max_depth, insns, ctypes.byref(sol_len))
        if found < 0:
            raise RuntimeError(self.lib.pcagb_last_error().decode())
        if found:
            return True, sol_len.value, [insns[i] for i in range(sol_len.value)]
        return False, 0, []

    def exhaustive_states_explored(self):
        return self.lib.search_exhaustive_states_explored()

    def evaluate(self, spec, prog):
        arr = (ctypes.c_uint16 * len(prog))(*prog)
        return self.lib.task_evaluate(ctypes.byref(spec), arr, len(prog))

    def disasm(self, insn):
        buf = ctypes.create_string_buffer(64)
        self.lib.pca_disasm(insn, buf, 64)
        return buf.value.decode()


def task_from_dict(d: dict) -> "TaskSpec":
    """A task spec from the task JSON's fields (tasks/spec.c:80-184: name,
    max_cycles, input_ports, output_ports, tests[{in, out}], values masked to
    16 bits, at most 32 tests)."""
    s = TaskSpec()
    s.name = str(d.get("name", "")).encode()[:63]
    s.max_cycles = int(d.get("max_cycles", 1000))
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


def make_task(name, inputs, outputs, max_cycles=100, input_ports=None) -> TaskSpec:
    """Build a TaskSpec from rows of input values and single outputs."""
    spec = TaskSpec()
    spec.name = name.encode()[:63]
    spec.max_cycles = max_cycles
    n_in = len(inputs[0]) if len(inputs) else 1
    ports = input_ports if input_ports is not None else list(range(n_in))
    spec.num_inputs = n_in
    for i, p in enumerate(ports):
        spec.input_ports[i] = p
    spec.num_outputs = 1
    spec.output_ports[0] = 0
    if len(inputs) > MAX_TESTS:
        raise ValueError("at most 32 tests")
    for t, (row, out) in enumerate(zip(inputs, outputs)):
        for i, v in enumerate(row):
            spec.tests[t].inputs[i] = int(v) & 0xFFFF
        spec.tests[t].outputs[0] = int(out) & 0xFFFF
    spec.num_tests = len(inputs)
    return spec


@dataclass
class Solution:
    optimal_depth: int
    programs: list = field(default_factory=list)
    total_solutions: int = 0
    candidates: list = field(default_factory=list)
    evaluations: list = field(default_factory=list)
    tried: list = field(default_factory=list)
    pruned_cum: list = field(default_factory=list)
    level_children: list = field(default_factory=list)
    level_survivors: list = field(default_factory=list)
    seconds: float = 0.0
    gpu_ms_expand: float = 0.0
    gpu_ms_suffix: float = 0.0
    gpu_ms_insert: float = 0.0
    kernel_launches: int = 0
    insert_launches: int = 0
    suffix_launches: int = 0
    h2d_bytes: int = 0
    d2h_bytes: int = 0
    insert_children: int = 0
    split_used: int = 0
    prefixes_at_optimal: int = 0
    prefixes_to_first: int = 0
    ms_to_first: float = 0.0
    evaluations_run: int = 0
    gpu_ms_lanes: list = field(default_factory=list)


class EngineError(RuntimeError):
    pass


RESULT_SCALARS = ("seconds", "gpu_ms_expand", "gpu_ms_suffix", "gpu_ms_insert", "kernel_launches",
                  "insert_launches", "suffix_launches", "h2d_bytes", "d2h_bytes",
                  "insert_children", "split_used", "prefixes_at_optimal", "prefixes_to_first",
                  "ms_to_first", "evaluations_run")
RESULT_ARRAYS = ("candidates", "evaluations", "tried", "pruned_cum", "level_children",
                 "level_survivors", "gpu_ms_lanes")


def solution_from_result(r: "SolveResult", progs, lens, base: int, max_depth: int) -> "Solution":
    """A Solution from a pcagb_result_t and its programs (progs[(base + k) *
    16 ...], lens[base + k] for k < r.stored)."""
    sol = Solution(optimal_depth=r.optimal_depth, total_solutions=r.total_solutions)
    for name in RESULT_SCALARS:
        setattr(sol, name, getattr(r, name))
    for k in range(r.stored):
        sol.programs.append([progs[(base + k) * 16 + j] for j in range(lens[base + k])])
    last = r.optimal_depth if r.optimal_depth >= 0 else max_depth
    for name in RESULT_ARRAYS:
        arr = getattr(r, name)
        setattr(sol, name, [arr[k] for k in range(min(last + 1, MAXD))])
    return sol


def device_memory(device: int = 0, lib: ctypes.CDLL | None = None):
    """(free, total) bytes of a CUDA device."""
    lib = lib or load_library()
    free, total = ctypes.c_size_t(0), ctypes.c_size_t(0)
    rc = lib.pcagb_device_memory(device, ctypes.byref(free), ctypes.byref(total))
    if rc != 0:
        raise EngineError(lib.pcagb_last_error().decode())
    return free.value, total.value


class Engine:
    """One GPU engine (device buffers in an HBM arena)."""

    def __init__(self, device: int = 0, hbm_budget_bytes: int = 0, lib: ctypes.CDLL | None = None):
        self.lib = lib or load_library()
        self.h = ctypes.c_void_p()
        rc = self.lib.pcagb_engine_create(device, hbm_budget_bytes, ctypes.byref(self.h))
        if rc != 0:
            raise EngineError(f"engine create failed ({rc}): {self.lib.pcagb_last_error().decode()}")

    def close(self):
        if self.h:
            self.lib.pcagb_engine_destroy(self.h)
            self.h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, task: TaskSpec, max_depth=4, oep_mode=OEP_EXACT_LIVE, split_depth=-1,
              count_levels=False, first_only=False, min_depth=0, sol_cap=4096, first_tests=0,
              suffix_chunk=0, stage_launch=0, full_levels=False) -> Solution:
        o = SolveOpts()
        self.lib.pcagb_default_opts(ctypes.byref(o))
        o.max_depth, o.min_depth, o.split_depth = max_depth, min_depth, split_depth
        o.oep_mode, o.count_levels, o.first_only = oep_mode, int(count_levels), int(first_only)
        o.first_tests, o.suffix_chunk, o.stage_launch = first_tests, suffix_chunk, stage_launch
        o.full_levels = int(full_levels)
        r = SolveResult()
        progs = (ctypes.c_uint16 * (16 * max(sol_cap, 1)))()
        lens = (ctypes.c_int * max(sol_cap, 1))()
        rc = self.lib.pcagb_solve(self.h, ctypes.byref(task), ctypes.byref(o), ctypes.byref(r),
                                  progs, lens, sol_cap)
        if rc != 0:
            raise EngineError(f"solve failed ({rc}): {self.lib.pcagb_last_error().decode()}")
        sol = Solution(optimal_depth=r.optimal_depth, total_solutions=r.total_solutions)
        for name in RESULT_SCALARS:
            setattr(sol, name, getattr(r, name))
        for i in range(r.stored):
            sol.programs.append([progs[i * 16 + j] for j in range(lens[i])])
        last = max(r.optimal_depth, max_depth if r.optimal_depth < 0 else r.optimal_depth)
        for name in RESULT_ARRAYS:
            arr = getattr(r, name)
            setattr(sol, name, [arr[k] for k in range(min(last + 1, MAXD))])
        return sol

    def tuning(self) -> dict:
        """The autotuner's measured costs and launch choices (pcagb_tuning)."""
        t = Tuning()
        if self.lib.pcagb_tuning(self.h, ctypes.byref(t)) != 0:
            raise EngineError(self.lib.pcagb_last_error().decode())
        grid = lambda a: [[a[i][j] for j in range(4)] for i in range(4)]  # noqa: E731
        return {"t_eval_ms": list(t.t_eval_ms), "t_child_ms": t.t_child_ms,
                "t_build_fixed_ms": t.t_build_fixed_ms, "dedup_ratio": t.dedup_ratio,
                "first_tests_ms": grid(t.first_tests_ms), "first_tests_n": grid(t.first_tests_n),
                "chunk_ms": grid(t.chunk_ms), "chunk_n": grid(t.chunk_n),
                "chunk_choices": grid(t.chunk_choices), "launch_rt_ms": t.launch_rt_ms,
                "t_child_lean_ms": t.t_child_lean_ms}

    def solve_batch(self, tasks, max_depth=4, oep_mode=OEP_EXACT_LIVE, split_depth=-1,
                    count_levels=False, sol_cap=64, on_done=None, first_only=False,
                    first_tests=0, suffix_chunk=0, shared_gpu=False, full_levels=False):
        """Solve many tasks in shared launches; returns one Solution per task
        (its `seconds` is that task's time-to-proven-optimal in the batch).
        on_done(i, Solution), if given, runs as soon as task i is decided.
        shared_gpu: other solves run on the GPU meanwhile (a server's slots),
        so this solve's times update none of the autotuner's costs."""
        n = len(tasks)
        arr = (TaskSpec * n)(*tasks)
        o = SolveOpts()
        self.lib.pcagb_default_opts(ctypes.byref(o))
        o.max_depth, o.split_depth, o.oep_mode = max_depth, split_depth, oep_mode
        o.count_levels, o.first_only = int(count_levels), int(first_only)
        o.first_tests, o.suffix_chunk = first_tests, suffix_chunk
        o.shared_gpu = int(shared_gpu)
        o.full_levels = int(full_levels)
        res = (SolveResult * n)()
        cap = max(sol_cap, 1)
        progs = (ctypes.c_uint16 * (16 * cap * n))()
        lens = (ctypes.c_int * (cap * n))()

        def convert(i, r):
            sol = Solution(optimal_depth=r.optimal_depth, total_solutions=r.total_solutions)
            for name in RESULT_SCALARS:
                setattr(sol, name, getattr(r, name))
            base = i * cap
            for k in range(r.stored):
                sol.programs.append([progs[(base + k) * 16 + j] for j in range(lens[base + k])])
            last = r.optimal_depth if r.optimal_depth >= 0 else max_depth
            for name in RESULT_ARRAYS:
                arr2 = getattr(r, name)
                setattr(sol, name, [arr2[k] for k in range(min(last + 1, MAXD))])
            return sol

        errors = []
        if on_done is None:
            rc = self.lib.pcagb_solve_batch(self.h, arr, n, ctypes.byref(o), res, progs, lens, cap)
        else:
            def done(i, rp, _user):
                # ctypes would print and drop an exception raised here: keep
                # the first one and raise it once the batch returns
                try:
                    on_done(i, convert(i, rp.contents))
                except BaseException as exc:  # noqa: BLE001 - re-raised after the batch
                    errors.append(exc)

            cb = DONE_CB(done)
            rc = self.lib.pcagb_solve_batch_cb(self.h, arr, n, ctypes.byref(o), res, progs, lens,
                                               cap, cb, None)
        if errors:
            raise errors[0]
        if rc != 0:
            raise EngineError(f"batch solve failed ({rc}): {self.lib.pcagb_last_error().decode()}")
        return [convert(i, res[i]) for i in range(n)]

    def solve_ordered(self, task: TaskSpec, order_fn, chunk=4096, max_depth=4,
                      oep_mode=OEP_EXACT_LIVE, split_depth=-1, sol_cap=256) -> Solution:
        """Solve with the suffix stages visiting the split level's prefixes in
        the order order_fn(view) returns (a device tensor of uint32/int32
        prefix indices, or None for DFS order), `chunk` prefixes in the first
        launch of a stage and twice as many in each next one, stopping at the
        first launch of the optimal depth with a solution. An order_fn with a
        new_solve() method has it called before the solve starts."""
        o = SolveOpts()
        self.lib.pcagb_default_opts(ctypes.byref(o))
        o.max_depth, o.split_depth, o.oep_mode = max_depth, split_depth, oep_mode
        keep, errors = [], []
        # an order object that keeps per-level state (ValueOrder's scored
        # levels, keyed by device address) starts every solve afresh: a new
        # solve's level can sit at a freed level's address
        new_solve = getattr(order_fn, "new_solve", None)
        if new_solve is not None:
            new_solve()

        def cb(vp, _user):
            # An exception must not cross the C boundary (ctypes would hand
            # the engine an undefined pointer): record it, visit this stage in
            # DFS order, and raise once the solve returns.
            try:
                view = vp.contents
                out = order_fn(view)
                if out is None:
                    return None
                import torch
                if (not isinstance(out, torch.Tensor) or not out.is_cuda or out.dim() != 1
                        or out.numel() != view.n or out.element_size() != 4
                        or out.dtype.is_floating_point or not out.is_contiguous()):
                    raise EngineError("order callback must return None or a contiguous 1-D "
                                      f"int32 CUDA tensor of {view.n} prefix indices")
                keep.append(out)
                return out.data_ptr()
            except BaseException as exc:  # noqa: BLE001 - re-raised after the solve
                errors.append(exc)
                return None

        ccb = ORDER_CB(cb)
        r = SolveResult()
        progs = (ctypes.c_uint16 * (16 * max(sol_cap, 1)))()
        lens = (ctypes.c_int * max(sol_cap, 1))()
        rc = self.lib.pcagb_solve_ordered(self.h, ctypes.byref(task), ctypes.byref(o), ccb, None,
                                          chunk, ctypes.byref(r), progs, lens, sol_cap)
        if errors:
            raise errors[0]
        if rc != 0:
            raise EngineError(f"ordered solve failed ({rc}): {self.lib.pcagb_last_error().decode()}")
        sol = Solution(optimal_depth=r.optimal_depth, total_solutions=r.total_solutions)
        for name in RESULT_SCALARS:
            setattr(sol, name, getattr(r, name))
        for i in range(r.stored):
            sol.programs.append([progs[i * 16 + j] for j in range(lens[i])])
        sol.candidates = [r.candidates[k] for k in range(MAXD)]
        return sol

    @property
    def stream(self) -> int:
        """cudaStream_t of the engine, as an integer handle."""
        return self.lib.pcagb_engine_stream(self.h) or 0

    def solve_branch(self, task: TaskSpec, max_depth: int = 4, sol_cap: int = 100,
                     last_level_max_children: int | None = None,
                     first_only: bool = False) -> Solution:
        """Branch mode (CMP / forward BR / DIV / MOD): the reference solver's
        default search, with its per-depth counters and its first programs.
        last_level_max_children: above it a depth's last level is not built
        (None = the library's default). first_only: the reference hybrid
        solver's stopping rule (the optimal depth's search ends at the first
        launch with a solution; the same optimal depth and first programs)."""
        r = SolveResult()
        cap = max(sol_cap, 1)
        progs = (ctypes.c_uint16 * (16 * cap))()
        lens = (ctypes.c_int * cap)()
        if first_only:
            rc = self.lib.pcagb_solve_branch_first(self.h, ctypes.byref(task), max_depth,
                                                   ctypes.byref(r), progs, lens, cap)
        elif last_level_max_children is None:
            rc = self.lib.pcagb_solve_branch(self.h, ctypes.byref(task), max_depth,
                                             ctypes.byref(r), progs, lens, cap)
        else:
            rc = self.lib.pcagb_solve_branch_ex(self.h, ctypes.byref(task), max_depth,
                                                last_level_max_children, ctypes.byref(r), progs,
                                                lens, cap)
        if rc != 0:
            raise EngineError(f"branch solve failed ({rc}): "
                              f"{self.lib.pcagb_branch_last_error().decode()}")
        sol = Solution(optimal_depth=r.optimal_depth, total_solutions=r.total_solutions)
        sol.seconds = r.seconds
        for i in range(r.stored):
            sol.programs.append([progs[i * 16 + j] for j in range(lens[i])])
        last = r.optimal_depth if r.optimal_depth >= 0 else max_depth
        sol.tried = [r.tried[k] for k in range(last + 1)]
        sol.pruned_cum = [r.pruned_cum[k] for k in range(last + 1)]
        sol.split_used = r.split_used
        return sol

    def record(self, task: TaskSpec, out_dir: str, max_depth: int = 4, task_id: int = 0,
               neg_stride: int = 8) -> dict:
        """The reference's recording pass (`enumerate --record`) from the GPU
        levels: writes states_<id>.bin / edges_<id>.bin into out_dir and
        returns the counts ({} fields of pcagb_record_stats_t); nothing is
        written when no program of kernel depth <= max_depth exists."""
        st = RecordStats()
        rc = self.lib.pcagb_record(self.h, ctypes.byref(task), max_depth, task_id, neg_stride,
                                   os.fsencode(out_dir), ctypes.byref(st))
        if rc < 0:
            raise EngineError(f"record failed ({rc}): {self.lib.pcagb_last_error().decode()}")
        return {name: getattr(st, name) for name, _ in RecordStats._fields_}

    def complete(self, ctx: SearchCtx, state: SearchState, max_depth: int):
        insns = (ctypes.c_uint16 * 16)()
        n = ctypes.c_int(0)
        explored = ctypes.c_uint64(0)
        rc = self.lib.pcagb_complete(self.h, ctypes.byref(ctx), ctypes.byref(state), max_depth,
                                     insns, ctypes.byref(n), ctypes.byref(explored))
        if rc < 0:
            raise EngineError(f"complete failed ({rc}): {self.lib.pcagb_last_error().decode()}")
        return bool(rc), n.value, [insns[i] for i in range(n.value)], explored.value

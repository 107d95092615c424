"""Fixed small workloads, one per kernel family, for profiling under ncu.

    python profile_cases.py engine_depths   # k_suffix<32, 2/3>, k_leaf
    python profile_cases.py suffix_depth2   # one k_suffix<32, 2> depth-4 stage
    python profile_cases.py noalloc         # k_suffix_noalloc
    python profile_cases.py valuenet        # training and scoring kernels
    python profile_cases.py orders          # k_check_perm
    python profile_cases.py branch          # branch-mode kernels
    python profile_cases.py branch_saturating_add   # the same, two inputs, depth 4
    python profile_cases.py misc            # leaf, mark-all, paths, recording, twins, sampling

Each case runs its work `--reps` times (default 2) and prints one timing line
per repetition (CUDA events); the device memory it holds stays below a few
GB so that a capture of any of its launches ends quickly. The headline solve
(bench.py) covers the level kernels and k_suffix<32, 1>.
"""
from __future__ import annotations

import argparse
import ctypes
import time

import numpy as np


def _events():
    import torch
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def case_engine_depths(reps: int):
    """is_power2 (32 tests) to kernel depth 4 with the suffix stage started
    from level 1 and level 2 (suffix depths 3 and 2), each with a warp per
    (prefix, chunk of 16 middles) and with a lane per innermost middle, and
    depth 3 from level 3 (the leaf check)."""
    from pca_gb300.pcalib import Engine
    from pca_gb300.taskgen import is_power2_task
    eng = Engine(0, 4 << 30)
    task = is_power2_task()
    for _ in range(reps):
        for split, depth, chunk in ((1, 4, 16), (1, 4, 1024), (2, 4, 16), (2, 4, 1024),
                                    (3, 3, 0)):
            t0 = time.perf_counter()
            s = eng.solve(task, max_depth=depth, split_depth=split, sol_cap=1,
                          count_levels=split == 3, suffix_chunk=chunk)
            print(f"engine_depths split={split} depth={depth} shape={chunk or 'auto'}: "
                  f"K*={s.optimal_depth} {time.perf_counter() - t0:.4f} s, "
                  f"suffix {s.gpu_ms_suffix:.3f} ms", flush=True)


def case_suffix_depth2(reps: int):
    """is_power2 (32 tests) to kernel depth 4 from level 2: the depth-4 stage
    is one k_suffix<32, 2> launch (the fourth k_suffix launch of a solve)."""
    from pca_gb300.pcalib import Engine
    from pca_gb300.taskgen import is_power2_task
    eng = Engine(0, 4 << 30)
    task = is_power2_task()
    for _ in range(reps):
        t0 = time.perf_counter()
        s = eng.solve(task, max_depth=4, split_depth=2, sol_cap=1, first_only=True)
        print(f"suffix_depth2: K*={s.optimal_depth} {time.perf_counter() - t0:.4f} s, "
              f"suffix {s.gpu_ms_suffix:.3f} ms", flush=True)


def case_noalloc(reps: int):
    """The no-allocation entry point to kernel depth 3 on is_power2 (32
    tests, no program that short: every depth searched completely) and on a
    2-input synthetic task (27 tests)."""
    from pca_gb300.pcalib import load_library
    from pca_gb300.taskgen import is_power2_task, synthetic_task
    lib = load_library()
    cap = 1 << 12
    progs = (ctypes.c_uint16 * (16 * cap))()
    lens = (ctypes.c_int * cap)()
    for _ in range(reps):
        for name, task in (("is_power2", is_power2_task()), ("synthetic_2in", synthetic_task(5, 6)[0])):
            opt, total = ctypes.c_int(-9), ctypes.c_uint64(0)
            t0 = time.perf_counter()
            rc = lib.pcagb_solve_small_noalloc(ctypes.byref(task), 3, None, ctypes.byref(opt),
                                               ctypes.byref(total), progs, lens, cap)
            if rc < 0:
                raise RuntimeError(lib.pcagb_noalloc_last_error().decode())
            print(f"noalloc {name}: K*={opt.value} programs={total.value} "
                  f"{time.perf_counter() - t0:.4f} s", flush=True)


def _random_states(n, TP, seed=0):
    import torch
    rng = np.random.default_rng(seed)
    dev = "cuda"
    Ts = np.array([16, 24, 32], dtype=np.int32) if TP == 32 else np.array([16], dtype=np.int32)
    task = rng.integers(0, len(Ts), size=n)
    regs = rng.integers(0, 1 << 16, size=(n, 8, TP), dtype=np.uint16)
    regs[:, 0, :] = 0
    flags = rng.integers(0, 16, size=(n, TP), dtype=np.uint8)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)  # noqa: E731
    return dict(regs=t(regs.astype(np.int16)), flags=t(flags),
                live=t((rng.integers(0, 256, size=n) & 0xFE).astype(np.uint8)),
                task=t(task.astype(np.int16)), depth=t(rng.integers(1, 4, size=n).astype(np.uint8)),
                task_io=t(rng.integers(0, 1 << 16, size=(len(Ts), 3, 32),
                                       dtype=np.uint16).astype(np.int16)),
                task_T=t(Ts), label=t((rng.random(n) < 0.1).astype(np.float32)),
                remaining=t(rng.integers(0, 4, size=n).astype(np.int32)), TP=TP)


def case_valuenet(reps: int):
    """Training steps on 8,192 states (features, BF16 GEMMs forward and
    backward, pooling, loss, Adam) and scoring of 131,072 states through the
    fused tcgen05 encoder and the trunk."""
    import torch
    from pca_gb300.valuenet import ValueNet
    net = ValueNet(seed=0, lr=1e-3, pos_weight=8.0)
    train = _random_states(8192, 32, seed=1)
    score = _random_states(131072, 32, seed=2)
    for _ in range(reps):
        e0, e1 = _events()
        e0.record()
        loss = net.train_step(train)
        e1.record()
        torch.cuda.synchronize()
        print(f"valuenet train step (8192 states): {e0.elapsed_time(e1):.3f} ms "
              f"loss {float(loss):.4f}", flush=True)
        e0, e1 = _events()
        e0.record()
        loss = net.train_step_graph(train)
        e1.record()
        torch.cuda.synchronize()
        print(f"valuenet train step, graph replay (8192 states): {e0.elapsed_time(e1):.3f} ms "
              f"loss {float(loss):.4f}", flush=True)
        e0, e1 = _events()
        e0.record()
        L = net.forward_fused(score["regs"], score["flags"], score["live"], score["task"],
                              score["depth"], 32, score["task_io"], score["task_T"])
        e1.record()
        torch.cuda.synchronize()
        net.check_status()
        print(f"valuenet score (131072 states): {e0.elapsed_time(e1):.3f} ms "
              f"mean logit {float(L[:, 0].mean()):.4f}", flush=True)


def case_orders(reps: int):
    """An ordered solve (random order) of is_power2 to depth 4 from level 2:
    every stage's order is checked on the device before use."""
    import torch
    from pca_gb300.pcalib import Engine
    from pca_gb300.taskgen import is_power2_task
    eng = Engine(0, 4 << 30)
    gen = torch.Generator().manual_seed(0)

    def order(view):
        return torch.randperm(view.n, generator=gen).to(torch.int32).cuda()

    for _ in range(reps):
        t0 = time.perf_counter()
        s = eng.solve_ordered(is_power2_task(), order, chunk=4096, max_depth=4, split_depth=2)
        print(f"orders: K*={s.optimal_depth} {time.perf_counter() - t0:.4f} s", flush=True)


def _branch_case(name: str, reps: int):
    import json
    import os
    from pca_gb300.pcalib import Engine, task_from_dict
    fx = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "tests",
                      "golden", "ref_published.json")
    spec = next(t for t in json.load(open(fx)) if t["name"] == name)
    task = task_from_dict(spec["task"])
    K = spec["published_length"] - task.num_inputs - 2
    eng = Engine(0, 1 << 30)
    for _ in range(reps):
        t0 = time.perf_counter()
        s = eng.solve_branch(task, max_depth=K)
        print(f"branch {name}: length {s.optimal_depth + task.num_inputs + 2} in "
              f"{time.perf_counter() - t0:.3f} s", flush=True)


def case_branch(reps: int):
    """Branch mode on the reference's is_power2 task file (11 tests) to its
    documented optimal length 7 (kernel depth 4): levels 1..3 built with the
    exact pruner, the last position searched without its level."""
    _branch_case("is_power2", reps)


def case_branch_saturating_add(reps: int):
    """Branch mode on the reference's saturating_add task file (two inputs,
    8 tests) to its documented optimal length 8 (kernel depth 4)."""
    _branch_case("saturating_add", reps)


def case_misc(reps: int):
    """The engine's smaller kernels on small cases: the leaf check of a
    built level (k_leaf, count mode), the unpruned level marking (k_mark_all,
    no OEP), solution paths (k_gather_paths), the recording pass
    (k_record_keys, k_record_states), the flag-twin pass (k_twins), the
    depth-1 evaluation count (k_count_evals), and a sampled value ranking
    (k_gather_sample, k_compose_order)."""
    import os
    import tempfile

    import torch
    from pca_gb300.guided import ValueOrder
    from pca_gb300.pcalib import Engine, OEP_EXACT, OEP_NONE
    from pca_gb300.taskgen import negate_task, synthetic_batch
    from pca_gb300.valuenet import ValueNet
    eng = Engine(0, 4 << 30)
    # tasks of the batched workload's generator whose optimum is at kernel
    # depth 3 (one input: the recording pass) and 4 (the ordered solve ranks
    # a sample of its level 2 or 3)
    pool = synthetic_batch(400, seed=41)
    sols = eng.solve_batch(pool, max_depth=4, sol_cap=1, first_only=True)
    t3 = next(t for t, s in zip(pool, sols) if s.optimal_depth == 3 and t.num_inputs == 1)
    t4 = next(t for t, s in zip(pool, sols) if s.optimal_depth == 4)
    net = ValueNet(seed=0)
    vo = ValueOrder(net, sample=4096, min_states=1, gain=0.0)
    for _ in range(reps):
        t0 = time.perf_counter()
        a = eng.solve(t3, max_depth=3, oep_mode=OEP_EXACT, count_levels=True, sol_cap=4096)
        b = eng.solve(negate_task(1), max_depth=2, oep_mode=OEP_NONE, count_levels=True)
        with tempfile.TemporaryDirectory() as d:
            st = eng.record(t3, d, max_depth=3, task_id=1, neg_stride=8)
            n_files = len(os.listdir(d))
        c = eng.solve_ordered(t4, vo, chunk=256, max_depth=4, split_depth=2)
        torch.cuda.synchronize()
        print(f"misc: K*={a.optimal_depth} ({len(a.programs)} programs), no-OEP "
              f"K*={b.optimal_depth}, recorded {n_files} files ({st}), ordered "
              f"K*={c.optimal_depth}: {time.perf_counter() - t0:.3f} s", flush=True)
    vo.close()
    eng.close()


CASES = {"engine_depths": case_engine_depths, "suffix_depth2": case_suffix_depth2, "misc": case_misc,
         "noalloc": case_noalloc,
         "valuenet": case_valuenet, "orders": case_orders, "branch": case_branch,
         "branch_saturating_add": case_branch_saturating_add}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("case", choices=sorted(CASES))
    ap.add_argument("--reps", type=int, default=2)
    args = ap.parse_args(argv)
    from pca_gb300.build import build_engine
    build_engine()
    CASES[args.case](args.reps)


if __name__ == "__main__":
    main()

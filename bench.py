"""Benchmark: verified candidates/s of the exhaustive PCA-16 solve on one GB300.

Workload (one step): the hybrid solve of is_power2 -- 32 test vectors (12
powers of two below 2^15, 0, 0x8000, 18 uniform non-powers; seed 1),
branchless subset, iterative deepening to program length 7 (kernel depth 4),
levels 1..3 built with the exact OEP pruner and the last instruction
enumerated by the suffix kernel (split depth 3). A step proves whether a
length-7 program exists. Synthetic data, generated from the seed.

  value       candidates decided per second, device time (CUDA events on the
              engine's stream around each solve)
  e2e         the same count per second of wall time around pcagb_solve, the
              C-ABI call with host buffers (task in, programs out)
  roofline    the dominant kernel against its bound
  cpu_baseline the reference algorithm (oracle port of tools/enumerate.c)
              on the host cores, time-bounded sample of the same workload

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

With N > 1 (torchrun) every rank runs the same solve on its own GPU: the
search does not shard (one task, one device), so ranks are independent
replicas and value sums them over the max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "verified candidates/s"
UNIT = "candidates/s"
WORKLOAD = ("is_power2, 32 tests, branchless, IDDFS to kernel depth 4 "
            "(program length 7), split depth 3")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--max-depth", type=int, default=4)
    ap.add_argument("--split", type=int, default=3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--cpu-budget", type=float, default=12.0,
                    help="seconds of CPU work in the cpu_baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--hbm-gb", type=float, default=0.0,
                    help="engine arena size in GB (0: 60%% of free HBM)")
    ap.add_argument("--workload", default="power2",
                    choices=["power2", "batched", "served", "guided", "branch"],
                    help="power2: the headline solve (default); batched: 1,000 synthetic "
                         "tasks plain vs batched; served: Poisson arrivals, served vs plain; "
                         "guided: value-ordered vs DFS-ordered search")
    ap.add_argument("--rate", type=float, default=50.0, help="served: arrivals per second")
    ap.add_argument("--requests", type=int, default=200, help="served: number of requests")
    ap.add_argument("--tasks", type=int, default=1000, help="batched: number of tasks")
    ap.add_argument("--source", default="synthetic", choices=["synthetic", "reference"],
                    help="batched: this project's generator of the configured distribution, or "
                         "the reference's own corpus generator (10 tests, length 3-8)")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return p, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


def cpu_baseline(task, depth: int, budget: float):
    """The reference algorithm (oracle port of tools/enumerate.c, 32-bit OEP)
    on every host core for `budget` seconds of the same workload."""
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    n, secs, _ = O.sample_throughput(task, depth, cores, budget)
    return {"value": n / secs if secs > 0 else 0.0, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": (f"kernel depth {depth} DFS of the same task over (root, level-1) "
                       f"candidate pairs handed out in DFS order, {secs:.1f} s on {cores} threads, "
                       f"{n} candidates")}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_over_ranks(t_dev: float, t_wall: float, cands: float, device) -> tuple:
    """Replica aggregation over the process group: the slowest rank's device
    and wall times (MAX) and the candidates every rank decided (SUM)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([t_dev, t_wall], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([float(cands)], dtype=torch.float64, device=device)
    dist.all_reduce(c)
    return float(t[0]), float(t[1]), float(c[0])


def run_reference(args):
    """Reference arm: the reference's CPU solver algorithm on the host cores."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from pca_gb300 import taskgen
    from oracle.build import build_oracle
    build_oracle()
    task = taskgen.is_power2_task(args.seed)
    per_step = max(2.0, min(10.0, 150.0 / max(1, args.steps + args.warmup)))
    from oracle import oracle as O
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        O.sample_throughput(task, args.max_depth, cores, per_step)
    tot_n, tot_s = 0, 0.0
    for _ in range(args.steps):
        n, s, _ = O.sample_throughput(task, args.max_depth, cores, per_step)
        tot_n += n
        tot_s += s
    v = tot_n / tot_s
    sample = (f"kernel depth {args.max_depth} DFS of the workload over (root, level-1) candidate "
              f"pairs, {per_step:.0f} s per step on {cores} threads")
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000 * tot_s / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16",
            "data": "synthetic", "config": {"workload": WORKLOAD, "seed": args.seed},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def pct(xs, p):
    xs = sorted(xs)
    if not xs:
        return None
    return xs[min(len(xs) - 1, max(0, int(round(p / 100.0 * len(xs) + 0.5)) - 1))]


def run_batched(args):
    """1,000 seeded synthetic tasks (source length 3..8, 16..32 tests, 1..2
    inputs), proven optimal up to kernel depth 4 (or proven longer): one task
    at a time vs shared batched launches. Metric: tasks decided per second."""
    from pca_gb300 import corpus, taskgen
    from pca_gb300.pcalib import Engine
    if args.source == "reference":
        tasks = corpus.corpus_tasks(args.tasks, seed=42, min_len=3, max_len=8)
        workload = (f"{len(tasks)} tasks of the reference's corpus generator (seed 42, kernel "
                    "length 3-8, 10 tests, 1-2 inputs), kernel depth <= 4, all submitted at once; "
                    "batched = 4 engine slots x up to 256 tasks per launch")
    else:
        tasks = taskgen.synthetic_batch(args.tasks, seed=7)
        workload = (f"{len(tasks)} synthetic tasks, source length 3-8, 16-32 tests, 1-2 inputs, "
                    "kernel depth <= 4, all submitted at once; batched = 4 engine slots x up to "
                    "256 tasks per launch")
    eng = Engine(0, int(args.hbm_gb * (1 << 30)))
    eng.solve_batch(tasks[:50], max_depth=4, sol_cap=1, first_only=True)  # warm-up
    t0 = time.perf_counter()
    plain, plain_done = [], []
    for t in tasks:
        plain.append(eng.solve(t, max_depth=4, sol_cap=1, first_only=True))
        plain_done.append(time.perf_counter() - t0)
    t_plain = time.perf_counter() - t0
    eng.close()
    from pca_gb300.serve import Server, replay
    srv = Server(slots=4, max_batch=256, max_depth=4, sol_cap=1)
    replay(srv, [(0.0, t) for t in tasks[:50]])  # warm-up
    srv.close()
    srv = Server(slots=4, max_batch=256, max_depth=4, sol_cap=1)
    reqs = replay(srv, [(0.0, t) for t in tasks])
    srv.close()
    t_batch = max(r.finish for r in reqs) - min(r.arrival for r in reqs)
    batched = [r.solution for r in reqs]
    for r in reqs:
        r.solution.seconds = r.latency
    same = all((a.optimal_depth, a.programs[:1]) == (b.optimal_depth, b.programs[:1])
               for a, b in zip(plain, batched))
    cands = sum(sum(s.candidates) for s in batched)
    hist = {}
    for s in batched:
        hist[s.optimal_depth] = hist.get(s.optimal_depth, 0) + 1
    line = {"metric": "tasks proven per second (batched)", "value": len(tasks) / t_batch,
            "unit": "tasks/s", "higher_is_better": True, "n_gpus": 1, "data": "synthetic",
            "config": {"workload": workload},
            "plain_tasks_per_s": len(tasks) / t_plain, "speedup_vs_plain": t_plain / t_batch,
            "plain_seconds": t_plain, "batched_seconds": t_batch,
            "time_to_proven_optimal_in_mix": {
                "note": "per task, from the moment the whole mix is submitted",
                "plain_mean_s": statistics.mean(plain_done), "plain_p50_s": pct(plain_done, 50),
                "plain_p99_s": pct(plain_done, 99),
                "batched_mean_s": statistics.mean(s.seconds for s in batched),
                "batched_p50_s": pct([s.seconds for s in batched], 50),
                "batched_p99_s": pct([s.seconds for s in batched], 99)},
            "plain_solve_p50_s": pct([s.seconds for s in plain], 50),
            "plain_solve_p99_s": pct([s.seconds for s in plain], 99),
            "same_answers": same, "candidates_per_s": cands / t_batch,
            "optimal_depth_histogram": {str(k): v for k, v in sorted(hist.items())}}
    print(json.dumps(line), flush=True)


def run_served(args):
    """Poisson arrivals of synthetic tasks (source length mix 4:30%, 5:30%,
    6:25%, 7:10%, 8:5%), each proven optimal up to kernel depth 4: the
    continuous-batching server vs one task at a time."""
    from pca_gb300 import taskgen
    from pca_gb300.serve import SerialServer, Server, latency_summary, replay
    trace = taskgen.poisson_stream(args.requests, rate=args.rate, seed=11)
    out = {}
    for name, make in (("served", lambda: Server(slots=4, max_batch=256, max_depth=4)),
                       ("plain", lambda: SerialServer(max_depth=4))):
        srv = make()
        replay(srv, trace[:20])  # warm-up
        srv.close()
        srv = make()
        reqs = replay(srv, trace)
        srv.close()
        out[name] = latency_summary(reqs)
        out[name]["batches"] = len(srv.batches)
    s, p = out["served"], out["plain"]
    line = {"metric": "p99 time-to-proven-optimal (served)", "value": s["p99_s"], "unit": "s",
            "higher_is_better": False, "n_gpus": 1, "data": "synthetic",
            "config": {"workload": f"Poisson {args.rate:g} req/s, {args.requests} requests, "
                                   "source length mix 4-8, kernel depth <= 4, 4 engine slots"},
            "served": s, "plain": p,
            "p99_ratio_plain_over_served": p["p99_s"] / s["p99_s"] if s["p99_s"] else None,
            "p50_ratio_plain_over_served": p["p50_s"] / s["p50_s"] if s["p50_s"] else None}
    print(json.dumps(line), flush=True)


def run_guided(args):
    """The value network trained on the solver's own labels, then held-out
    tasks solved by the plain engine (the whole optimal-depth stage) and by
    ordered solves (DFS, random and value order, 256 prefixes per launch,
    stopping at the first launch with a correct program): time to proven
    optimal and the fraction of the optimal depth's prefixes visited before
    the first correct program."""
    import torch
    from pca_gb300 import taskgen
    from pca_gb300.guided import RandomOrder, ValueOrder, build_dataset, train
    from pca_gb300.pcalib import Engine
    from pca_gb300.valuenet import ValueNet
    eng = Engine(0, int(args.hbm_gb * (1 << 30)))
    t0 = time.perf_counter()
    ds, used = build_dataset(eng, taskgen.synthetic_batch(3000, seed=101), max_depth=4, seed=1)
    t_label = time.perf_counter() - t0
    net = ValueNet(seed=0, lr=1e-3, pos_weight=8.0)
    t0 = time.perf_counter()
    losses = train(net, ds, epochs=10)
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    ev = taskgen.synthetic_batch(2000, seed=202)
    sols = eng.solve_batch(ev, max_depth=4, sol_cap=1, first_only=True)
    sel = [t for t, s in zip(ev, sols) if s.optimal_depth in (3, 4)]
    vo = ValueOrder(net, sample=4096)
    orders = (("dfs", lambda v: None), ("random", RandomOrder(1)), ("value", vo),
              ("dfs_every_stage", lambda v: None),
              ("value_every_stage", ValueOrder(net, min_states=1, gain=0.0)))
    # dfs, random and value orders run with the engine's automatic split
    # (stages it expects to be cheap run plain); value_every_stage orders
    # every stage from level 2, to measure the ordering itself
    split = {"dfs": -1, "random": -1, "value": -1, "dfs_every_stage": 2, "value_every_stage": 2}
    for t in sel[:3]:  # warm-up (lazy kernel loading)
        eng.solve(t, max_depth=4, sol_cap=1, first_only=True)
        for name, fn in orders:
            eng.solve_ordered(t, fn, chunk=256, max_depth=4, split_depth=split[name])
    vo.score_ms = 0.0
    res = {"plain": [], "dfs": [], "random": [], "value": [], "dfs_every_stage": [],
           "value_every_stage": []}
    for t in sel:
        p = eng.solve(t, max_depth=4, sol_cap=1, first_only=True)
        res["plain"].append((1.0, None, p.seconds))
        for name, fn in orders:
            s = eng.solve_ordered(t, fn, chunk=256, max_depth=4, split_depth=split[name])
            assert s.optimal_depth == p.optimal_depth
            res[name].append((s.prefixes_to_first / max(s.prefixes_at_optimal, 1), s.ms_to_first,
                              s.seconds))
    summ = {}
    for k, v in res.items():
        summ[k] = {"mean_fraction_to_first": statistics.mean(a[0] for a in v),
                   "median_fraction_to_first": statistics.median(a[0] for a in v),
                   "mean_time_to_proven_optimal_s": statistics.mean(a[2] for a in v),
                   "median_time_to_proven_optimal_s": statistics.median(a[2] for a in v)}
        if k != "plain":
            summ[k]["mean_ms_to_first_in_optimal_stage"] = statistics.mean(a[1] for a in v)
    plain_t = summ["plain"]["mean_time_to_proven_optimal_s"]
    for k in ("dfs", "random", "value", "dfs_every_stage", "value_every_stage"):
        summ[k]["speedup_vs_plain"] = plain_t / summ[k]["mean_time_to_proven_optimal_s"]
    line = {"metric": "time-to-proven-optimal, plain engine / value-ordered (mean over tasks)",
            "value": summ["value"]["speedup_vs_plain"],
            "unit": "x", "higher_is_better": True, "n_gpus": 1, "data": "synthetic",
            "prefixes_before_first_value_over_dfs":
                summ["value_every_stage"]["mean_fraction_to_first"]
                / summ["dfs_every_stage"]["mean_fraction_to_first"],
            "config": {"workload": f"{len(sel)} held-out synthetic tasks with optimal kernel depth "
                                   "3-4; ordered solves with the engine's automatic split (stages "
                                   "predicted under 2 ms run plain; value ranks a 4,096-prefix "
                                   "sample spread over the level by a CUDA-graph replay, the rest "
                                   "follows in the sample map's order), value_every_stage "
                                   "scores whole levels from split level 2; first launch 256 "
                                   "prefixes, doubling",
                       "train_tasks_used": used, "train_states": ds.n,
                       "params": net.n_params(), "epochs": 10},
            "label_seconds": t_label, "train_seconds": t_train, "train_loss": losses,
            "orders": summ, "value_scoring_ms_per_task": vo.score_ms / max(len(sel), 1)}
    for _, fn in orders:
        if isinstance(fn, ValueOrder):
            fn.close()
    torch.cuda.synchronize()
    print(json.dumps(line), flush=True)


def run_branch(args):
    """Branch mode (CMP, forward BR, DIV, MOD) on the reference's own task
    files at their documented optimal lengths: time to the proven optimum
    per task (every shorter depth searched completely). The task specs come
    from the committed fixture of the reference's tasks."""
    from pca_gb300.pcalib import Engine, task_from_dict
    fixture = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden",
                           "ref_published.json")
    eng = Engine(0, 1 << 30)
    rows = []
    for t in json.load(open(fixture)):
        task = task_from_dict(t["task"])
        K = t["published_length"] - task.num_inputs - 2
        eng.solve_branch(task, max_depth=K)  # warm-up
        t0 = time.perf_counter()
        s = eng.solve_branch(task, max_depth=K)
        dt = time.perf_counter() - t0
        rows.append({"task": t["name"], "published_length": t["published_length"],
                     "found_length": s.optimal_depth + task.num_inputs + 2
                     if s.optimal_depth >= 0 else None, "seconds": dt,
                     "candidates": int(sum(s.tried))})
    total = sum(r["seconds"] for r in rows)
    line = {"metric": "branch-mode time to proven optimal (sum over the reference's tasks)",
            "value": total, "unit": "s", "higher_is_better": False, "n_gpus": 1,
            "data": "the reference's task files", "config": {"workload": "branch mode, "
            "reference tasks at their documented optimal lengths (saturating_add 8, is_power2 7, "
            "max 7, abs 6, ...)"},
            "all_lengths_match": all(r["found_length"] == r["published_length"] for r in rows),
            "tasks": rows}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload != "power2":
        from pca_gb300.build import build_engine
        build_engine()
        return {"batched": run_batched, "served": run_served, "guided": run_guided,
                "branch": run_branch}[args.workload](args)
    rank, world, local = dist_env()
    import torch
    from pca_gb300.build import build_engine
    if rank == 0 or not os.path.exists(os.path.join(REPO, "pca_gb300", "_lib", "libpcagb.so")):
        build_engine()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist.barrier()
    from pca_gb300 import taskgen
    from pca_gb300.pcalib import Engine, OEP_EXACT_LIVE
    torch.cuda.set_device(local)
    task = taskgen.is_power2_task(args.seed)
    eng = Engine(local, int(args.hbm_gb * (1 << 30)))
    stream = torch.cuda.ExternalStream(eng.stream, device=local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def step():
        return eng.solve(task, max_depth=args.max_depth, split_depth=args.split,
                         oep_mode=OEP_EXACT_LIVE, sol_cap=1 << 12)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    sampler = ClockSampler(local)
    sampler.start()
    dev_ms, wall_s, cands, evals = [], [], 0, 0
    launches, h2d, d2h = 0, 0, 0
    insert_ms, insert_n, insert_children, suffix_ms, suffix_n = 0.0, 0, 0, 0.0, 0
    expand_ms = 0.0
    sol = None
    for _ in range(args.steps):
        flush.fill_(1)  # L2 flush between timed steps (256 MB > 126 MB L2)
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        t0 = time.perf_counter()
        sol = step()
        t1 = time.perf_counter()
        ev1.record(stream)
        ev1.synchronize()
        dev_ms.append(ev0.elapsed_time(ev1))
        wall_s.append(t1 - t0)
        cands += sum(sol.candidates)
        evals += sum(sol.evaluations)
        launches += sol.kernel_launches
        h2d += sol.h2d_bytes
        d2h += sol.d2h_bytes
        insert_ms += sol.gpu_ms_insert
        expand_ms += sol.gpu_ms_expand
        insert_n += sol.insert_launches
        insert_children += sol.insert_children
        suffix_ms += sol.gpu_ms_suffix
        suffix_n += sol.suffix_launches
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clocks = sampler.stop()
    t_dev = sum(dev_ms) / 1000.0
    t_wall = sum(wall_s)
    if world > 1:
        t_dev, t_wall, total_cands = reduce_over_ranks(t_dev, t_wall, cands, f"cuda:{local}")
    else:
        total_cands = float(cands)
    if rank != 0:
        dist.destroy_process_group()
        return
    pk, pk_kind = peaks()
    sm_max = pk.get("sm_max_mhz", 2070.0)
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    # suffix kernel: value classes evaluated per second against the issue
    # roofline (one warp instruction per SM sub-partition per clock)
    suffix_evals_per_s = evals / (suffix_ms / 1000.0) if suffix_ms > 0 else 0.0
    line = {
        "metric": METRIC, "value": total_cands / t_dev, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": max(3, args.warmup),
        "ms_per_step": 1000.0 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u16", "data": "synthetic",
        "config": {"workload": WORKLOAD, "seed": args.seed, "max_kernel_depth": args.max_depth,
                   "split_depth": args.split, "oep": "exact regs+flags+live",
                   "l2": "flushed between steps (256 MB write)",
                   "parallelism": f"replicas x{world}"},
        "optimal_depth": sol.optimal_depth if sol else None,
        "candidates_per_step": cands // args.steps,
        "evaluations_per_step": evals // args.steps,
        "e2e": {"value": total_cands / t_wall, "unit": UNIT,
                "h2d_bytes_per_step": h2d // args.steps, "d2h_bytes_per_step": d2h // args.steps},
        "gpu_launches": launches,
        "clocks": clocks,
        # expand_total: every level build (insert, mark, scan, materialise)
        "kernels_ms_per_step": {"suffix": suffix_ms / args.steps, "insert": insert_ms / args.steps,
                                "expand_total": expand_ms / args.steps},
        "launches_per_step": {"insert": insert_n / args.steps, "suffix": suffix_n / args.steps},
        "children_inserted_per_step": insert_children // args.steps,
    }
    # Roofline of the suffix kernel: integer-issue bound. Peak = one warp
    # instruction per SM sub-partition per clock at the measured max clock.
    # Achieved = this run's value-class evaluations of the full candidate
    # space per second of suffix-kernel time x the kernel's warp instructions
    # per such evaluation, measured by ncu (profiles/k_suffix_is_power2_t32_k4.md:
    # 1.26e9 instructions for the depth-4 launch, whose full space is 7.30e8
    # evaluations; the kernel scans only the classes that can solve).
    inst_per_eval = 1255101666 / 7.30e8
    peak_issue = sms * 4 * sm_max * 1e6
    achieved_issue = suffix_evals_per_s * inst_per_eval
    line["roofline"] = {
        "kernel": "k_suffix<32,1> (last instruction over value classes)",
        "bound": "int_issue", "unit": "Gwarp-inst/s",
        "achieved": achieved_issue / 1e9, "peak": peak_issue / 1e9,
        "frac": achieved_issue / peak_issue,
        "traffic": 2735377000 + 3757056,
        "evaluations_per_s": suffix_evals_per_s,
        "peak_source": f"{sms} SMs x 4 issue slots x sm_max_mhz from MEASURED_PEAKS.json ({pk_kind})",
        "ncu": "profiles/k_suffix_is_power2_t32_k4.md",
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(task, args.max_depth, args.cpu_budget)
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

"""The learned part: labels from the exhaustive solver, GPU training of the
value network, and value-ordered search.

Labels (the reference's recorder, tools/enumerate.c:493-533, restated on
this engine): the GPU solver proves a task's optimal depth K* and returns its
optimal programs; every state those programs pass through at depth
1..K*-1 is a positive ("can finish optimally", remaining steps K* - d),
and states reached by random generator walks that are not positive are
negatives.

Ordering: at each suffix stage the engine hands the split level to
`ValueOrder`, which scores every prefix state with the network (chunks of
the level through the project's BF16 kernels, on the engine's stream) and
returns the prefixes by decreasing score (the encoder runs as one fused
tcgen05 kernel per chunk, the trunk on the pooled rows). The engine visits them in that
order, chunk by chunk, and stops the optimal depth's stage at the first
chunk with a correct program. Depths below the optimum are searched
completely in any order, so the optimal depth stays proven: the network
reorders work, it never prunes. DFS order (the plain engine) is the
fallback and the judge.
"""
from __future__ import annotations

import ctypes
import random

import numpy as np
import torch

from .pcalib import PCALib, SearchState
from .valuenet import ROWS, ValueNet


def _state_arrays(states, T):
    """search_state_t list -> level-layout arrays (regs [n][8][32], flags
    [n][32], live [n])."""
    n = len(states)
    regs = np.zeros((n, 8, 32), dtype=np.uint16)
    flags = np.zeros((n, 32), dtype=np.uint8)
    live = np.zeros(n, dtype=np.uint8)
    for i, s in enumerate(states):
        r = np.frombuffer(bytes(s.regs), dtype=np.uint16).reshape(32, 8)
        regs[i] = r.T
        regs[i, :, T:] = 0
        f = np.frombuffer(bytes(s.flags), dtype=np.uint8)
        flags[i, :T] = f[:T]
        live[i] = s.live
    return regs, flags, live


def task_io_array(task):
    io = np.zeros((3, 32), dtype=np.uint16)
    for t in range(task.num_tests):
        io[0, t] = task.tests[t].inputs[0]
        if task.num_inputs > 1:
            io[1, t] = task.tests[t].inputs[1]
        io[2, t] = task.tests[t].outputs[0]
    return io


def label_task(lib: PCALib, task, programs, optimal_depth, rng, neg_ratio=16):
    """Positive states along the optimal programs, negative states from
    random generator walks. Returns (states, depth, label, remaining)."""
    ctx = lib.init_ctx(task)
    root = lib.init_root(ctx)
    K = optimal_depth
    pos = {}
    for prog in programs:
        kern = prog[task.num_inputs:task.num_inputs + K]
        s = root
        for d, insn in enumerate(kern[:-1], start=1):
            s = lib.step(ctx, s, insn)
            key = (d, bytes(s))
            pos.setdefault(key, s)
    states, depth, label, remaining = [], [], [], []
    for (d, _), s in pos.items():
        states.append(s)
        depth.append(d)
        label.append(1.0)
        remaining.append(K - d)
    want = max(neg_ratio * len(pos), neg_ratio)
    tries = 0
    while sum(1 for x in label if x == 0.0) < want and tries < 20 * want:
        tries += 1
        d = rng.randrange(1, K)
        s = root
        for _ in range(d):
            c = lib.gen_candidates(s)
            s = lib.step(ctx, s, rng.choice(c))
        if (d, bytes(s)) in pos:
            continue
        states.append(s)
        depth.append(d)
        label.append(0.0)
        remaining.append(-1)
    return states, depth, label, remaining


class Dataset:
    """Labelled states of many tasks, kept on the device."""

    def __init__(self, device="cuda"):
        self.dev = torch.device(device)
        self.parts = []
        self.task_io, self.task_T = [], []

    def add_task(self, task, states, depth, label, remaining):
        tid = len(self.task_io)
        self.task_io.append(task_io_array(task))
        self.task_T.append(task.num_tests)
        regs, flags, live = _state_arrays(states, task.num_tests)
        self.parts.append(dict(regs=regs, flags=flags, live=live,
                               depth=np.array(depth, dtype=np.uint8),
                               label=np.array(label, dtype=np.float32),
                               remaining=np.array(remaining, dtype=np.int32),
                               task=np.full(len(states), tid, dtype=np.uint16)))

    def finalize(self):
        cat = {k: np.concatenate([p[k] for p in self.parts]) for k in self.parts[0]}
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(self.dev)  # noqa: E731
        self.n = len(cat["label"])
        self.data = dict(regs=t(cat["regs"].astype(np.int16)), flags=t(cat["flags"]),
                         live=t(cat["live"]), depth=t(cat["depth"]), label=t(cat["label"]),
                         remaining=t(cat["remaining"]), task=t(cat["task"].astype(np.int16)))
        self.data["task_io"] = t(np.stack(self.task_io).astype(np.int16))
        self.data["task_T"] = t(np.array(self.task_T, dtype=np.int32))
        return self

    def batches(self, size, gen):
        perm = torch.randperm(self.n, generator=gen).to(self.dev)
        for i in range(0, self.n - size + 1, size):
            idx = perm[i:i + size]
            b = {k: self.data[k][idx] for k in ("regs", "flags", "live", "depth", "label",
                                                   "remaining", "task")}
            b.update(task_io=self.data["task_io"], task_T=self.data["task_T"], TP=32)
            yield b


def build_dataset(engine, tasks, max_depth=4, seed=0, neg_ratio=16, device="cuda"):
    lib = PCALib()
    rng = random.Random(seed)
    ds = Dataset(device)
    sols = engine.solve_batch(tasks, max_depth=max_depth, sol_cap=512)
    used = 0
    for task, sol in zip(tasks, sols):
        if sol.optimal_depth < 2 or not sol.programs:
            continue
        ds.add_task(task, *label_task(lib, task, sol.programs, sol.optimal_depth, rng, neg_ratio))
        used += 1
    return ds.finalize(), used


def train(net: ValueNet, ds: Dataset, epochs=8, batch=2048, seed=0, log=None):
    gen = torch.Generator().manual_seed(seed)
    losses = []
    for ep in range(epochs):
        tot, nb = 0.0, 0
        for b in ds.batches(batch, gen):
            tot += net.train_step(b)
            nb += 1
        losses.append(tot / max(nb, 1))
        if log:
            log(f"epoch {ep + 1}: loss {losses[-1]:.4f}")
    return losses


class ValueOrder:
    """Order callback for Engine.solve_ordered: prefixes by decreasing
    predicted probability of finishing optimally. A level is scored once
    (stages at several depths reuse its order). Stages keep DFS order when
    scoring would cost more than it can save: levels below `min_states`,
    and stages the engine expects to finish in less than `gain` x the
    scoring time (fixed_ms + scored states / states_per_ms).

    With `sample` set, a level larger than it is scored on a uniform random
    sample of that many prefixes: the order is the sample by decreasing
    score, then every other prefix in random order. The first correct
    program usually sits in the first few percent of a good order, so the
    ranked sample decides the first launches at a fraction of the scoring
    cost; the order stays a permutation of the whole level."""

    def __init__(self, net: ValueNet, chunk_states=1 << 20, min_states=4096, gain=2.0,
                 fixed_ms=0.25, states_per_ms=1.0e5, sample=None, seed=0):
        self.net = net
        self.chunk_states = chunk_states
        self.min_states = min_states
        self.gain, self.fixed_ms, self.states_per_ms = gain, fixed_ms, states_per_ms
        self.sample = sample
        self.gen = torch.Generator(device=net.dev).manual_seed(seed)
        self.score_ms = 0.0
        self._cache = {}

    def __call__(self, view):
        n = view.n
        if n < self.min_states:
            return None
        key = (view.regs, n, view.depth)
        scored = n if not self.sample else min(n, self.sample)
        if key not in self._cache and \
                view.est_stage_ms < self.gain * (self.fixed_ms + scored / self.states_per_ms):
            return None
        if key in self._cache:
            return self._cache[key]
        dev = self.net.dev
        stream = torch.cuda.ExternalStream(view.stream, device=dev)
        tp = view.tp
        with torch.cuda.stream(stream):
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            ntask = view.ntasks
            task_io = _device_view(view.task_io, ntask * 3 * 32, torch.int16, dev)
            task_T = _device_view(view.task_T, ntask, torch.int32, dev)
            if scored < n:
                order = self._sampled_order(view, n, scored, tp, task_io, task_T, dev)
                ev1.record(stream)
                ev1.synchronize()
                self.net.check_status()
                self.score_ms += ev0.elapsed_time(ev1)
                self._cache = {key: order}
                return order
            scores = torch.empty(n, device=dev, dtype=torch.float32)
            for b0 in range(0, n, self.chunk_states):
                m = min(self.chunk_states, n - b0)
                regs = _device_view(view.regs + b0 * 8 * tp * 2, m * 8 * tp, torch.int16, dev)
                flags = _device_view(view.flags + b0 * tp, m * tp, torch.uint8, dev)
                live = _device_view(view.live + b0, m, torch.uint8, dev)
                task = _device_view(view.task + b0 * 2, m, torch.int16, dev)
                depth = torch.full((m,), view.depth, device=dev, dtype=torch.uint8)
                scores[b0:b0 + m] = self.net.forward_fused(regs, flags, live, task, depth, tp,
                                                           task_io, task_T)[:, 0]
            order = torch.argsort(scores, descending=True, stable=True).to(torch.int32)
            ev1.record(stream)
        ev1.synchronize()
        self.net.check_status()
        self.score_ms += ev0.elapsed_time(ev1)
        self._cache = {key: order}
        return order


    def _sampled_order(self, view, n, m, tp, task_io, task_T, dev):
        perm = torch.randperm(n, device=dev, generator=self.gen)
        head = perm[:m]
        regs = _device_view(view.regs, n * 8 * tp, torch.int16, dev).view(n, 8 * tp)
        flags = _device_view(view.flags, n * tp, torch.uint8, dev).view(n, tp)
        live = _device_view(view.live, n, torch.uint8, dev)
        task = _device_view(view.task, n, torch.int16, dev)
        depth = torch.full((m,), view.depth, device=dev, dtype=torch.uint8)
        scores = self.net.forward_fused(regs.index_select(0, head).reshape(-1),
                                        flags.index_select(0, head).reshape(-1),
                                        live.index_select(0, head), task.index_select(0, head),
                                        depth, tp, task_io, task_T)[:, 0]
        ranked = head[torch.argsort(scores, descending=True, stable=True)]
        return torch.cat([ranked, perm[m:]]).to(torch.int32)


class RandomOrder:
    def __init__(self, seed=0):
        self.gen = torch.Generator().manual_seed(seed)

    def __call__(self, view):
        if view.n == 0:
            return None
        return torch.randperm(view.n, generator=self.gen).to(torch.int32).cuda()


def _device_view(addr, count, dtype, dev):
    """A torch tensor over `count` elements of existing device memory at
    `addr` (engine-owned; valid during the callback)."""
    itemsize = torch.empty(0, dtype=dtype).element_size()

    class _Iface:
        __cuda_array_interface__ = {
            "shape": (count,), "typestr": {1: "|u1", 2: "<i2", 4: "<i4"}[itemsize]
            if dtype != torch.float32 else "<f4",
            "data": (int(addr), False), "version": 3}
    t = torch.as_tensor(_Iface(), device=dev)
    return t.view(dtype) if t.dtype != dtype else t

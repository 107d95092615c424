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
fallback, and its answers are the ones an ordered solve must reproduce.
"""
from __future__ import annotations

import atexit
import ctypes
import math
import random
import weakref

import numpy as np
import torch

from .pcalib import PCALib
from .valuenet import ValueNet


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
        tot, nb = None, 0
        for b in ds.batches(batch, gen):
            loss = net.train_step_graph(b)
            tot = loss if tot is None else tot + loss
            nb += 1
        losses.append(float(tot) / max(nb, 1) if nb else 0.0)   # one read per epoch
        net.check_status()
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

    With `sample` set, a level larger than it is scored on a sample of that
    many prefixes spread over it (prefix (a * i + b) mod n for sample i, a
    coprime to n, a and b drawn per level): the order is the sample by
    decreasing score, then every other prefix in the same map's order (a
    permutation of the whole level). The first correct program usually sits
    in the first few percent of a good order, so the ranked sample decides
    the first launches at a fraction of the scoring cost. The ranking (the
    gather of the sample, the fused encoder, the trunk and the sort) is a
    CUDA graph captured once per test width and task table and replayed on
    the engine's stream; the level's addresses reach it through a small
    device buffer, so one replay and one order kernel serve any level. A
    stage expected to take at least `full_gain` times the cost of scoring
    the whole level (a deep stage: seconds against milliseconds) has its
    whole level ranked instead.

    The score of a state is the logit of "finishes optimally"; for a long
    stage, ranked whole, with `steps_head` also the log-probability the
    steps head gives a positive state for finishing in exactly the stage's
    remaining instructions (target depth - level depth): a state that can
    finish, but only in more steps, ranks lower. `net` may be a list of networks: the whole-level ranking
    then orders by the sum of their scores; a sampled ranking uses the
    first."""

    def __init__(self, net: ValueNet, chunk_states=1 << 20, min_states=4096, gain=2.0,
                 fixed_ms=0.25, states_per_ms=1.0e5, sample=None, seed=0, full_gain=50.0,
                 steps_head=True):
        self.nets = list(net) if isinstance(net, (list, tuple)) else [net]
        self.net = self.nets[0]
        self.chunk_states = chunk_states
        self.min_states = min_states
        self.gain, self.fixed_ms, self.states_per_ms = gain, fixed_ms, states_per_ms
        self.sample = sample
        # with `sample` set, a stage the engine expects to take at least
        # full_gain x the cost of scoring its whole level is ranked whole
        # (None: always sampled)
        self.full_gain = full_gain
        # whole-level ranking: add the log-probability the steps head gives
        # a positive state for finishing in exactly the stage's remaining
        # instructions (target depth - level depth)
        self.steps_head = steps_head
        self.rng = random.Random(seed)
        self.score_ms = 0.0
        self._cache = {}
        self._graphs = {}
        _LIVE_ORDERS.add(self)

    def new_solve(self):
        """Forget the levels scored so far (Engine.solve_ordered calls this
        before each solve): levels are keyed by device address, size and
        depth, which a level of another solve can repeat."""
        self._cache = {}

    def close(self):
        """Release the captured ranking graphs and their buffers (also done
        for every live ValueOrder when the interpreter exits, while the CUDA
        context still exists)."""
        self._cache = {}
        for G in self._graphs.values():
            G.pop("graph", None)
        self._graphs = {}

    def __call__(self, view):
        n = view.n
        if n < self.min_states:
            return None
        # a long stage (full_gain x the cost of scoring its whole level) is
        # ranked whole and for its own remaining depth; a short one reuses
        # its level's order across depths
        long_stage = self.full_gain is not None and \
            view.est_stage_ms >= self.full_gain * (self.fixed_ms + n / self.states_per_ms)
        rem = view.target_depth - view.depth if self.steps_head and long_stage else -1
        key = (view.regs, n, view.depth, rem)
        scored = n if not self.sample else min(n, self.sample)
        if scored < n and long_stage:
            scored = n
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
                status, order = self._sampled_order(view, n, scored, tp, task_io, task_T, dev,
                                                    stream)
                ev1.record(stream)
                ev1.synchronize()
                if int(status.item()):
                    status.zero_()
                    raise RuntimeError("tensor-core kernel aborted (barrier wait timed out)")
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
                sc = None
                for nt in self.nets:
                    L = nt.forward_fused(regs, flags, live, task, depth, tp, task_io,
                                         task_T).float()
                    lg = L[:, 0]
                    if 0 <= rem <= 8:
                        lg = lg + torch.log_softmax(L[:, 1:10], dim=1)[:, rem]
                    sc = lg if sc is None else sc + lg
                scores[b0:b0 + m] = sc
            order = torch.argsort(scores, descending=True, stable=True).to(torch.int32)
            ev1.record(stream)
        ev1.synchronize()
        for nt in self.nets:
            nt.check_status()
        self.score_ms += ev0.elapsed_time(ev1)
        self._cache = {key: order}
        return order


    def _ranking_graph(self, m, tp, task_io, task_T, dev):
        """The sampled ranking captured as a CUDA graph for m samples of
        width tp against one task table."""
        gkey = (m, tp, task_io.data_ptr(), task_T.data_ptr())
        if gkey in self._graphs:
            return self._graphs[gkey]
        lib = self.net.lib
        G = {"src": torch.zeros(8, device=dev, dtype=torch.int64),
             "src_host": torch.zeros(8, dtype=torch.int64),
             "regs": torch.zeros(m * 8 * tp, device=dev, dtype=torch.int16),
             "flags": torch.zeros(m * tp, device=dev, dtype=torch.uint8),
             "live": torch.zeros(m, device=dev, dtype=torch.uint8),
             "task": torch.zeros(m, device=dev, dtype=torch.int16),
             "depth": torch.zeros(m, device=dev, dtype=torch.uint8)}

        def body():
            st = ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
            rc = lib.pcagb_vnet_gather_sample(
                ctypes.c_void_p(G["src"].data_ptr()), ctypes.c_void_p(G["regs"].data_ptr()),
                ctypes.c_void_p(G["flags"].data_ptr()), ctypes.c_void_p(G["live"].data_ptr()),
                ctypes.c_void_p(G["task"].data_ptr()), ctypes.c_void_p(G["depth"].data_ptr()),
                m, tp, st)
            if rc != 0:
                raise RuntimeError(f"sample gather failed ({rc})")
            logits = self.net.forward_fused(G["regs"], G["flags"], G["live"], G["task"], G["depth"],
                                            tp, task_io, task_T)
            # the network's status word (a fixed address the captured
            # launches keep reporting to)
            G["status"] = self.net._status_word()
            G["ranked"] = torch.argsort(logits[:, 0], descending=True, stable=True)

        # the warm-up and capture runs read the sample buffers themselves, a
        # valid level of m states (sample i = state i)
        G["src"].copy_(torch.tensor([G["regs"].data_ptr(), G["flags"].data_ptr(),
                                     G["live"].data_ptr(), G["task"].data_ptr(), m, 1, 0, 0],
                                    dtype=torch.int64))
        side = torch.cuda.Stream(device=dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            body()   # allocations and lazy initialisation outside the capture
        torch.cuda.current_stream(dev).wait_stream(side)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=side):
            body()
        G["graph"] = graph
        self._graphs[gkey] = G
        return G

    def _sampled_order(self, view, n, m, tp, task_io, task_T, dev, stream):
        G = self._ranking_graph(m, tp, task_io, task_T, dev)
        a = map_multiplier(n, self.rng.randrange(len(_MAP_PRIMES)))
        G["src_host"].numpy()[:] = (view.regs, view.flags, view.live, view.task, n, a,
                                    self.rng.randrange(n), view.depth)
        G["src"].copy_(G["src_host"])   # 64 bytes, ordered on the engine's stream
        G["graph"].replay()
        order = torch.empty(n, device=dev, dtype=torch.int32)
        rc = self.net.lib.pcagb_vnet_compose_order(
            ctypes.c_void_p(G["src"].data_ptr()), ctypes.c_void_p(G["ranked"].data_ptr()), m,
            ctypes.c_void_p(order.data_ptr()), n, ctypes.c_void_p(stream.cuda_stream))
        if rc != 0:
            raise RuntimeError(f"order composition failed ({rc})")
        return G["status"], order


# Graph memory freed after the CUDA context is gone aborts the process, so
# the graphs of every live ValueOrder are released at interpreter exit.
_LIVE_ORDERS = weakref.WeakSet()


@atexit.register
def _release_graphs():
    for vo in list(_LIVE_ORDERS):
        vo.close()
    if torch.cuda.is_initialized():
        torch.cuda.synchronize()


# multipliers of the sample map: primes, so a level size shares no factor
# with one of them unless it is a multiple of it
_MAP_PRIMES = [1000003, 1000033, 1000037, 1000039, 1000081, 1000099, 1000117, 1000121,
               1000133, 1000151, 1000159, 1000171, 1000183, 1000187, 1000193, 1000199]


def map_multiplier(n: int, start: int = 0) -> int:
    """The multiplier a of the sample map i -> (a*i + b) mod n: the first of
    the primes (from index `start`, wrapping) that is coprime to n, reduced
    mod n, so the map is a permutation of 0..n-1 for any b. A level size
    divisible by all sixteen primes (over 10^95) is out of reach."""
    if n < 1:
        raise ValueError(f"sample map over {n} prefixes")
    for p in _MAP_PRIMES[start:] + _MAP_PRIMES[:start]:
        if math.gcd(p, n) == 1:
            return p % n
    raise ValueError(f"no multiplier coprime to {n}")


class RandomOrder:
    """Order callback: a uniformly random permutation of each level, drawn
    on the device (a level of tens of millions of prefixes would take the
    host seconds)."""

    def __init__(self, seed=0, device="cuda"):
        self.gen = torch.Generator(device=device).manual_seed(seed)
        self.device = device

    def __call__(self, view):
        if view.n == 0:
            return None
        stream = torch.cuda.ExternalStream(view.stream, device=self.device)
        with torch.cuda.stream(stream):
            return torch.randperm(view.n, generator=self.gen, device=self.device,
                                  dtype=torch.int32)


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

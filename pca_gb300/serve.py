"""Continuous-batching solve server.

`Server` keeps `slots` GPU engines (each with its own CUDA stream and HBM
arena, sized from the device's free memory) and one worker thread per
engine. Requests wait in a queue; whenever a worker is free it takes every
request queued at that moment (up to `max_batch`) as one batch, so requests
that arrive while others are on the GPU join the next free slot, batches on
different slots overlap on the device, and each request's answer is
delivered as soon as its own task is decided (pcagb_solve_batch_cb), not
when its batch ends. An answer is the task's proven optimal depth and its
first optimal program in DFS order, which does not depend on the batch it
ran in or the split level the engine's autotuner chose; a solve's state
(levels, OEP tables, test order) lives only in its batch's arena and is
keyed by task, so each result is the same alone and in the mix. A solve
that fails (an engine error) hands its exception to every request of the
batch still open (Request.error); the worker goes on with the next batch.
`close()` stops new submissions and answers every request queued before it.

`NativeServer` is the native server (server.cu) behind the same interface.

`replay(trace)` drives a server from an arrival trace ((seconds, task)
pairs, e.g. taskgen.poisson_stream) in real time and returns per-request
records: arrival, completion, latency (time-to-proven-optimal), optimal
depth and programs.
"""
from __future__ import annotations

import ctypes
import queue
import threading
import time
import warnings
from dataclasses import dataclass, field

from .pcalib import (Engine, EngineError, OEP_EXACT_LIVE, ServerConfig, ServerStats, Solution,
                     SolveResult, device_memory, load_library, solution_from_result)


@dataclass
class Request:
    rid: int
    task: object
    arrival: float
    max_depth: int
    done: threading.Event = field(default_factory=threading.Event)
    finish: float = 0.0
    solution: Solution | None = None
    batch_size: int = 0
    error: Exception | None = None   # the engine's error, when the solve failed
    admitted: float = -1.0           # NativeServer: when a worker took it (server clock)
    finished: float = -1.0           # NativeServer: when its task was decided (server clock)

    @property
    def latency(self) -> float:
        return self.finish - self.arrival


class Server:
    def __init__(self, slots: int = 4, max_batch: int = 256, max_depth: int = 4, device: int = 0,
                 hbm_fraction: float = 0.8, sol_cap: int = 16, oep_mode: int = OEP_EXACT_LIVE,
                 engine_factory=None):
        if engine_factory is None:
            free, _ = device_memory(device)
            budget = int(free * hbm_fraction / max(1, slots))

            def engine_factory():
                return Engine(device, budget)
        # engine_factory() -> an object with Engine's solve_batch and close
        self.engines = [engine_factory() for _ in range(slots)]
        self.max_batch = max_batch
        self.max_depth = max_depth
        self.sol_cap = sol_cap
        self.oep_mode = oep_mode
        self.q: queue.Queue[Request | None] = queue.Queue()
        self.t0 = time.perf_counter()
        self.batches: list[int] = []
        self._stop = False
        self._lock = threading.Lock()
        self.threads = [threading.Thread(target=self._worker, args=(e,), daemon=True)
                        for e in self.engines]
        for t in self.threads:
            t.start()

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, rid: int, task, max_depth: int | None = None) -> Request:
        r = Request(rid, task, self.now(), self.max_depth if max_depth is None else max_depth)
        with self._lock:
            if self._stop:
                raise RuntimeError("the server is closed")
            self.q.put(r)
        return r

    def _take_batch(self) -> list[Request]:
        first = self.q.get()
        if first is None:
            return []
        batch = [first]
        while len(batch) < self.max_batch:
            try:
                r = self.q.get_nowait()
            except queue.Empty:
                break
            if r is None:
                self.q.put(None)
                break
            batch.append(r)
        return batch

    def _worker(self, eng: Engine):
        """Solve batches until the end marker, then free this worker's engine
        (here, not in close(): a worker still inside a solve when close()
        stops waiting frees its engine once that solve ends)."""
        try:
            self._serve(eng)
        finally:
            eng.close()

    def _serve(self, eng: Engine):
        while True:
            batch = self._take_batch()
            if not batch:
                self.q.put(None)   # the end marker, for the other workers
                return
            with self._lock:
                self.batches.append(len(batch))
            depth = max(r.max_depth for r in batch)

            def deliver(i, sol, batch=batch):
                r = batch[i]
                r.solution = sol
                r.finish = self.now()
                r.batch_size = len(batch)
                r.done.set()

            try:
                eng.solve_batch([r.task for r in batch], max_depth=depth, oep_mode=self.oep_mode,
                                sol_cap=self.sol_cap, on_done=deliver, first_only=True,
                                shared_gpu=len(self.engines) > 1)
            except Exception as exc:  # noqa: BLE001 -- handed to the requests it leaves open
                for r in batch:
                    if not r.done.is_set():
                        r.error = exc
                        r.finish = self.now()
                        r.batch_size = len(batch)
                        r.done.set()

    def close(self, timeout: float = 60.0):
        """Take no new requests, answer those already queued, and wait up to
        `timeout` seconds per worker. Each worker frees its own engine when
        it exits; one still inside a solve after the timeout frees it when
        that solve ends (freeing it under the solve would crash the
        process)."""
        with self._lock:
            self._stop = True
            self.q.put(None)
        for t in self.threads:
            t.join(timeout=timeout)
            if t.is_alive():
                warnings.warn(f"serving worker still busy after {timeout:g} s; it frees its "
                              "engine when its solve ends", RuntimeWarning)


class SerialServer(Server):
    """The plain baseline: one engine, one task at a time, first come first
    served (the reference's one-task-per-run model, on the GPU)."""

    def __init__(self, max_depth: int = 4, device: int = 0, hbm_fraction: float = 0.8,
                 sol_cap: int = 16, oep_mode: int = OEP_EXACT_LIVE, engine_factory=None):
        super().__init__(slots=1, max_batch=1, max_depth=max_depth, device=device,
                         hbm_fraction=hbm_fraction, sol_cap=sol_cap, oep_mode=oep_mode,
                         engine_factory=engine_factory)


class NativeServer:
    """The native server (pcagb_server, server.cu) behind Server's interface:
    admission by free HBM from one device pool (each solve reserves an arena
    slice), up to `workers` solves at once on their own CUDA streams,
    requests found queued together sharing one batched solve, and each
    answer delivered when its task is decided. A collector thread takes
    finished requests from the server in the order they finish."""

    def __init__(self, workers: int = 8, max_batch: int = 64, max_depth: int = 4,
                 device: int = 0, pool_bytes: int = 0, arena_bytes: int = 1 << 30,
                 sol_cap: int = 16, oep_mode: int = OEP_EXACT_LIVE, lib=None):
        self.lib = lib or load_library()
        cfg = ServerConfig()
        self.lib.pcagb_server_default_config(ctypes.byref(cfg))
        cfg.device, cfg.pool_bytes, cfg.arena_bytes = device, pool_bytes, arena_bytes
        cfg.workers, cfg.max_batch, cfg.sol_cap = workers, max_batch, sol_cap
        cfg.opts.oep_mode = oep_mode
        cfg.opts.first_only = 1
        self.h = ctypes.c_void_p()
        rc = self.lib.pcagb_server_create(ctypes.byref(cfg), ctypes.byref(self.h))
        if rc != 0:
            raise EngineError(f"server create failed ({rc}): "
                              f"{self.lib.pcagb_server_last_error().decode()}")
        self.max_depth = max_depth
        self.sol_cap = sol_cap
        self.t0 = time.perf_counter()
        self.batches: list[int] = []
        self._pending: dict[int, Request] = {}
        self._lock = threading.Lock()
        self._stop = False
        self._collector = threading.Thread(target=self._collect, daemon=True)
        self._collector.start()

    def now(self) -> float:
        return time.perf_counter() - self.t0

    def submit(self, rid: int, task, max_depth: int | None = None) -> Request:
        r = Request(rid, task, self.now(), self.max_depth if max_depth is None else max_depth)
        with self._lock:
            if self._stop:
                raise RuntimeError("the server is closed")
            nid = ctypes.c_uint64(0)
            rc = self.lib.pcagb_server_submit(self.h, ctypes.byref(task), r.max_depth,
                                              ctypes.byref(nid))
            if rc != 0:
                raise EngineError(self.lib.pcagb_server_last_error().decode())
            self._pending[nid.value] = r
        return r

    def _collect(self):
        cap = max(self.sol_cap, 1)
        progs = (ctypes.c_uint16 * (16 * cap))()
        lens = (ctypes.c_int * cap)()
        times = (ctypes.c_double * 4)()
        res = SolveResult()
        nid = ctypes.c_uint64(0)
        while True:
            got = self.lib.pcagb_server_next(self.h, 0.1, ctypes.byref(nid))
            if got != 1:
                with self._lock:
                    if self._stop and not self._pending:
                        return
                continue
            rc = self.lib.pcagb_server_collect(self.h, nid.value, ctypes.byref(res), progs, lens,
                                               cap, times)
            with self._lock:
                r = self._pending.pop(nid.value, None)
            if r is None:
                continue
            if rc == 0:
                r.solution = solution_from_result(res, progs, lens, 0, r.max_depth)
            else:
                r.error = EngineError(f"solve failed ({rc}): "
                                      f"{self.lib.pcagb_server_last_error().decode()}")
            r.batch_size = int(times[3])
            r.admitted, r.finished = times[1], times[2]
            r.finish = self.now()
            r.done.set()

    def stats(self) -> dict:
        st = ServerStats()
        self.lib.pcagb_server_stats(self.h, ctypes.byref(st))
        return {n: getattr(st, n) for n, _ in ServerStats._fields_}

    def close(self, timeout: float = 120.0):
        """Take no new requests, answer those already submitted, free the
        server."""
        with self._lock:
            self._stop = True
        self._collector.join(timeout=timeout)
        if self.h:
            st = self.stats()
            self.batches = [0] * int(st["batches"])
            self.lib.pcagb_server_destroy(self.h)
            self.h = ctypes.c_void_p()


def replay(server: Server, trace, max_depth: int | None = None) -> list[Request]:
    """Submit the trace's tasks at their arrival times (real time) and wait
    for every answer."""
    start = server.now()
    reqs = []
    for rid, (t_arr, task) in enumerate(trace):
        wait = start + t_arr - server.now()
        if wait > 0:
            time.sleep(wait)
        reqs.append(server.submit(rid, task, max_depth))
    for r in reqs:
        r.done.wait()
    return reqs


def latency_summary(reqs: list[Request]) -> dict:
    """Latency percentiles (time-to-proven-optimal), throughput and the
    count of failed requests over a replayed trace."""
    lat = sorted(r.latency for r in reqs)

    def pct(p):
        if not lat:
            return None
        k = min(len(lat) - 1, max(0, int(round(p / 100.0 * len(lat) + 0.5)) - 1))
        return lat[k]

    span = max(r.finish for r in reqs) - min(r.arrival for r in reqs)
    cands = sum(sum(r.solution.candidates) for r in reqs if r.solution)
    return {"requests": len(reqs), "p50_s": pct(50), "p99_s": pct(99), "max_s": lat[-1],
            "mean_s": sum(lat) / len(lat),
            "proven_optimal": sum(1 for r in reqs if r.solution and r.solution.optimal_depth >= 0),
            "failed": sum(1 for r in reqs if r.error is not None),
            "span_s": span, "candidates": cands,
            "candidates_per_s": cands / span if span > 0 else 0.0}

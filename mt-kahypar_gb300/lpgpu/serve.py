"""Continuous-batching refine server over batched lpgpu sessions.

Requests (hypergraph, partition, k, eps, rounds) arrive over time. The server
keeps `slots` batched sessions, each with its own CUDA stream and driven by its
own thread (the C calls release the GIL, so slots overlap on the device). A
free slot takes every waiting request that fits the device-memory budget
(admission by lpgpu_estimate_footprint against the budget minus what the other
slots hold) and refines them together as one batch; requests that arrive while
batches run wait for the next free slot. Each request's result is exactly what
refining it alone gives, because a batched session assigns sub-rounds from
instance-local ids and decides rollbacks per instance.

`plain_loop` is the baseline: one request at a time, in arrival order, one
session call sequence per request.

Every request has its own shape, so a captured CUDA graph would be used once:
both the server and the plain loop default to direct launches
(LPGPU_FLAG_NO_GRAPH).
"""
from __future__ import annotations

import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import FLAG_NO_GRAPH, Session, default_config, estimate_footprint


@dataclass
class Request:
    rid: int
    hg: object            # lpgpu.gen.Hypergraph
    k: int
    eps: float
    part: np.ndarray
    rounds: int
    arrival: float = 0.0  # seconds relative to the stream start
    # filled by the server
    start: float = None
    finish: float = None
    result: np.ndarray = None
    km1: int = None
    slot: int = None
    batch_size: int = None

    @property
    def latency(self):
        return None if self.finish is None else self.finish - self.arrival

    def footprint(self, subrounds=7):
        return estimate_footprint(self.hg.n, self.hg.m, self.hg.num_pins, self.k, subrounds)


@dataclass
class ServeStats:
    latencies: list = field(default_factory=list)
    batch_sizes: list = field(default_factory=list)
    wall: float = 0.0
    pins: int = 0
    rejected: int = 0

    def summary(self):
        lat = np.array(self.latencies) if self.latencies else np.zeros(1)
        return {"requests": len(self.latencies), "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
                "wall_s": self.wall, "pins_per_s": self.pins / self.wall if self.wall > 0 else 0.0,
                "req_per_s": len(self.latencies) / self.wall if self.wall > 0 else 0.0,
                "mean_batch": float(np.mean(self.batch_sizes)) if self.batch_sizes else 0.0,
                "rejected": self.rejected}


def _run_batch(session, reqs, subrounds, flags=FLAG_NO_GRAPH):
    """Refines `reqs` together on one batched session; returns pins processed."""
    session.upload_instances([r.hg for r in reqs])
    session.set_partition_instances([r.k for r in reqs], [r.part for r in reqs],
                                    eps=np.array([r.eps for r in reqs]))
    res = session.refine(default_config(rounds=reqs[0].rounds, subrounds=subrounds, flags=flags))
    parts = session.partition_instances()
    km1 = session.instance_km1()
    for i, r in enumerate(reqs):
        r.result = parts[i]
        r.km1 = int(km1[i])
    return res.pins_processed


class RefineServer:
    """Continuous batching over `slots` concurrent batched sessions.

    `session_factory(device)` and `runner(session, requests, subrounds)` default to
    lpgpu sessions and `_run_batch`; `footprint(request, subrounds)` defaults to
    lpgpu_estimate_footprint. Tests replace them to check the scheduling alone.
    """

    def __init__(self, device=0, slots=2, budget_bytes=150 << 30, subrounds=7, max_batch=4096,
                 session_factory=Session, runner=_run_batch, footprint=None, max_batch_pins=None):
        self.device = device
        self.slots = slots
        self.budget = budget_bytes
        self.subrounds = subrounds
        self.max_batch = max_batch
        # a batch stops growing once it holds this many pins (None: memory budget only);
        # smaller batches finish their first requests sooner at some cost in throughput
        self.max_batch_pins = max_batch_pins
        self._runner = runner
        self._footprint = footprint or (lambda r, s: r.footprint(s))
        self._cv = threading.Condition()
        self._queue = []
        self._held = [0] * slots
        self._closed = False
        self.stats = ServeStats()
        self.errors = []
        self._t0 = None
        self._threads = []
        self._sessions = [session_factory(device) for _ in range(slots)]

    def now(self):
        return time.perf_counter() - self._t0

    def start(self):
        self._t0 = time.perf_counter()
        for s in range(self.slots):
            t = threading.Thread(target=self._worker, args=(s,), daemon=True)
            t.start()
            self._threads.append(t)

    def submit(self, req: Request):
        with self._cv:
            if self._footprint(req, self.subrounds) > self.budget:
                self.stats.rejected += 1
                req.finish = -1.0
                return False
            self._queue.append(req)
            self._cv.notify_all()
            return True

    def close(self):
        with self._cv:
            self._closed = True
            self._cv.notify_all()
        for t in self._threads:
            t.join()
        for s in self._sessions:
            s.close()

    def _admit(self, slot):
        """Takes waiting requests in arrival order while they fit the memory left."""
        free = self.budget - sum(h for i, h in enumerate(self._held) if i != slot)
        take, used, pins = [], 0, 0
        rounds = self._queue[0].rounds if self._queue else 0
        for r in list(self._queue):
            if r.rounds != rounds:  # a batch runs one round count for all its requests
                continue
            f = self._footprint(r, self.subrounds)
            if len(take) >= self.max_batch or used + f > free:
                break
            if take and self.max_batch_pins is not None and pins + r.hg.num_pins > self.max_batch_pins:
                break
            take.append(r)
            used += f
            pins += r.hg.num_pins
        for r in take:
            self._queue.remove(r)
        self._held[slot] = used
        return take

    def _worker(self, slot):
        session = self._sessions[slot]
        while True:
            with self._cv:
                while not self._queue and not self._closed:
                    self._cv.wait()
                if not self._queue and self._closed:
                    return
                batch = self._admit(slot)
                if not batch:  # the head request waits for memory held by other slots
                    self._cv.wait(0.001)
                    continue
            t = self.now()
            for r in batch:
                r.start, r.slot, r.batch_size = t, slot, len(batch)
            try:
                pins = self._runner(session, batch, self.subrounds)
            except Exception as exc:  # the batch fails as a whole; the slot keeps serving
                with self._cv:
                    self.errors.append((tuple(r.rid for r in batch), exc))
                    for r in batch:
                        r.finish = -1.0
                    self._held[slot] = 0
                    self._cv.notify_all()
                continue
            t = self.now()
            with self._cv:
                for r in batch:
                    r.finish = t
                    self.stats.latencies.append(r.latency)
                self.stats.batch_sizes.append(len(batch))
                self.stats.pins += pins
                self._held[slot] = 0
                self._cv.notify_all()


def replay(server: RefineServer, requests):
    """Submits requests at their arrival times (seconds from start) and waits for all."""
    server.start()
    for r in sorted(requests, key=lambda r: r.arrival):
        delay = r.arrival - server.now()
        if delay > 0:
            time.sleep(delay)
        server.submit(r)
    server.close()
    done = [r.finish for r in requests if r.finish is not None and r.finish >= 0]
    server.stats.wall = max(done) if done else 0.0
    return server.stats


def plain_loop(requests, device=0, subrounds=7, flags=FLAG_NO_GRAPH):
    """Baseline: one request at a time in arrival order on one session."""
    stats = ServeStats()
    t0 = time.perf_counter()
    with Session(device) as s:
        for r in sorted(requests, key=lambda r: r.arrival):
            now = time.perf_counter() - t0
            if now < r.arrival:
                time.sleep(r.arrival - now)
            r.start = time.perf_counter() - t0
            s.upload(r.hg)
            s.set_partition(r.k, r.part, eps=r.eps)
            res = s.refine(default_config(rounds=r.rounds, subrounds=subrounds, flags=flags))
            r.result = s.partition()
            r.km1 = int(s.metrics()[0])
            r.finish = time.perf_counter() - t0
            r.batch_size = 1
            stats.latencies.append(r.latency)
            stats.batch_sizes.append(1)
            stats.pins += res.pins_processed
    stats.wall = time.perf_counter() - t0
    return stats


def poisson_arrivals(count, rate, seed):
    rng = np.random.default_rng([seed, 7])
    return np.cumsum(rng.exponential(1.0 / rate, size=count))

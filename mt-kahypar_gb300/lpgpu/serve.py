"""Continuous batching of refine requests at round granularity.

Requests (hypergraph, partition, k, eps, rounds) arrive over time; a
request's hypergraph and partition state stay on the device from admission to
completion.

* Small requests (at most `large_pins` pins and k <= 64) each get a session
  from a pool and join the stepper's running set at the next round boundary.
  Every step runs one LP round of every running request in one persistent
  launch (lpgpu_stepper_launch). While a step runs, the requests admitted for
  the next one are uploaded on their own streams; after it, finished requests
  leave and their partitions are read back. A request never waits for the
  remaining rounds of another: it joins after at most one round and leaves as
  soon as its own rounds are done.
* Large requests go to `solo_slots` lanes that refine one request at a time
  with the multi-launch pipeline on their own streams, concurrently with the
  stepper.

Admission is by device-memory footprint (lpgpu_estimate_footprint) against the
budget: admitted requests count with their estimate, idle pooled sessions with
the memory they still hold (they are released when a request needs it).
Each request's result is exactly what refining it alone gives (tested).

`plain_loop` is the baseline: one request at a time, in arrival order, one
session call sequence per request.
"""
from __future__ import annotations

import json
import threading
import time
from dataclasses import dataclass, field

import numpy as np

from . import (FLAG_NO_GRAPH, PERSISTENT_MAX_K, TUNING_PATH, Session, Stepper, default_config,
               estimate_footprint)


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
    lane: str = None      # "stepped" or "solo"
    batch_size: int = None  # requests in its first step (stepped) or 1 (solo)

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
    steps: int = 0
    solo: int = 0

    def summary(self):
        lat = np.array(self.latencies) if self.latencies else np.zeros(1)
        return {"requests": len(self.latencies), "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3), "mean_ms": float(lat.mean() * 1e3),
                "wall_s": self.wall, "pins_per_s": self.pins / self.wall if self.wall > 0 else 0.0,
                "req_per_s": len(self.latencies) / self.wall if self.wall > 0 else 0.0,
                "mean_batch": float(np.mean(self.batch_sizes)) if self.batch_sizes else 0.0,
                "steps": self.steps, "solo": self.solo, "rejected": self.rejected}


def default_large_pins():
    """Pins above which a request is refined alone: the largest mean instance
    size for which the tuning table chose persistent rounds (1,000,000 without
    a table)."""
    try:
        with open(TUNING_PATH) as f:
            rows = [r for r in json.load(f)["entries"] if r["mode"] == 1]
        return max(int(r["max_mean_pins"]) for r in rows) if rows else 0
    except (OSError, ValueError, KeyError):
        return 1_000_000


class DeviceBackend:
    """The device side of the server: a stepper, a pool of stepped sessions,
    and one session per solo lane."""

    def __init__(self, device=0, subrounds=7):
        self.device = device
        self.subrounds = subrounds
        self.stepper = Stepper(device)
        self._idle = []

    def cfg(self, r, flags=FLAG_NO_GRAPH):
        return default_config(rounds=r.rounds, subrounds=self.subrounds, flags=flags)

    # stepped lane (one thread)
    def acquire(self):
        return self._idle.pop() if self._idle else Session(self.device)

    def release(self, s):
        self._idle.append(s)

    def idle_bytes(self):
        return sum(s.footprint() for s in self._idle)

    def drop_idle(self):
        while self._idle:
            self._idle.pop().close()

    def begin(self, s, r):
        s.upload(r.hg)
        s.set_partition(r.k, r.part, eps=r.eps)
        s.begin_rounds(self.cfg(r))

    def launch(self, sessions):
        self.stepper.launch(sessions)

    def wait(self):
        return self.stepper.wait()

    def finish(self, s, r):
        res = s.end_rounds()
        r.result = s.partition()
        r.km1 = int(res.km1_after)
        return res.pins_processed

    # solo lanes (one session per lane thread)
    def solo_session(self):
        return Session(self.device)

    def solo(self, s, r):
        s.upload(r.hg)
        s.set_partition(r.k, r.part, eps=r.eps)
        res = s.refine(self.cfg(r))
        r.result = s.partition()
        r.km1 = int(res.km1_after)
        return res.pins_processed

    def close(self):
        self.drop_idle()
        self.stepper.close()


class RefineServer:
    """Round-granular continuous batching; see the module docstring.

    `backend` defaults to DeviceBackend and `footprint(request, subrounds)` to
    lpgpu_estimate_footprint; tests replace both to check the scheduling alone.
    """

    def __init__(self, device=0, budget_bytes=150 << 30, subrounds=7, solo_slots=1, large_pins=None,
                 max_running=4096, backend=None, footprint=None):
        self.budget = budget_bytes
        self.subrounds = subrounds
        self.solo_slots = solo_slots
        self.large_pins = default_large_pins() if large_pins is None else large_pins
        self.max_running = max_running
        self.backend = backend or DeviceBackend(device, subrounds)
        self._footprint = footprint or (lambda r, s: r.footprint(s))
        self._cv = threading.Condition()
        self._queue = []
        self._held = 0         # estimated bytes of admitted requests
        self._idle_bytes = 0   # bytes idle pooled sessions hold
        self._closed = False
        self.stats = ServeStats()
        self.errors = []
        self._t0 = None
        self._threads = []

    def now(self):
        return time.perf_counter() - self._t0

    def stepped(self, r):
        return r.hg.num_pins <= self.large_pins and r.k <= PERSISTENT_MAX_K

    def start(self):
        self._t0 = time.perf_counter()
        lanes = [self._stepper_lane] + [self._solo_lane] * self.solo_slots
        for fn in lanes:
            t = threading.Thread(target=fn, daemon=True)
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
        self.backend.close()

    # -------------------------------------------------------------- lanes

    def _take(self, stepped, limit):
        """Waiting requests of one lane, in arrival order, while they fit the
        memory left (call with the lock held); a request that does not fit
        waits, later ones may still be taken."""
        take = []
        free = self.budget - self._held - self._idle_bytes
        for r in list(self._queue):
            if len(take) >= limit:
                break
            if self.stepped(r) != stepped:
                continue
            f = self._footprint(r, self.subrounds)
            if f > free:
                continue
            take.append(r)
            free -= f
            self._held += f
        for r in take:
            self._queue.remove(r)
        return take

    def _waiting(self, stepped):
        return any(self.stepped(r) == stepped for r in self._queue)

    def _done(self, r, pins):
        with self._cv:
            r.finish = self.now()
            self.stats.latencies.append(r.latency)
            self.stats.pins += pins
            self._held -= self._footprint(r, self.subrounds)
            self._cv.notify_all()

    def _fail(self, reqs, exc):
        with self._cv:
            self.errors.append((tuple(r.rid for r in reqs), exc))
            for r in reqs:
                r.finish = -1.0
                self._held -= self._footprint(r, self.subrounds)
            self._cv.notify_all()

    def _stepper_lane(self):
        be = self.backend
        running = []  # (request, session)
        while True:
            with self._cv:
                admit = self._take(True, self.max_running - len(running))
                if not admit and not running:
                    if self._closed and not self._waiting(True):
                        return
                    if self._waiting(True) and self._idle_bytes > 0:
                        be.drop_idle()  # waiting requests need the memory idle sessions hold
                        self._idle_bytes = 0
                        continue
                    self._cv.wait(0.002)
                    continue
            try:
                if running:
                    be.launch([s for _, s in running])
            except Exception as exc:  # the step fails its requests; their sessions are dropped
                self._fail([r for r, _ in running], exc)
                running = []
            joined = []
            for r in admit:  # uploads overlap the running step on their own streams
                r.start, r.lane = self.now(), "stepped"
                s = be.acquire()
                try:
                    be.begin(s, r)
                except Exception as exc:
                    self._fail([r], exc)
                    be.release(s)
                    continue
                joined.append((r, s))
            if running:
                try:
                    done = be.wait()
                    self.stats.steps += 1
                except Exception as exc:
                    self._fail([r for r, _ in running], exc)
                    done, running = [], []
                keep = []
                for (r, s), d in zip(running, done):
                    if not d:
                        keep.append((r, s))
                        continue
                    try:
                        pins = be.finish(s, r)
                    except Exception as exc:
                        self._fail([r], exc)
                    else:
                        self._done(r, pins)
                    be.release(s)
                running = keep
            for r, s in joined:
                r.batch_size = len(running) + len(joined)
                self.stats.batch_sizes.append(r.batch_size)
                if r.rounds > 0:
                    running.append((r, s))
                else:  # nothing to run
                    self._done(r, be.finish(s, r))
                    be.release(s)
            with self._cv:
                self._idle_bytes = be.idle_bytes()
                self._cv.notify_all()

    def _solo_lane(self):
        be = self.backend
        s = None
        while True:
            with self._cv:
                while True:
                    take = self._take(False, 1)
                    if take or (self._closed and not self._waiting(False)):
                        break
                    self._cv.wait(0.002)
            if not take:
                if s is not None:
                    s.close()
                return
            r = take[0]
            r.start, r.lane, r.batch_size = self.now(), "solo", 1
            try:
                if s is None:
                    s = be.solo_session()
                pins = be.solo(s, r)
            except Exception as exc:
                self._fail([r], exc)
                continue
            with self._cv:
                self.stats.solo += 1
                self.stats.batch_sizes.append(1)
            self._done(r, pins)


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


__all__ = ["Request", "ServeStats", "RefineServer", "DeviceBackend", "replay", "plain_loop",
           "poisson_arrivals", "default_large_pins"]

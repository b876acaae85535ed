"""Scheduling of the round-granular refine server, with a fake backend in
place of the device: admission by memory budget, joining a running set at a
round boundary, leaving it when a request's own rounds are done, the solo lane
for large requests, rejection and failure isolation."""
import threading
import time
from types import SimpleNamespace

import numpy as np
import pytest

serve = pytest.importorskip("lpgpu.serve")


class FakeSession:
    def __init__(self):
        self.left = 0
        self.rid = None
        self.closed = False

    def close(self):
        self.closed = True


class FakeBackend:
    """Counts rounds per request; records every step's running set and the
    memory in use while steps and solo refinements run."""

    def __init__(self, fail_begin=None, solo_delay=0.003, step_delay=0.001):
        self.lock = threading.Lock()
        self.steps = []            # rids of every step
        self.solo_runs = []
        self.idle = []
        self.sessions = []
        self.fail_begin = fail_begin
        self.solo_delay = solo_delay
        self.step_delay = step_delay
        self.launched = None
        self.concurrent = 0
        self.peak_concurrent = 0

    def acquire(self):
        if self.idle:
            return self.idle.pop()
        s = FakeSession()
        self.sessions.append(s)
        return s

    def release(self, s):
        self.idle.append(s)

    def idle_bytes(self):
        return 0

    def drop_idle(self):
        self.idle.clear()

    def begin(self, s, r):
        if r.rid == self.fail_begin:
            raise RuntimeError("planted failure")
        s.left, s.rid = r.rounds, r.rid

    def _enter(self):
        with self.lock:
            self.concurrent += 1
            self.peak_concurrent = max(self.peak_concurrent, self.concurrent)

    def _leave(self):
        with self.lock:
            self.concurrent -= 1

    def launch(self, sessions):
        assert all(s.left > 0 for s in sessions)
        self.launched = sessions
        self.steps.append([s.rid for s in sessions])
        self._enter()

    def wait(self):
        time.sleep(self.step_delay)
        for s in self.launched:
            s.left -= 1
        self._leave()
        return [s.left == 0 for s in self.launched]

    def finish(self, s, r):
        r.km1 = 7 * r.rid
        r.result = np.full(r.hg.n, r.rid, np.int32)
        return r.hg.num_pins

    def solo_session(self):
        return FakeSession()

    def solo(self, s, r):
        self._enter()
        time.sleep(self.solo_delay)
        self._leave()
        with self.lock:
            self.solo_runs.append(r.rid)
        r.km1 = 7 * r.rid
        r.result = np.full(r.hg.n, r.rid, np.int32)
        return r.hg.num_pins

    def close(self):
        pass


def _requests(count, seed, rounds=(2, 8), spacing=0.0003, big_every=0):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(10, 100))
        pins = 4 * n if not (big_every and i % big_every == 0) else 10 ** 7
        out.append(serve.Request(i, SimpleNamespace(n=n, m=n, num_pins=pins), 4, 0.03, None,
                                 int(rng.choice(rounds)), arrival=i * spacing))
    return out


def _server(be, budget=400, solo_slots=1, large_pins=10 ** 6):
    return serve.RefineServer(budget_bytes=budget, solo_slots=solo_slots, large_pins=large_pins, backend=be,
                              footprint=lambda r, s: r.hg.n)


def test_every_request_served_once_within_budget():
    reqs = _requests(200, 1)
    be = FakeBackend()
    srv = _server(be)
    peak = [0]
    orig = srv._take

    def take(stepped, limit):
        out = orig(stepped, limit)
        peak[0] = max(peak[0], srv._held)
        return out

    srv._take = take
    st = serve.replay(srv, reqs)
    assert peak[0] <= 400
    assert all(r.km1 == 7 * r.rid and r.finish >= r.start >= 0 and r.latency >= 0 for r in reqs)
    assert st.summary()["requests"] == len(reqs) and st.pins == sum(r.hg.num_pins for r in reqs)
    # every stepped request ran exactly its own number of rounds
    rounds = {}
    for step in be.steps:
        for rid in step:
            rounds[rid] = rounds.get(rid, 0) + 1
    assert all(rounds[r.rid] == r.rounds for r in reqs)


def test_requests_join_a_running_set_and_leave_when_done():
    """A request arriving while a long one runs joins at the next round
    boundary and leaves after its own rounds, before the long one ends."""
    long = serve.Request(0, SimpleNamespace(n=10, m=10, num_pins=40), 4, 0.03, None, 40, arrival=0.0)
    short = [serve.Request(i, SimpleNamespace(n=10, m=10, num_pins=40), 4, 0.03, None, 2, arrival=0.01 * i)
             for i in range(1, 4)]
    be = FakeBackend(step_delay=0.002)
    serve.replay(_server(be), [long] + short)
    mixed = [s for s in be.steps if 0 in s and len(s) > 1]
    assert mixed, "no step ran the long request together with a later one"
    for r in short:
        assert r.finish < long.finish
        assert r.lane == "stepped"
    last = max(i for i, s in enumerate(be.steps) if 0 in s)
    assert all(len(s) == 1 for s in be.steps[last - 5:last + 1])  # the short ones had left


def test_large_requests_go_to_the_solo_lane_concurrently():
    reqs = _requests(60, 4, big_every=5)
    be = FakeBackend(solo_delay=0.01)
    serve.replay(_server(be, budget=10 ** 6, solo_slots=2), reqs)
    big = sorted(r.rid for r in reqs if r.hg.num_pins > 10 ** 6)
    assert sorted(be.solo_runs) == big
    assert all(r.lane == ("solo" if r.rid in big else "stepped") for r in reqs)
    assert be.peak_concurrent >= 2  # solo work overlapped the stepper or another solo lane


def test_rejects_request_larger_than_budget():
    reqs = _requests(10, 3)
    reqs[4].hg = SimpleNamespace(n=1000, m=1, num_pins=1)
    be = FakeBackend()
    st = serve.replay(_server(be), reqs)
    assert st.rejected == 1 and reqs[4].finish == -1.0 and reqs[4].km1 is None
    assert all(r.km1 == 7 * r.rid for r in reqs if r.rid != 4)


def test_failed_request_does_not_stop_the_server():
    reqs = _requests(60, 9)
    be = FakeBackend(fail_begin=17)
    srv = _server(be)
    serve.replay(srv, reqs)
    assert len(srv.errors) == 1 and srv.errors[0][0] == (17,)
    for r in reqs:
        assert r.finish == -1.0 if r.rid == 17 else r.km1 == 7 * r.rid
    assert srv._held == 0


def test_poisson_arrivals_rate():
    a = serve.poisson_arrivals(20000, 2000.0, 1)
    assert np.all(np.diff(a) > 0)
    assert abs(20000 / a[-1] - 2000.0) < 60.0

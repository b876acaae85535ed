"""Scheduling of the continuous-batching refine server, with a fake session and
runner in place of the device: admission by memory budget, arrival order,
one round count per batch, rejection, failure isolation."""
import threading
import time
from types import SimpleNamespace

import numpy as np
import pytest

serve = pytest.importorskip("lpgpu.serve")


class FakeSession:
    def __init__(self, device):
        self.closed = False

    def close(self):
        self.closed = True


class Recorder:
    """Runner that checks the budget across slots while batches run."""

    def __init__(self, budget, fail_rid=None, delay=0.002):
        self.lock = threading.Lock()
        self.running = 0
        self.peak = 0
        self.batches = []
        self.budget = budget
        self.fail_rid = fail_rid
        self.delay = delay

    def __call__(self, session, reqs, subrounds):
        use = sum(r.hg.n for r in reqs)
        with self.lock:
            self.running += use
            self.peak = max(self.peak, self.running)
            self.batches.append([r.rid for r in reqs])
        try:
            time.sleep(self.delay)
            if self.fail_rid is not None and any(r.rid == self.fail_rid for r in reqs):
                raise RuntimeError("planted failure")
            for r in reqs:
                r.km1 = 7 * r.rid
                r.result = np.full(r.hg.n, r.rid, np.int32)
            return sum(r.hg.n for r in reqs)
        finally:
            with self.lock:
                self.running -= use


def _requests(count, seed, rounds=(8,), spacing=0.0002):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(10, 100))
        out.append(serve.Request(i, SimpleNamespace(n=n, m=n, num_pins=4 * n), 4, 0.03, None,
                                 int(rng.choice(rounds)), arrival=i * spacing))
    return out


def _server(rec, slots=3, budget=400):
    return serve.RefineServer(slots=slots, budget_bytes=budget, session_factory=FakeSession,
                              runner=rec, footprint=lambda r, s: r.hg.n)


@pytest.mark.parametrize("slots", [1, 2, 4])
def test_every_request_served_once_within_budget(slots):
    reqs = _requests(200, slots)
    rec = Recorder(400)
    st = serve.replay(_server(rec, slots=slots), reqs)
    served = sorted(i for b in rec.batches for i in b)
    assert served == list(range(len(reqs)))
    assert rec.peak <= 400
    assert all(r.km1 == 7 * r.rid and r.finish >= r.start >= 0 and r.latency >= 0 for r in reqs)
    assert st.summary()["requests"] == len(reqs) and st.pins == sum(r.hg.n for r in reqs)
    assert sum(st.batch_sizes) == len(reqs)


def test_single_slot_keeps_arrival_order_and_round_groups():
    reqs = _requests(120, 5, rounds=(5, 8))
    rec = Recorder(400)
    serve.replay(_server(rec, slots=1), reqs)
    by_id = {r.rid: r for r in reqs}
    for b in rec.batches:
        assert len({by_id[i].rounds for i in b}) == 1
        assert b == sorted(b)
    # requests of the same round count start in arrival order
    for rounds in (5, 8):
        starts = [by_id[i].start for i in sorted(by_id) if by_id[i].rounds == rounds]
        assert starts == sorted(starts)


def test_rejects_request_larger_than_budget():
    reqs = _requests(10, 3)
    reqs[4].hg = SimpleNamespace(n=1000, m=1, num_pins=1)
    rec = Recorder(400)
    st = serve.replay(_server(rec, slots=2), reqs)
    assert st.rejected == 1 and reqs[4].finish == -1.0 and reqs[4].km1 is None
    assert sorted(i for b in rec.batches for i in b) == [i for i in range(10) if i != 4]


def test_failed_batch_does_not_stop_the_server():
    reqs = _requests(60, 9)
    rec = Recorder(400, fail_rid=17)
    srv = _server(rec, slots=2)
    serve.replay(srv, reqs)
    assert len(srv.errors) == 1 and 17 in srv.errors[0][0]
    failed = set(srv.errors[0][0])
    for r in reqs:
        if r.rid in failed:
            assert r.finish == -1.0
        else:
            assert r.km1 == 7 * r.rid
    assert all(s.closed for s in srv._sessions)


def test_poisson_arrivals_rate():
    a = serve.poisson_arrivals(20000, 2000.0, 1)
    assert np.all(np.diff(a) > 0)
    assert abs(20000 / a[-1] - 2000.0) < 60.0


def test_pin_cap_limits_batches():
    reqs = _requests(100, 11)
    for r in reqs:
        r.hg.num_pins = 10
    rec = Recorder(10 ** 6)
    srv = serve.RefineServer(slots=1, budget_bytes=10 ** 6, session_factory=FakeSession, runner=rec,
                             footprint=lambda r, s: r.hg.n, max_batch_pins=35)
    serve.replay(srv, reqs)
    assert max(len(b) for b in rec.batches) <= 3
    assert sorted(i for b in rec.batches for i in b) == list(range(100))

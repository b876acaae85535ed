"""Served refinement on the device: requests refined by the round-granular
server (stepped lane and solo lanes) end exactly as when each is refined
alone (plain loop and oracle), and a session that joins a running stepper
after some rounds ends as its own refine would."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ["active", "pins", "candidates", "moved", "reverted", "delta", "moved_pins"]


def _requests(serve, gen, count, seed, rate=4000.0):
    arr = serve.poisson_arrivals(count, rate, seed)
    out = []
    for i in range(count):
        x = gen.served_request(seed, i, lo=512, hi=20000, ks=(2, 3, 8, 33), rounds=4)
        out.append(serve.Request(i, x.hg, x.k, x.eps, x.part, x.rounds, float(arr[i])))
    return out


@pytest.mark.parametrize("solo_slots", [1, 2])
def test_served_equals_plain_loop(lp, orc, solo_slots):
    from lpgpu import gen, serve
    rs = _requests(serve, gen, 32, 3 + solo_slots)
    rp = _requests(serve, gen, 32, 3 + solo_slots)
    large = int(np.median([r.hg.num_pins for r in rs]))  # half the requests go to the solo lanes
    srv = serve.RefineServer(solo_slots=solo_slots, subrounds=8, large_pins=large)
    st = serve.replay(srv, rs)
    assert not srv.errors
    serve.plain_loop(rp, subrounds=8)
    s = st.summary()
    assert s["requests"] == 32 and 0 < s["solo"] < 32 and s["steps"] > 0
    assert max(st.batch_sizes) > 1  # stepped requests shared rounds
    for a, b in zip(rs, rp):
        assert a.km1 == b.km1
        assert np.array_equal(a.result, b.result), f"request {a.rid} ({a.lane})"
    for a in rs[:4]:
        x = gen.served_request(3 + solo_slots, a.rid, lo=512, hi=20000, ks=(2, 3, 8, 33), rounds=4)
        ref, _ = orc.lp_sync(x.hg, x.k, x.lmax, x.part, perfect=x.perfect, rounds=4, subrounds=8,
                             revert=1, rollback=1, zero_gain=1)
        assert np.array_equal(a.result, ref)


def test_session_joining_a_running_stepper(lp):
    """Sessions A and B run two rounds, then C joins; every session ends with
    the partition, round statistics and result of its own refine call."""
    from lpgpu import gen
    xs = [gen.served_request(21, i, lo=800, hi=6000, ks=(2, 8, 33), rounds=6) for i in range(3)]
    cfgs = [lp.default_config(rounds=x.rounds, subrounds=7) for x in xs]
    alone = []
    for x, cfg in zip(xs, cfgs):
        with lp.Session(0) as s:
            s.upload(x.hg)
            s.set_partition(x.k, x.part, eps=x.eps)
            r = s.refine(cfg)
            alone.append((r, s.partition(), s.round_stats()))
    sessions = [lp.Session(0) for _ in xs]
    with lp.Stepper(0) as st:
        def begin(i):
            sessions[i].upload(xs[i].hg)
            sessions[i].set_partition(xs[i].k, xs[i].part, eps=xs[i].eps)
            sessions[i].begin_rounds(cfgs[i])
        begin(0)
        begin(1)
        running = [0, 1]
        rounds = 0
        out = {}
        while running:
            if rounds == 2:
                begin(2)
                running.append(2)
            done = st.round([sessions[i] for i in running])
            rounds += 1
            for i, d in zip(list(running), done):
                if d:
                    out[i] = (sessions[i].end_rounds(), sessions[i].partition(), sessions[i].round_stats())
                    running.remove(i)
    for i in range(3):
        r, part, stats = out[i]
        ra, pa, sa = alone[i]
        assert np.array_equal(part, pa), f"session {i}"
        assert [[x[k] for k in KEYS] for x in stats] == [[x[k] for k in KEYS] for x in sa]
        assert (r.km1_before, r.km1_after, r.delta, r.moves, r.rounds) == \
               (ra.km1_before, ra.km1_after, ra.delta, ra.moves, ra.rounds)
    for s in sessions:
        s.close()


def test_stepper_rejects_bad_lists(lp):
    from lpgpu import gen
    x = gen.served_request(5, 0, lo=600, hi=700, ks=(4,), rounds=2)
    with lp.Session(0) as s, lp.Stepper(0) as st:
        s.upload(x.hg)
        s.set_partition(x.k, x.part)
        with pytest.raises(lp.LpgpuError):
            st.launch([s])  # not begun
        s.begin_rounds(lp.default_config(rounds=1))
        with pytest.raises(lp.LpgpuError):
            st.launch([s, s])  # listed twice
        assert list(st.round([s])) == [True]
        with pytest.raises(lp.LpgpuError):
            st.launch([s])  # no round left
        r = s.end_rounds()
        assert r.km1_after == r.km1_before + r.delta


def test_graph_and_direct_launches_agree(lp):
    from lpgpu import gen
    x = gen.served_request(11, 0, lo=4000, hi=5000, ks=(8,), rounds=4)
    out = []
    for flags in (0, lp.FLAG_NO_GRAPH):
        with lp.Session(0) as s:
            s.upload(x.hg)
            s.set_partition(x.k, x.part, eps=x.eps)
            r = s.refine(lp.default_config(rounds=4, subrounds=8, flags=flags))
            out.append((s.partition(), r.km1_after, r.delta))
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1:] == out[1][1:]

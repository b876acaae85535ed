"""Device path vs the CPU oracle, bit-exact (integer work: no tolerance).

Every test goes through the C ABI (liblpgpu.so via ctypes)."""
import numpy as np
import pytest

from conftest import load_golden, seven_vertex_fixture

pytestmark = pytest.mark.gpu

INF = np.iinfo(np.int32).max
GOLDEN = ["twocenters", "contracted_unweighted_ibm01", "contracted_ibm01",
          "hypergraph_with_node_and_edge_weights", "karate_club.graph", "test_instance",
          "powersim.mtx"]


def session(lp, hg, k, part, lmax=None, perfect=None, eps=0.03):
    s = lp.Session(0)
    s.upload(hg)
    s.set_partition(k, part, eps=eps, lmax=lmax, perfect=perfect)
    return s


def check_state(orc, s, hg, k, part):
    phi, conn, bw = orc.init_partition(hg, k, part)
    assert np.array_equal(s.pin_counts(), phi)
    assert np.array_equal(s.connectivity(), conn)
    assert np.array_equal(s.block_weights(), bw)
    km1, cut = orc.metrics(hg, k, conn)
    dk, dc, _ = s.metrics()
    assert (dk, dc) == (km1, cut)


@pytest.mark.parametrize("name", GOLDEN)
def test_golden_state_and_moves(lp, orc, name):
    hg, d = load_golden(name)
    for k in (2, 3, 8):
        part = d[f"k{k}_part"]
        s = session(lp, hg, k, part, lmax=d[f"k{k}_lmax"], perfect=d[f"k{k}_perfect"])
        assert np.array_equal(s.pin_counts(), d[f"k{k}_phi"])
        assert np.array_equal(s.connectivity(), d[f"k{k}_conn"])
        assert np.array_equal(s.block_weights(), d[f"k{k}_bw"])
        km1, cut, _ = s.metrics()
        assert (km1, cut) == (int(d[f"k{k}_km1"]), int(d[f"k{k}_cut"]))
        to, gain, border = s.best_moves()
        assert np.array_equal(to, d[f"k{k}_to"])
        assert np.array_equal(gain, d[f"k{k}_gain"])
        assert np.array_equal(border, d[f"k{k}_border"])
        ben, pen = s.gain_cache()
        assert np.array_equal(ben, d[f"k{k}_benefit"])
        assert np.array_equal(pen, d[f"k{k}_penalty"])
        cfg = lp.default_config(rounds=5, subrounds=4, revert=1, rollback=1, rebalancing=1)
        r = s.refine(cfg)
        assert np.array_equal(s.partition(), d[f"k{k}_lp_part"])
        stats = s.round_stats()
        assert [st["delta"] for st in stats] == d[f"k{k}_lp_delta"].tolist()
        assert r.km1_after == r.km1_before + r.delta
        s.close()


def test_incidence_matches_stable_transpose(lp, orc):
    from lpgpu import gen
    inst = gen.plain_small(seed=1)
    hg = inst.hg
    s = session(lp, hg, inst.k, inst.part)
    vo, ie = s.incidence(hg.num_pins)
    assert np.array_equal(vo, hg.vtx_off)
    for v in range(hg.n):
        a, b = vo[v], vo[v + 1]
        assert np.array_equal(np.sort(ie[a:b]), hg.inets[a:b])
    s.close()


KM1_CASES = [
    (2, [1, 0, 0, 0, 0, 1, 1], 0, (0, -2)),
    (2, [0, 0, 0, 1, 0, 1, 1], 3, (0, -1)),
    (2, [0, 0, 0, 0, 0, 1, 1], 4, (0, 0)),
    (4, [0, 1, 2, 3, 3, 1, 2], 0, (1, -1)),
    (4, [0, 3, 1, 2, 2, 0, 3], 6, (0, -1)),
    (4, [0, 3, 1, 2, 2, 0, 3], 3, (2, 0)),
]


@pytest.mark.parametrize("k,part,v,expected", KM1_CASES)
def test_km1_policy_known_answers_on_device(lp, k, part, v, expected):
    """gain_policy_test.cc:63-276 through the C ABI."""
    hg = seven_vertex_fixture()
    s = session(lp, hg, k, np.array(part, np.int32), lmax=np.full(k, INF, np.int64))
    to, gain, _ = s.best_moves()
    assert (to[v], gain[v]) == expected
    s.close()


@pytest.mark.parametrize("moves,delta", [
    ([(0, 1, 0)], -2),
    ([(3, 1, 0)], -1),
])
def test_km1_delta_known_answers_on_device(lp, moves, delta):
    hg = seven_vertex_fixture()
    part = [1, 0, 0, 0, 0, 1, 1] if moves[0][0] == 0 else [0, 0, 0, 1, 0, 1, 1]
    s = session(lp, hg, 2, np.array(part, np.int32))
    v, f, t = zip(*moves)
    assert s.apply_moves(v, f, t) == delta
    s.close()


CONCURRENT = [
    [(0, 0, 1), (3, 1, 2), (2, 0, 2), (5, 2, 1), (6, 2, 0), (4, 1, 2)],
    [(0, 0, 1), (1, 0, 2)],
    [(3, 1, 2), (6, 2, 0)],
    [(0, 0, 1), (2, 0, 2), (4, 1, 0), (6, 2, 1), (1, 0, 2), (3, 1, 0), (5, 2, 1)],
    [(0, 0, 1), (3, 1, 0), (6, 2, 0), (1, 0, 2), (2, 0, 1), (4, 1, 0), (5, 2, 1)],
]


@pytest.mark.parametrize("moves", CONCURRENT)
def test_concurrent_moves_on_device(lp, orc, moves):
    """partitioned_hypergraph_test.cc:181-378: moves applied concurrently on the
    device give the pin counts, connectivity sets and part weights of the
    sequential oracle, and the attributed delta equals the km1 change."""
    hg = seven_vertex_fixture()
    base = np.array([0, 0, 0, 1, 1, 2, 2], np.int32)
    s = session(lp, hg, 3, base)
    km0 = s.metrics()[0]
    v, f, t = zip(*moves)
    d = s.apply_moves(v, f, t)
    p = base.copy()
    p[list(v)] = list(t)
    check_state(orc, s, hg, 3, p)
    assert np.array_equal(s.partition(), p)
    assert s.metrics()[0] == km0 + d
    s.close()


@pytest.mark.parametrize("seed", range(8))
@pytest.mark.parametrize("k", [1, 2, 3, 31, 32, 33, 64, 100, 128, 200, 1024])
def test_random_state_and_best_moves(lp, orc, seed, k):
    from lpgpu import gen
    inst = gen.random_small(seed, n=300, m=360, k=k, max_size=12)
    hg, part = inst.hg, inst.part
    s = session(lp, hg, k, part, lmax=inst.lmax, perfect=inst.perfect)
    check_state(orc, s, hg, k, part)
    to, gain, border = s.best_moves()
    eto, egain, eborder = orc.best_moves(hg, k, part, inst.lmax)
    assert np.array_equal(to, eto) and np.array_equal(gain, egain) and np.array_equal(border, eborder)
    if k <= 200:
        ben, pen = s.gain_cache()
        eben, epen = orc.gain_cache(hg, k, part)
        assert np.array_equal(ben, eben) and np.array_equal(pen, epen)
    s.close()


@pytest.mark.parametrize("seed", range(3))
@pytest.mark.parametrize("k", [2, 5, 32, 64, 100, 128, 129])
@pytest.mark.parametrize("weighted", [False, True])
def test_hub_vertices_and_heavy_weights(lp, orc, seed, k, weighted):
    """Tiles that mix light vertices (lane-per-vertex counters) with hub vertices
    of degree > 100 (warp windows), and vertex weights above 16 (feasibility
    computed per lane instead of from the precomputed masks)."""
    from lpgpu import gen
    inst = gen.random_small(seed, n=500, m=600, k=k, max_size=10, weighted=weighted, hubs=5, vw_hi=40)
    hg, part = inst.hg, inst.part
    deg = np.diff(hg.vtx_off)
    assert deg.max() > 100
    s = session(lp, hg, k, part, lmax=inst.lmax, perfect=inst.perfect)
    to, gain, border = s.best_moves()
    eto, egain, eborder = orc.best_moves(hg, k, part, inst.lmax)
    assert np.array_equal(to, eto) and np.array_equal(gain, egain) and np.array_equal(border, eborder)
    s.close()
    for mode in (LP_MODES[1], LP_MODES[3]):
        out = run_both(lp, orc, inst, 4, mode)
        assert_same_run(*out, orc, inst)
        out[0].close()


@pytest.mark.parametrize("weighted", [False, True])
def test_heavy_vertices_above_128_blocks(lp, orc, weighted):
    """k = 200 (8 words per net record): hubs of degree > 1,024 are heavy for the
    warp-window sweep, so they lead their sub-round's list and run on the
    sweep's dedicated CTAs (LP rounds) or in k_sweep_heavy (best-move query)."""
    from lpgpu import gen
    inst = gen.random_small(7, n=3000, m=4000, k=200, max_size=6, weighted=weighted, hubs=2, hub_frac=0.4,
                            vw_hi=3)
    hg, part = inst.hg, inst.part
    assert np.diff(hg.vtx_off).max() > 1024
    s = session(lp, hg, inst.k, part, lmax=inst.lmax, perfect=inst.perfect)
    to, gain, border = s.best_moves()
    eto, egain, eborder = orc.best_moves(hg, inst.k, part, inst.lmax)
    assert np.array_equal(to, eto) and np.array_equal(gain, egain) and np.array_equal(border, eborder)
    s.close()
    for mode in (LP_MODES[1], LP_MODES[2]):
        out = run_both(lp, orc, inst, 3, mode)
        assert_same_run(*out, orc, inst)
        out[0].close()


def test_every_vertex_heavy(lp, orc):
    """Net weights up to 2,000: w(e) >= 2^8 makes every vertex with an incident
    net heavy for the lane counters, so nearly all of the sweep runs on its
    heavy CTAs (one vertex per CTA) and one CTA walks the rest."""
    from lpgpu import gen
    inst = gen.random_small(3, n=400, m=480, k=6, max_size=7, weighted=True)
    rng = np.random.default_rng(9)
    hg = inst.hg
    w_e = rng.integers(1, 2000, size=hg.m).astype(np.int32)
    w_e[0] = 1999
    heavy = gen.Hypergraph(hg.n, hg.m, hg.net_off, hg.pins, hg.w_v, w_e).with_incidence()
    inst2 = gen.Instance("heavy", heavy, inst.k, inst.eps, inst.part, 4)
    s = session(lp, heavy, inst2.k, inst2.part, lmax=inst2.lmax, perfect=inst2.perfect)
    to, gain, border = s.best_moves()
    eto, egain, eborder = orc.best_moves(heavy, inst2.k, inst2.part, inst2.lmax)
    assert np.array_equal(to, eto) and np.array_equal(gain, egain) and np.array_equal(border, eborder)
    s.close()
    for mode in (LP_MODES[1], LP_MODES[2]):
        out = run_both(lp, orc, inst2, 4, mode)
        assert_same_run(*out, orc, inst2)
        out[0].close()


LP_MODES = [
    dict(subrounds=1, revert=0, rollback=0, rebalancing=1),
    dict(subrounds=1, revert=1, rollback=1, rebalancing=1),
    dict(subrounds=4, revert=1, rollback=0, rebalancing=0),
    dict(subrounds=16, revert=1, rollback=1, rebalancing=1),
    dict(subrounds=64, revert=0, rollback=1, rebalancing=1),
]


def run_both(lp, orc, inst, rounds, mode, threshold=100):
    hg, k = inst.hg, inst.k
    s = session(lp, hg, k, inst.part, lmax=inst.lmax, perfect=inst.perfect)
    cfg = lp.default_config(rounds=rounds, activation_threshold=threshold, **mode)
    r = s.refine(cfg)
    dpart = s.partition()
    dstats = s.round_stats()
    epart, estats = orc.lp_sync(hg, k, inst.lmax, inst.part, perfect=inst.perfect, rounds=rounds,
                                activation_threshold=threshold, subrounds=mode["subrounds"],
                                revert=mode["revert"], rollback=mode["rollback"],
                                zero_gain=mode["rebalancing"])
    return s, r, dpart, dstats, epart, estats


def assert_same_run(s, r, dpart, dstats, epart, estats, orc, inst):
    assert np.array_equal(dpart, epart)
    keys = ["active", "pins", "candidates", "moved", "reverted", "delta"]
    assert [[st[k] for k in keys] for st in dstats] == [[st[k] for k in keys] for st in estats]
    check_state(orc, s, inst.hg, inst.k, epart)
    assert r.km1_after == r.km1_before + r.delta
    # no block ends above its bound, or above its initial weight if it started above
    _, _, bw0 = orc.init_partition(inst.hg, inst.k, inst.part)
    assert (s.block_weights() <= np.maximum(inst.lmax, bw0)).all()


@pytest.mark.parametrize("mode", LP_MODES)
@pytest.mark.parametrize("seed", range(4))
def test_lp_rounds_bit_exact_small(lp, orc, mode, seed):
    from lpgpu import gen
    inst = gen.random_small(seed, n=400, m=480, k=[2, 4, 7, 33][seed], max_size=10)
    out = run_both(lp, orc, inst, 6, mode)
    assert_same_run(*out, orc, inst)
    out[0].close()


@pytest.mark.parametrize("mode", LP_MODES[1:4])
def test_lp_rounds_bit_exact_plain_small(lp, orc, mode):
    """The 16,384-vertex k=2 workload: 5 rounds plus full recompute, bit-exact."""
    from lpgpu import gen
    inst = gen.plain_small(seed=0)
    out = run_both(lp, orc, inst, 5, mode)
    assert_same_run(*out, orc, inst)
    out[0].close()


@pytest.mark.parametrize("threshold", [40, 64, 65, 1000])
@pytest.mark.parametrize("seed", range(2))
def test_activation_of_large_nets(lp, orc, threshold, seed):
    """Nets of up to 200 pins (several 32-pin groups in the stamped-net
    expansion), with activation thresholds below, at and above the 32- and
    64-pin group boundaries."""
    from lpgpu import gen
    inst = gen.random_small(seed, n=1200, m=400, k=[3, 16][seed], max_size=200)
    assert np.diff(inst.hg.net_off).max() > 65
    for mode in (LP_MODES[1], LP_MODES[2]):
        out = run_both(lp, orc, inst, 5, mode, threshold=threshold)
        assert_same_run(*out, orc, inst)
        out[0].close()


@pytest.mark.parametrize("big", [65535, 65536])
def test_pin_count_width_boundary(lp, orc, big):
    """A net of 65,535 pins keeps 16-bit pin counts (two per 32-bit word, a count
    can reach 65,535); one of 65,536 pins switches the session to 32-bit counts.
    Most of the big net starts in block 0, so moves push its counts up to the
    width's limit and down again."""
    from lpgpu import gen
    rng = np.random.default_rng([big, 3])
    n, m_small, k = big + 64, 3000, 3
    sizes = rng.integers(2, 7, size=m_small)
    small = [rng.choice(n, size=s, replace=False) for s in sizes]
    nets = [np.arange(big)] + small
    off = np.zeros(len(nets) + 1, np.int64)
    np.cumsum([len(x) for x in nets], out=off[1:])
    pins = np.concatenate(nets).astype(np.int32)
    hg = gen.Hypergraph(n, len(nets), off, pins, np.ones(n, np.int32), np.ones(len(nets), np.int32)).with_incidence()
    part = np.where(rng.random(n) < 0.9, 0, rng.integers(1, k, size=n)).astype(np.int32)
    inst = gen.Instance("bignet", hg, k, 0.03, part, 3)
    inst.lmax = np.full(k, n, np.int64)  # room for every move, block 0 included
    s = session(lp, hg, k, part, lmax=inst.lmax, perfect=inst.perfect)
    check_state(orc, s, hg, k, part)
    s.close()
    for mode in (LP_MODES[1], LP_MODES[2]):
        out = run_both(lp, orc, inst, 3, mode)
        assert_same_run(*out, orc, inst)
        out[0].close()


def test_quality_against_async_lp(lp, orc):
    """Quality bar: with the default configuration the device's km1 after
    refinement is at most 0.5 % above the reference-style asynchronous LP's
    (oracle, 4 threads), mean over seeds of the 16,384-vertex workload."""
    from lpgpu import gen
    dev, ref = [], []
    for seed in range(3):
        inst = gen.plain_small(seed=seed)
        s = session(lp, inst.hg, inst.k, inst.part, lmax=inst.lmax, perfect=inst.perfect)
        r = s.refine(lp.default_config(rounds=inst.rounds))
        s.close()
        pa, _ = orc.lp_async(inst.hg, inst.k, inst.lmax, inst.perfect, inst.part, rounds=inst.rounds, threads=4,
                             seed=seed)
        _, conn, _ = orc.init_partition(inst.hg, inst.k, pa)
        dev.append(r.km1_after)
        ref.append(orc.metrics(inst.hg, inst.k, conn)[0])
    assert np.mean(dev) <= 1.005 * np.mean(ref), (dev, ref)


def test_refinement_nodes_and_threshold(lp, orc):
    from lpgpu import gen
    inst = gen.random_small(5, n=500, m=600, k=4)
    s = session(lp, inst.hg, inst.k, inst.part, lmax=inst.lmax, perfect=inst.perfect)
    nodes = np.arange(0, 500, 3, dtype=np.int32)
    r = s.refine(lp.default_config(rounds=3, subrounds=2), nodes=nodes)
    st = s.round_stats()
    assert st[0]["active"] == len(nodes)
    assert r.km1_after == r.km1_before + r.delta
    s.close()


def test_edge_cases(lp, orc):
    from lpgpu import gen
    # no nets at all
    hg = gen.Hypergraph(10, 0, np.zeros(1, np.int64), np.zeros(0, np.int32), np.ones(10, np.int32),
                        np.zeros(0, np.int32)).with_incidence()
    s = session(lp, hg, 2, np.arange(10, dtype=np.int32) % 2)
    assert s.metrics()[:2] == (0, 0)
    r = s.refine(lp.default_config())
    assert r.moves == 0 and r.km1_after == 0
    s.close()
    # single-pin nets and isolated vertices are kept and never counted
    off = np.array([0, 1, 3, 4, 6], np.int64)
    pins = np.array([0, 1, 2, 3, 4, 5], np.int32)
    hg = gen.Hypergraph(8, 4, off, pins, np.ones(8, np.int32), np.array([5, 1, 2, 3], np.int32)).with_incidence()
    part = np.array([0, 1, 0, 1, 0, 1, 0, 1], np.int32)
    s = session(lp, hg, 2, part, eps=0.5)
    check_state(orc, s, hg, 2, part)
    s.close()


def test_invalid_arguments_are_rejected(lp):
    from lpgpu import gen
    s = lp.Session(0)
    bad = gen.Hypergraph(4, 1, np.array([0, 2], np.int64), np.array([0, 9], np.int32),
                         np.ones(4, np.int32), np.ones(1, np.int32))
    with pytest.raises(lp.LpgpuError) as e:
        s.upload(bad)
    assert e.value.status == lp.ERR_INVALID_ARG
    with pytest.raises(lp.LpgpuError) as e:
        s.set_partition(2, np.zeros(4, np.int32))
    assert e.value.status == lp.ERR_STATE
    ok = gen.Hypergraph(4, 1, np.array([0, 2], np.int64), np.array([0, 1], np.int32),
                        np.ones(4, np.int32), np.ones(1, np.int32))
    s.upload(ok)
    with pytest.raises(lp.LpgpuError):
        s.set_partition(2, np.array([0, 1, 2, 0], np.int32))
    with pytest.raises(lp.LpgpuError):
        s.set_partition(2000, np.zeros(4, np.int32))
    s.set_partition(2, np.array([0, 1, 0, 1], np.int32))
    with pytest.raises(lp.LpgpuError):
        s.apply_moves([0], [1], [0])   # wrong source block
    s.close()


def test_device_side_input_checks(lp, orc):
    """Per-pin / per-net / per-vertex checks run on the device after the copy;
    each failure is reported as INVALID_ARG and leaves the session usable."""
    from lpgpu import gen
    H = gen.Hypergraph
    ones = lambda k: np.ones(k, np.int32)  # noqa: E731
    cases = [
        ("offsets", H(4, 2, np.array([0, 3, 2], np.int64), np.array([0, 1, 2], np.int32), ones(4), ones(2))),
        ("net weight", H(4, 1, np.array([0, 2], np.int64), np.array([0, 1], np.int32), ones(4),
                         np.array([-1], np.int32))),
        ("vertex weight", H(4, 1, np.array([0, 2], np.int64), np.array([0, 1], np.int32),
                            np.array([1, -2, 1, 1], np.int32), ones(1))),
        ("pin", H(4, 1, np.array([0, 2], np.int64), np.array([0, -1], np.int32), ones(4), ones(1))),
        ("gain bound", H(4, 1, np.array([0, 3], np.int64), np.array([0, 1, 2], np.int32), ones(4),
                         np.array([10 ** 9], np.int32))),
        ("total weight", H(3, 1, np.array([0, 2], np.int64), np.array([0, 1], np.int32),
                           np.array([1_500_000_000, 1_500_000_000, 1], np.int32), ones(1))),
    ]
    ok = gen.random_small(3, n=300, m=360, k=4)
    with lp.Session(0) as s:
        for name, hg in cases:
            with pytest.raises(lp.LpgpuError) as e:
                s.upload(hg)
            assert e.value.status == lp.ERR_INVALID_ARG, name
            with pytest.raises(lp.LpgpuError) as e:
                s.set_partition(2, np.zeros(hg.n, np.int32))
            assert e.value.status == lp.ERR_STATE, name
        s.upload(ok.hg)
        bad = ok.part.copy()
        bad[123] = 4
        with pytest.raises(lp.LpgpuError) as e:
            s.set_partition(4, bad)
        assert e.value.status == lp.ERR_INVALID_ARG
        s.set_partition(4, ok.part, lmax=ok.lmax, perfect=ok.perfect)
        check_state(orc, s, ok.hg, 4, ok.part)
    # batch: a local block id above its instance's k
    insts = [gen.random_small(10 + i, n=100, m=120, k=3) for i in range(3)]
    with lp.Session(0) as s:
        s.upload_batch([x.hg for x in insts])
        parts = [x.part.copy() for x in insts]
        parts[1][7] = 3
        with pytest.raises(lp.LpgpuError) as e:
            s.set_partition_batch([3, 3, 3], parts)
        assert e.value.status == lp.ERR_INVALID_ARG
        s.set_partition_batch([3, 3, 3], [x.part for x in insts])
        assert s.instance_km1().shape == (3,)


@pytest.mark.parametrize("form", ["union", "instances"])
def test_batched_input_checks(lp, form):
    """Batched uploads are checked per instance on the device: a pin outside
    its instance's vertex range, a negative net weight and decreasing offsets
    inside one instance are each rejected with INVALID_ARG, and the session then
    refines a valid batch exactly as one session per instance does."""
    from lpgpu import gen
    insts = [gen.random_small(40 + i, n=150 + 20 * i, m=170, k=3) for i in range(3)]

    def broken(kind):
        hgs = [x.hg for x in insts]
        h = hgs[1]
        if kind == "pin":
            pins = h.pins.copy()
            pins[5] = h.n  # local id one past the instance's last vertex
            hgs[1] = gen.Hypergraph(h.n, h.m, h.net_off, pins, h.w_v, h.w_e)
        elif kind == "net weight":
            w_e = h.w_e.copy()
            w_e[3] = -1
            hgs[1] = gen.Hypergraph(h.n, h.m, h.net_off, h.pins, h.w_v, w_e)
        else:  # decreasing offsets inside the instance
            off = h.net_off.copy()
            off[4] = off[6]
            off[5] = off[3]
            hgs[1] = gen.Hypergraph(h.n, h.m, off, h.pins, h.w_v, h.w_e)
        return hgs

    def upload(s, hgs):
        return s.upload_batch(hgs) if form == "union" else s.upload_instances(hgs)

    cfg = lp.default_config(rounds=3)
    with lp.Session(0) as s:
        for kind in ("pin", "net weight", "offsets"):
            with pytest.raises(lp.LpgpuError) as e:
                upload(s, broken(kind))
            assert e.value.status == lp.ERR_INVALID_ARG, kind
        upload(s, [x.hg for x in insts])
        s.set_partition_batch([x.k for x in insts], [x.part for x in insts])
        s.refine(cfg)
        got = s.instance_km1()
    want = []
    for x in insts:
        with lp.Session(0) as t:
            t.upload(x.hg)
            t.set_partition(x.k, x.part)
            want.append(t.refine(cfg).km1_after)
    assert list(got) == want


def test_one_shot_entry_point(lp, orc):
    from lpgpu import gen
    inst = gen.plain_small(seed=2)
    cfg = lp.default_config(rounds=5, subrounds=8)
    p, r = lp.refine_km1(inst.hg, inst.k, inst.part, eps=0.03, cfg=cfg)
    ep, est = orc.lp_sync(inst.hg, inst.k, inst.lmax, inst.part, perfect=inst.perfect, rounds=5,
                          subrounds=8, revert=1, rollback=1, zero_gain=1)
    assert np.array_equal(p, ep)
    assert r.km1_after == r.km1_before + r.delta and r.km1_after < r.km1_before


@pytest.mark.parametrize("seed", range(3))
@pytest.mark.parametrize("k,weighted", [(2, True), (7, False), (33, True), (128, True)])
def test_maintained_gain_cache_equals_recomputation(lp, orc, seed, k, weighted):
    """The device gain cache kept by apply_moves (gainCacheUpdate rules, many
    concurrent moves per batch) equals initializeGainCache on the final state."""
    from lpgpu import gen
    inst = gen.random_small(seed, n=400, m=480, k=k, max_size=10, weighted=weighted, hubs=2)
    hg = inst.hg
    rng = np.random.default_rng([seed, k])
    s = session(lp, hg, k, inst.part, lmax=inst.lmax, perfect=inst.perfect)
    s.init_gain_cache()
    part = inst.part.copy()
    for batch in range(4):
        vs = rng.choice(hg.n, size=int(rng.integers(1, 120)), replace=False).astype(np.int32)
        to = ((part[vs] + rng.integers(1, k, size=len(vs))) % k).astype(np.int32) if k > 1 else part[vs]
        s.apply_moves(vs, part[vs], to)
        part[vs] = to
        ben, pen = s.gain_cache()
        eben, epen = orc.gain_cache(hg, k, part)
        assert np.array_equal(ben, eben), f"benefit, batch {batch}"
        assert np.array_equal(pen, epen), f"penalty, batch {batch}"
    check_state(orc, s, hg, k, part)
    s.refine(lp.default_config(rounds=2, subrounds=2))  # drops the maintained cache
    ben, pen = s.gain_cache()
    eben, epen = orc.gain_cache(hg, k, s.partition())
    assert np.array_equal(ben, eben) and np.array_equal(pen, epen)
    s.close()


def _contract_pairs(hg, rng):
    """A coarse hypergraph from a random matching of vertex pairs: coarse nets are
    the fine nets with pins mapped and duplicates removed; nets left with one pin
    are dropped, parallel nets kept (weights as in the fine nets)."""
    from lpgpu import gen
    perm = rng.permutation(hg.n)
    cmap = np.empty(hg.n, np.int32)
    cmap[perm] = np.arange(hg.n) // 2
    nc = (hg.n + 1) // 2
    off, pins, we = [0], [], []
    for e in range(hg.m):
        p = np.unique(cmap[hg.pins[hg.net_off[e]:hg.net_off[e + 1]]])
        if len(p) < 2:
            continue
        pins.extend(p.tolist())
        off.append(len(pins))
        we.append(hg.w_e[e])
    w_v = np.zeros(nc, np.int32)
    np.add.at(w_v, cmap, hg.w_v)
    coarse = gen.Hypergraph(nc, len(we), np.array(off, np.int64), np.array(pins, np.int32), w_v,
                            np.array(we, np.int32)).with_incidence()
    return coarse, cmap


@pytest.mark.parametrize("seed", range(3))
@pytest.mark.parametrize("k", [2, 8, 64])
def test_projection_between_levels(lp, orc, seed, k):
    """Coarse refine, then device-to-device projection to the fine level: the fine
    partition is coarse_part[map], with the coarse bounds and a fresh state."""
    from lpgpu import gen
    rng = np.random.default_rng([seed, k, 5])
    inst = gen.random_small(seed, n=600, m=700, k=k, max_size=8)
    coarse, cmap = _contract_pairs(inst.hg, rng)
    cpart = gen.random_balanced_partition(coarse.n, k, rng)
    perfect, lmax = gen.part_weights(int(coarse.w_v.sum()), k, 0.1)
    with lp.Session(0) as c, lp.Session(0) as f:
        c.upload(coarse)
        c.set_partition(k, cpart, lmax=lmax, perfect=perfect)
        c.refine(lp.default_config(rounds=3, subrounds=4))
        cp = c.partition()
        f.upload(inst.hg)
        f.project_partition(c, cmap)
        fp = f.partition()
        assert np.array_equal(fp, cp[cmap])
        check_state(orc, f, inst.hg, k, fp)
        # the fine level refines from there as usual (against the oracle)
        r = f.refine(lp.default_config(rounds=3, subrounds=4))
        ref, _ = orc.lp_sync(inst.hg, k, lmax, fp, perfect=perfect, rounds=3, subrounds=4, revert=1,
                             rollback=1, zero_gain=1)
        assert np.array_equal(f.partition(), ref)
        assert r.km1_after == r.km1_before + r.delta
        bad = cmap.copy()
        bad[5] = coarse.n
        with pytest.raises(lp.LpgpuError) as e:
            f.project_partition(c, bad)
        assert e.value.status == lp.ERR_INVALID_ARG


@pytest.mark.parametrize("seed,n,m,k", [(116, 60, 120, 2), (149, 60, 120, 2), (11, 100, 300, 3), (128, 100, 300, 3)])
def test_rollback_path(lp, orc, seed, n, m, k):
    """Instances where a whole sub-round is rolled back (one sub-round, no
    revert): the oracle's result differs with and without rollback, and the
    device follows the oracle."""
    from lpgpu import gen
    inst = gen.random_small(seed, n=n, m=m, k=k, max_size=3)
    kw = dict(perfect=inst.perfect, rounds=4, subrounds=1, revert=0, zero_gain=1)
    with_rb, _ = orc.lp_sync(inst.hg, k, inst.lmax, inst.part, rollback=1, **kw)
    without, _ = orc.lp_sync(inst.hg, k, inst.lmax, inst.part, rollback=0, **kw)
    assert not np.array_equal(with_rb, without)  # the rollback path is taken
    out = run_both(lp, orc, inst, 4, dict(subrounds=1, revert=0, rollback=1, rebalancing=1))
    assert_same_run(*out, orc, inst)
    out[0].close()

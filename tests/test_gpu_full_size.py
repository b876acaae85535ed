"""Bit-exact parity on the full-size workloads that the benchmark measures.

The 1,048,576-vertex plain_large workload (k = 32, Zipf nets up to 4,096
pins, weighted) and the 4,194,304 x 4,194,304 row-net workload (k = 128,
33.7M pins, hubs of degree ~4,100, 16-bit pin counts under sustained
atomics) go through the C ABI exactly as the benchmark runs them, and are
compared with the CPU oracle (threaded: its sweep is a pure function of the
sub-round snapshot, so threads change nothing):

* after set_partition: pin counts Φ, connectivity sets Λ, block weights,
  km1, cut (initializePartition, partitioned_hypergraph.h:1067-1110;
  metrics::km1, metrics.cpp:49-65) and every vertex's Km1Policy best move
  (gain_policy.h:108-167) with its isBorderNode flag (h:605-620);
* after the default refinement (10 rounds, 7 sub-rounds, reverts, rollback,
  rebalancing moves): the partition, every round's statistics and the final
  state, against the oracle's synchronous LP.

A last case puts one vertex in 100,001 nets: isBorderNode is false above
100,000 incident nets (partitioned_hypergraph.h:67, 605-620), so it is never
swept and never moves, while a vertex of exactly 100,000 nets is treated as
any other.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


@pytest.fixture(scope="module", params=["plain_large", "rownet"])
def workload(request):
    from lpgpu import gen
    return getattr(gen, request.param)(seed=0)


def _check_state(orc, s, inst, part):
    hg, k = inst.hg, inst.k
    phi, conn, bw = orc.init_partition(hg, k, part)
    assert np.array_equal(s.block_weights(), bw)
    assert np.array_equal(s.connectivity(), conn)
    assert np.array_equal(s.pin_counts(), phi)
    del phi
    km1, cut = orc.metrics(hg, k, conn)
    dk, dc, _ = s.metrics()
    assert (dk, dc) == (km1, cut)


def test_full_size_state_and_best_moves(lp, orc, workload):
    inst = workload
    with lp.Session(0) as s:
        s.upload(inst.hg)
        s.set_partition(inst.k, inst.part, lmax=inst.lmax, perfect=inst.perfect)
        _check_state(orc, s, inst, inst.part)
        to, gain, border = s.best_moves()
    eto, egain, eborder = orc.best_moves(inst.hg, inst.k, inst.part, inst.lmax)
    assert np.array_equal(border, eborder)
    assert np.array_equal(to, eto)
    assert np.array_equal(gain, egain)
    assert (gain < 0).sum() > 0


def test_full_size_refine_bit_exact(lp, orc, workload):
    inst = workload
    cfg = lp.default_config(rounds=inst.rounds)  # 7 sub-rounds, reverts, rollback, rebalancing
    with lp.Session(0) as s:
        s.upload(inst.hg)
        s.set_partition(inst.k, inst.part, lmax=inst.lmax, perfect=inst.perfect)
        r = s.refine(cfg)
        dpart = s.partition()
        dstats = s.round_stats()
        epart, estats = orc.lp_sync(inst.hg, inst.k, inst.lmax, inst.part, perfect=inst.perfect,
                                    rounds=inst.rounds, activation_threshold=cfg.activation_threshold,
                                    subrounds=cfg.subrounds, revert=1, rollback=1, zero_gain=1,
                                    threads=THREADS)
        keys = ["active", "pins", "candidates", "moved", "reverted", "delta"]
        assert [[st[x] for x in keys] for st in dstats] == [[st[x] for x in keys] for st in estats]
        assert np.array_equal(dpart, epart)
        _check_state(orc, s, inst, epart)
        assert r.km1_after == r.km1_before + r.delta
        assert r.km1_after == estats[-1]["km1_after"]
        assert r.delta < 0
        bw = s.block_weights()
    assert (bw <= inst.lmax).all()
    assert (bw >= 1).all()


def _hub_instance(k):
    """Vertex 0 in 100,001 two-pin nets, vertex H = 100,002 in exactly 100,000,
    plus 60,000 random nets of 2..6 pins over the other vertices."""
    from lpgpu import gen
    rng = np.random.default_rng([k, 100001])
    a_deg, b_deg = 100001, 100000
    H = a_deg + 1
    n = H + b_deg + 1 + 5000
    nets = [np.array([0, i]) for i in range(1, a_deg + 1)]
    nets += [np.array([H, H + j]) for j in range(1, b_deg + 1)]
    others = np.setdiff1d(np.arange(n), [0, H])  # the hubs' degrees stay exact
    for _ in range(60000):
        nets.append(rng.choice(others, size=int(rng.integers(2, 7)), replace=False))
    off = np.zeros(len(nets) + 1, np.int64)
    np.cumsum([len(e) for e in nets], out=off[1:])
    pins = np.concatenate(nets).astype(np.int32)
    hg = gen.Hypergraph(n, len(nets), off, pins, np.ones(n, np.int32), np.ones(len(nets), np.int32))
    hg.with_incidence()
    part = gen.random_balanced_partition(n, k, rng)
    return gen.Instance(f"hubs[k={k}]", hg, k, 0.03, part, 4), H


@pytest.mark.parametrize("k", [2, 5])
def test_vertex_above_high_degree_threshold_is_never_border(lp, orc, k):
    inst, H = _hub_instance(k)
    hg = inst.hg
    assert hg.vtx_off[1] - hg.vtx_off[0] == 100001
    assert hg.vtx_off[H + 1] - hg.vtx_off[H] == 100000
    with lp.Session(0) as s:
        s.upload(hg)
        s.set_partition(k, inst.part, lmax=inst.lmax, perfect=inst.perfect)
        to, gain, border = s.best_moves()
        eto, egain, eborder = orc.best_moves(hg, k, inst.part, inst.lmax)
        assert not border[0] and not eborder[0]
        assert border[H] and eborder[H]
        assert to[0] == inst.part[0] and gain[0] == 0
        assert np.array_equal(border, eborder) and np.array_equal(to, eto) and np.array_equal(gain, egain)
        for mode in (dict(subrounds=7, revert=1, rollback=1, rebalancing=1),
                     dict(subrounds=1, revert=0, rollback=0, rebalancing=0)):
            s.set_partition(k, inst.part, lmax=inst.lmax, perfect=inst.perfect)
            r = s.refine(lp.default_config(rounds=inst.rounds, **mode))
            dpart, dstats = s.partition(), s.round_stats()
            epart, estats = orc.lp_sync(hg, k, inst.lmax, inst.part, perfect=inst.perfect, rounds=inst.rounds,
                                        subrounds=mode["subrounds"], revert=mode["revert"],
                                        rollback=mode["rollback"], zero_gain=mode["rebalancing"],
                                        threads=THREADS)
            keys = ["active", "pins", "candidates", "moved", "reverted", "delta"]
            assert [[st[x] for x in keys] for st in dstats] == [[st[x] for x in keys] for st in estats]
            assert np.array_equal(dpart, epart)
            assert dpart[0] == inst.part[0]  # the hub above the threshold never moves
            assert r.km1_after == r.km1_before + r.delta
            _check_state(orc, s, inst, epart)

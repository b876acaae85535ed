"""Pins the CPU oracle to the reference's own known-answer tests.

Each test restates an assertion of Mt-KaHyPar's gtest suite (file:line cited)
on the oracle. The oracle is then trusted as the checker of the device path.
"""
import numpy as np
import pytest

from conftest import load_golden, seven_vertex_fixture

INF = np.iinfo(np.int32).max


def _apply(orc, hg, k, part, moves):
    """Applies moves one after another with the oracle's changeNodePart restatement."""
    p = np.array(part, np.int32)
    for v, f, t in moves:
        assert p[v] == f
        p[v] = t
    return p


def _delta(orc, hg, k, before, after):
    _, c0, _ = orc.init_partition(hg, k, before)
    _, c1, _ = orc.init_partition(hg, k, after)
    return orc.metrics(hg, k, c1)[0] - orc.metrics(hg, k, c0)[0]


# gain_policy_test.cc:63-276 (Km1Policy, disable_randomization = true, unbounded max weights)
KM1_CASES = [
    (2, [1, 0, 0, 0, 0, 1, 1], 0, (1, 0, -2)),
    (2, [0, 0, 0, 1, 0, 1, 1], 3, (1, 0, -1)),
    (2, [0, 0, 0, 0, 0, 1, 1], 4, (0, 0, 0)),
    (4, [0, 1, 2, 3, 3, 1, 2], 0, (0, 1, -1)),
    (4, [0, 3, 1, 2, 2, 0, 3], 6, (3, 0, -1)),
    (4, [0, 3, 1, 2, 2, 0, 3], 3, (2, 2, 0)),
]


@pytest.mark.parametrize("k,part,v,expected", KM1_CASES)
def test_km1_policy_known_answers(orc, k, part, v, expected):
    hg = seven_vertex_fixture()
    lmax = np.full(k, INF, np.int64)
    to, gain, border = orc.best_moves(hg, k, np.array(part, np.int32), lmax)
    frm, exp_to, exp_gain = expected
    assert part[v] == frm
    assert (to[v], gain[v]) == (exp_to, exp_gain)


# gain_policy_test.cc:73-87,98-112,171-185,196-210: delta() after changeNodePart
@pytest.mark.parametrize("k,part,move,exp_delta", [
    (2, [1, 0, 0, 0, 0, 1, 1], (0, 1, 0), -2),
    (2, [0, 0, 0, 1, 0, 1, 1], (3, 1, 0), -1),
    (4, [0, 1, 2, 3, 3, 1, 2], (0, 0, 1), -1),
    (4, [0, 3, 1, 2, 2, 0, 3], (6, 3, 0), -1),
])
def test_km1_delta_known_answers(orc, k, part, move, exp_delta):
    hg = seven_vertex_fixture()
    after = _apply(orc, hg, k, part, [move])
    assert _delta(orc, hg, k, part, after) == exp_delta


BASE = [0, 0, 0, 1, 1, 2, 2]  # partitioned_hypergraph_test.cc:65-73


def test_initial_state_known_answers(orc):
    hg = seven_vertex_fixture()
    phi, conn, bw = orc.init_partition(hg, 3, np.array(BASE, np.int32))
    assert bw.tolist() == [3, 2, 2]                                        # :168-171
    assert phi.tolist() == [[2, 0, 0], [2, 2, 0], [0, 2, 1], [1, 0, 2]]    # :191-196
    assert [int(c[0]) for c in conn] == [0b001, 0b011, 0b110, 0b101]       # :694-713
    to, gain, border = orc.best_moves(hg, 3, np.array(BASE, np.int32), np.full(3, INF, np.int64))
    assert border.all()                                                    # :381-395


# partitioned_hypergraph_test.cc:198-296 (pin counts after concurrent moves)
PIN_COUNT_CASES = [
    ([(0, 0, 1), (1, 0, 2)], [[1, 1, 0], [0, 3, 1], [0, 2, 1], [1, 0, 2]]),
    ([(3, 1, 2), (6, 2, 0)], [[2, 0, 0], [2, 1, 1], [1, 1, 1], [2, 0, 1]]),
    ([(3, 1, 2), (4, 1, 2)], [[2, 0, 0], [2, 0, 2], [0, 0, 3], [1, 0, 2]]),
    ([(2, 0, 2), (5, 2, 0)], [[1, 0, 1], [2, 2, 0], [0, 2, 1], [1, 0, 2]]),
    ([(0, 0, 1), (6, 2, 1)], [[1, 1, 0], [1, 3, 0], [0, 3, 0], [1, 1, 1]]),
    ([(0, 0, 1), (2, 0, 2), (4, 1, 0), (6, 2, 1), (1, 0, 2), (3, 1, 0), (5, 2, 1)],
     [[0, 1, 1], [2, 1, 1], [2, 1, 0], [0, 2, 1]]),
]


@pytest.mark.parametrize("moves,expected", PIN_COUNT_CASES)
def test_pin_counts_after_moves(orc, moves, expected):
    hg = seven_vertex_fixture()
    p = _apply(orc, hg, 3, BASE, moves)
    phi, _, _ = orc.init_partition(hg, 3, p)
    assert phi.tolist() == expected


# partitioned_hypergraph_test.cc:299-378 (connectivity sets after moves)
CONN_CASES = [
    ([(6, 2, 0), (0, 0, 1)], [{0, 1}, {0, 1}, {0, 1}, {0, 2}]),
    ([(5, 2, 0), (2, 0, 2)], [{0, 2}, {0, 1}, {1, 2}, {0, 2}]),
    ([(0, 0, 1), (2, 0, 1)], [{1}, {0, 1}, {1, 2}, {1, 2}]),
    ([(4, 1, 0), (3, 1, 0)], [{0}, {0}, {0, 2}, {0, 2}]),
    ([(1, 0, 2), (3, 1, 2)], [{0}, {0, 1, 2}, {1, 2}, {0, 2}]),
    ([(0, 0, 1), (3, 1, 0), (6, 2, 0), (1, 0, 2), (2, 0, 1), (4, 1, 0), (5, 2, 1)],
     [{1}, {0, 1, 2}, {0}, {0, 1}]),
]


@pytest.mark.parametrize("moves,expected", CONN_CASES)
def test_connectivity_after_moves(orc, moves, expected):
    hg = seven_vertex_fixture()
    p = _apply(orc, hg, 3, BASE, moves)
    _, conn, _ = orc.init_partition(hg, 3, p)
    got = [{b for b in range(3) if (int(c[0]) >> b) & 1} for c in conn]
    assert got == expected


# partitioned_hypergraph_test.cc:397-464 (border nodes after moves)
@pytest.mark.parametrize("moves,border", [
    ([(4, 1, 0), (3, 1, 0)], [0, 0, 1, 1, 1, 1, 1]),
    ([(3, 1, 0), (1, 0, 1), (4, 1, 0), (2, 0, 1)], [1, 1, 1, 1, 1, 1, 1]),
    ([(6, 2, 0), (3, 1, 0), (5, 2, 0), (4, 1, 0)], [0, 0, 0, 0, 0, 0, 0]),
])
def test_border_nodes_after_moves(orc, moves, border):
    hg = seven_vertex_fixture()
    p = _apply(orc, hg, 3, BASE, moves)
    _, _, b = orc.best_moves(hg, 3, p, np.full(3, INF, np.int64))
    assert b.astype(int).tolist() == border


def test_gain_cache_twocenters_known_answers(orc):
    """gain_updates_test.cc:36-70 on tests/instances/twocenters.hgr."""
    hg, _ = load_golden("twocenters")
    part = np.zeros(hg.n, np.int32)
    part[[2, 3]] = 1
    part[12:20] = 1
    _, _, bw = orc.init_partition(hg, 2, part)
    assert bw.tolist() == [10, 10]
    ben, pen = orc.gain_cache(hg, 2, part)

    def km1gain(u, t):
        return ben[u] - pen[u, t]

    assert km1gain(0, 1) == -1 and ben[0] == 1 and pen[0, 1] == 2
    assert km1gain(2, 0) == -1
    assert km1gain(4, 1) == -1 and km1gain(6, 1) == -2
    assert km1gain(12, 0) == -1 and km1gain(14, 0) == -2
    # move 8 from 0 to 1, then km1Gain(8, 1, 0) == 2 and km1Gain(6, 0, 1) == 0
    part2 = part.copy()
    part2[8] = 1
    ben2, pen2 = orc.gain_cache(hg, 2, part2)
    assert ben2[8] - pen2[8, 0] == 2
    assert ben2[6] - pen2[6, 1] == 0


@pytest.mark.parametrize("seed", range(6))
def test_km1_gain_brute_force(orc, seed):
    """verifyAllKm1GainValues (partitioned_hypergraph_test.cc:120-135):
    km1Gain(u, from, to) == km1_before - km1_after for every vertex and block."""
    from lpgpu import gen
    inst = gen.random_small(seed, n=40, m=50, k=3 + seed % 3)
    hg, k, part = inst.hg, inst.k, inst.part
    ben, pen = orc.gain_cache(hg, k, part)
    _, conn, _ = orc.init_partition(hg, k, part)
    km1_0 = orc.metrics(hg, k, conn)[0]
    for u in range(hg.n):
        for t in range(k):
            if t == part[u]:
                continue
            p = part.copy()
            p[u] = t
            _, c1, _ = orc.init_partition(hg, k, p)
            assert ben[u] - pen[u, t] == km1_0 - orc.metrics(hg, k, c1)[0]


@pytest.mark.parametrize("seed", range(4))
def test_best_move_matches_brute_force(orc, seed):
    """Km1Policy's best move equals the minimum over blocks of the brute-force
    objective delta (ties to the lowest block, strict improvement, feasibility)."""
    from lpgpu import gen
    inst = gen.random_small(seed + 10, n=60, m=70, k=4)
    hg, k, part = inst.hg, inst.k, inst.part
    _, conn, bw = orc.init_partition(hg, k, part)
    lmax = np.full(k, int(bw.max()) + 2, np.int64)
    to, gain, border = orc.best_moves(hg, k, part, lmax)
    ben, pen = orc.gain_cache(hg, k, part)
    for u in range(hg.n):
        if not border[u]:
            assert to[u] == part[u] and gain[u] == 0
            continue
        best_t, best_g = part[u], 0
        for t in range(k):
            if t == part[u] or bw[t] + hg.w_v[u] > lmax[t]:
                continue
            g = -(ben[u] - pen[u, t])
            if g < best_g:
                best_t, best_g = t, g
        assert (to[u], gain[u]) == (best_t, best_g)


@pytest.mark.parametrize("k", [2, 4, 8])
@pytest.mark.parametrize("mode", ["async", "sync"])
def test_lp_refiner_properties_ibm01(orc, k, mode):
    """label_propagation_refiner_test.cc:133-153 on contracted_unweighted_ibm01
    (eps = 0.25): imbalance within eps + 0.05, tracked metric equals the
    recomputed km1, quality never worse. The reference's BFS initial partition
    is replaced by a seeded random balanced one."""
    from lpgpu import gen
    hg, _ = load_golden("contracted_unweighted_ibm01")
    part = gen.random_balanced_partition(hg.n, k, np.random.default_rng(k))
    perfect, lmax = gen.part_weights(int(hg.w_v.sum()), k, 0.25)
    _, conn, _ = orc.init_partition(hg, k, part)
    km1_0 = orc.metrics(hg, k, conn)[0]
    if mode == "async":
        p, stats = orc.lp_async(hg, k, lmax, perfect, part, rounds=5, threads=4, seed=1)
    else:
        p, stats = orc.lp_sync(hg, k, lmax, part, perfect=perfect, rounds=5, subrounds=4,
                               revert=1, rollback=1, zero_gain=1)
    _, conn1, bw1 = orc.init_partition(hg, k, p)
    km1_1 = orc.metrics(hg, k, conn1)[0]
    assert km1_1 == km1_0 + sum(s["delta"] for s in stats)
    assert km1_1 <= km1_0
    assert (bw1 / perfect).max() - 1.0 <= 0.25 + 0.05
    assert (bw1 <= lmax).all()


def _rebalance_test_partition(hg, k):
    """rebalance_test.cc:56-73: contracted_ibm01, k = 8, the first n / 4
    vertices in block 0, the next n / 4 in block 1, ...; blocks 4..7 empty."""
    per = hg.n // (k - 4)
    assert hg.n % (k - 4) == 0
    return (np.arange(hg.n) // per).astype(np.int32)


def test_repair_empty_blocks_finds_moves_ibm01(orc):
    """rebalance_test.cc:56-103 (FindsMoves): four moves, one per empty block;
    each gain equals km1Gain recomputed from the state (positive = better); a
    zero gain only for a vertex whose nets all hold it as their one pin in its
    block; sources are the filled blocks, targets the empty ones; after the
    moves are applied no block is empty and repairEmptyBlocks finds nothing."""
    from lpgpu import gen
    hg, _ = load_golden("contracted_ibm01")
    k = 8
    perfect, lmax = gen.part_weights(int(hg.w_v.sum()), k, 0.03)
    part = _rebalance_test_partition(hg, k)
    phi, _, bw = orc.init_partition(hg, k, part)
    benefit, penalty = orc.gain_cache(hg, k, part)
    moves = orc.repair_empty_blocks(hg, k, lmax, part)
    assert len(moves) == 4
    for v, f, t, g in moves:
        assert g == benefit[v] - penalty[v, t]  # km1Gain = moveFromBenefit - moveToPenalty
        if g == 0:
            assert all(phi[e, f] == 1 for e in hg.inets[hg.vtx_off[v]:hg.vtx_off[v + 1]])
        assert f == part[v] and bw[t] == 0
        assert t >= k - 4 and f < k - 4
    assert len({v for v, _, _, _ in moves}) == 4
    after = _apply(orc, hg, k, part, [(v, f, t) for v, f, t, _ in moves])
    assert orc.repair_empty_blocks(hg, k, lmax, after) == []


def test_rebalance_repairs_empty_blocks_first(orc):
    """rebalancer.cpp:34-62: an imbalanced partition with empty blocks gets the
    repair moves first (their record leads the statistics), then the rebalancing
    rounds; the result is balanced with no empty block and exact km1 bookkeeping."""
    from lpgpu import gen
    hg, _ = load_golden("contracted_ibm01")
    k = 8
    perfect, lmax = gen.part_weights(int(hg.w_v.sum()), k, 0.03)
    part = _rebalance_test_partition(hg, k)
    moves = orc.repair_empty_blocks(hg, k, lmax, part)
    p, stats = orc.rebalance(hg, k, lmax, part, 32)
    assert stats[0]["candidates"] == 4 and stats[0]["moved"] == 4 and stats[0]["active"] == hg.n
    assert stats[0]["delta"] == _delta(orc, hg, k, part, _apply(orc, hg, k, part, [m[:3] for m in moves]))
    _, conn, bw = orc.init_partition(hg, k, p)
    assert (bw <= lmax).all() and (bw > 0).all()
    _, conn0, _ = orc.init_partition(hg, k, part)
    assert orc.metrics(hg, k, conn)[0] == orc.metrics(hg, k, conn0)[0] + sum(s["delta"] for s in stats)

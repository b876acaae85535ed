"""Deterministic rebalancer on the device vs the oracle, bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _imbalanced(seed, k, weighted, hubs=0, frac=0.3):
    from lpgpu import gen
    inst = gen.random_small(seed, n=1500, m=1800, k=k, max_size=8, weighted=weighted, hubs=hubs)
    rng = np.random.default_rng([seed, k, 9])
    part = inst.part.copy()
    sel = rng.random(inst.hg.n) < frac
    part[sel] = rng.integers(0, max(1, k // 3), size=int(sel.sum()))
    return inst, part


@pytest.mark.parametrize("seed", range(3))
@pytest.mark.parametrize("k", [2, 5, 32, 100])
@pytest.mark.parametrize("weighted", [False, True])
def test_rebalance_matches_oracle(lp, orc, seed, k, weighted):
    inst, part = _imbalanced(seed, k, weighted, hubs=2 if seed == 1 else 0)
    hg = inst.hg
    with lp.Session(0) as s:
        s.upload(hg)
        s.set_partition(k, part, lmax=inst.lmax, perfect=inst.perfect)
        km0 = s.metrics()[0]
        r = s.rebalance(8)
        dpart = s.partition()
        dstats = s.round_stats()
        bw = s.block_weights()
        km1 = s.metrics()[0]
    epart, estats = orc.rebalance(hg, k, inst.lmax, part, 8)
    assert np.array_equal(dpart, epart)
    keys = ["active", "pins", "candidates", "moved", "delta"]
    assert [[st[x] for x in keys] for st in dstats] == [[st[x] for x in keys] for st in estats]
    assert km1 == km0 + r.delta == r.km1_after
    _, _, ebw = orc.init_partition(hg, k, epart)
    assert np.array_equal(bw, ebw)


def test_balanced_input_is_left_alone(lp):
    from lpgpu import gen
    inst = gen.random_small(4, n=800, m=900, k=4, weighted=False)  # counts = weights: balanced
    with lp.Session(0) as s:
        s.upload(inst.hg)
        s.set_partition(4, inst.part, lmax=inst.lmax, perfect=inst.perfect)
        r = s.rebalance(8)
        assert r.rounds == 0 and r.moves == 0
        assert np.array_equal(s.partition(), inst.part)


def test_rebalance_then_refine(lp, orc):
    inst, part = _imbalanced(7, 8, True)
    with lp.Session(0) as s:
        s.upload(inst.hg)
        s.set_partition(8, part, lmax=inst.lmax, perfect=inst.perfect)
        s.rebalance(16)
        p1 = s.partition()
        assert (s.block_weights() <= inst.lmax).all()
        s.refine(lp.default_config(rounds=3, subrounds=4))
        ref, _ = orc.lp_sync(inst.hg, 8, inst.lmax, p1, perfect=inst.perfect, rounds=3, subrounds=4,
                             revert=1, rollback=1, zero_gain=1)
        assert np.array_equal(s.partition(), ref)


def _ibm01_empty_blocks():
    """rebalance_test.cc:56-73: contracted_ibm01, k = 8, blocks 0..3 hold
    consecutive quarters of the vertices, blocks 4..7 are empty."""
    from conftest import load_golden
    from lpgpu import gen
    hg, _ = load_golden("contracted_ibm01")
    k = 8
    perfect, lmax = gen.part_weights(int(hg.w_v.sum()), k, 0.03)
    part = (np.arange(hg.n) // (hg.n // (k - 4))).astype(np.int32)
    return hg, k, perfect, lmax, part


def test_repair_empty_blocks_matches_oracle_and_reference_assertions(lp, orc):
    """rebalance_test.cc:56-103 on the device: four moves, one per empty block,
    equal to the oracle's; each gain is km1Gain from the device gain cache; after
    the moves no block is empty and a second repair finds nothing."""
    hg, k, perfect, lmax, part = _ibm01_empty_blocks()
    with lp.Session(0) as s:
        s.upload(hg)
        s.set_partition(k, part, lmax=lmax, perfect=perfect)
        moves = s.repair_empty_blocks()
        assert moves == orc.repair_empty_blocks(hg, k, lmax, part)
        assert len(moves) == 4
        benefit, penalty = s.gain_cache()
        bw = s.block_weights()
        for v, f, t, g in moves:
            assert g == benefit[v] - penalty[v, t]
            assert f == part[v] and bw[t] == 0 and t >= k - 4 and f < k - 4
        s.apply_moves([m[0] for m in moves], [m[1] for m in moves], [m[2] for m in moves])
        assert (s.block_weights() > 0).all()
        assert s.repair_empty_blocks() == []


@pytest.mark.parametrize("k", [8, 37])
def test_rebalance_with_empty_blocks_matches_oracle(lp, orc, k):
    """An imbalanced partition with empty blocks: repair first, then the
    rebalancing rounds, bit-exact against the oracle (partition, every
    statistics record including the repair's, block weights)."""
    from lpgpu import gen
    if k == 8:
        hg, k, perfect, lmax, part = _ibm01_empty_blocks()
    else:
        inst = gen.random_small(11, n=3000, m=3600, k=k, max_size=8, weighted=True)
        hg, perfect, lmax = inst.hg, inst.perfect, inst.lmax
        part = (inst.part % (k // 2)).astype(np.int32)  # blocks k/2.. empty, the others overloaded
    with lp.Session(0) as s:
        s.upload(hg)
        s.set_partition(k, part, lmax=lmax, perfect=perfect)
        km0 = s.metrics()[0]
        r = s.rebalance(16)
        dpart, dstats, bw = s.partition(), s.round_stats(), s.block_weights()
        km1 = s.metrics()[0]
    epart, estats = orc.rebalance(hg, k, lmax, part, 16)
    keys = ["active", "pins", "candidates", "moved", "delta"]
    assert [[st[x] for x in keys] for st in dstats] == [[st[x] for x in keys] for st in estats]
    assert np.array_equal(dpart, epart)
    assert estats[0]["active"] == hg.n and estats[0]["moved"] > 0
    assert km1 == km0 + r.delta == r.km1_after
    _, _, ebw = orc.init_partition(hg, k, epart)
    assert np.array_equal(bw, ebw) and (bw > 0).all()

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

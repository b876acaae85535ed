"""Persistent rounds (one launch per LP round, instances as work items of a
device queue) against the multi-launch sub-round pipeline and the oracle:
partitions, per-round statistics and per-instance km1 must be identical for
every configuration and every tuning variant."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KEYS = ["active", "pins", "candidates", "moved", "reverted", "delta", "moved_pins"]

MODES = [
    dict(subrounds=7, revert=1, rollback=1, rebalancing=1),
    dict(subrounds=1, revert=0, rollback=0, rebalancing=1),
    dict(subrounds=4, revert=1, rollback=0, rebalancing=0),
    dict(subrounds=16, revert=1, rollback=1, rebalancing=1),
    dict(subrounds=64, revert=0, rollback=1, rebalancing=1),
]


def _instances(seed, count, ks=(2, 3, 4, 7, 16, 33, 64), hubs=False):
    from lpgpu import gen
    out = []
    rng = np.random.default_rng([seed, 77])
    for i in range(count):
        n = int(rng.integers(40, 1500))
        m = int(n * rng.uniform(0.8, 1.4))
        k = int(rng.choice(ks))
        out.append(gen.random_small(3000 * seed + i, n=n, m=m, k=k, max_size=12, weighted=bool(i % 2),
                                    hubs=(2 if hubs and i % 3 == 0 else 0)))
    return out


def _run(lp, insts, cfg, tuning=None):
    with lp.Session(0) as s:
        s.upload_batch([x.hg for x in insts])
        s.set_partition_batch([x.k for x in insts], [x.part for x in insts], eps=0.03)
        if tuning:
            s.set_tuning(**tuning)
        r = s.refine(cfg)
        return r, s.partition(), s.round_stats(), s.instance_km1(), s.block_weights()


def _same(a, b):
    ra, pa, sa, ka, ba = a
    rb, pb, sb, kb, bb = b
    assert np.array_equal(pa, pb)
    assert [[x[k] for k in KEYS] for x in sa] == [[x[k] for k in KEYS] for x in sb]
    assert np.array_equal(ka, kb) and np.array_equal(ba, bb)
    assert (ra.km1_before, ra.km1_after, ra.delta, ra.moves, ra.rounds) == \
           (rb.km1_before, rb.km1_after, rb.delta, rb.moves, rb.rounds)


@pytest.mark.parametrize("mode", range(len(MODES)))
@pytest.mark.parametrize("seed", [0, 1])
def test_persistent_equals_multi_launch(lp, orc, seed, mode):
    insts = _instances(seed, 24, hubs=seed == 1)
    m = MODES[mode]
    per = _run(lp, insts, lp.default_config(rounds=5, flags=lp.FLAG_PERSISTENT, **m))
    mul = _run(lp, insts, lp.default_config(rounds=5, flags=lp.FLAG_MULTI_LAUNCH, **m))
    _same(per, mul)
    r, part, _, km, _ = per
    assert r.km1_after == r.km1_before + r.delta == km.sum()
    off = np.cumsum([0] + [x.hg.n for x in insts])
    for i in range(0, len(insts), 5):  # a sample against the oracle, instance by instance
        x = insts[i]
        ref, _ = orc.lp_sync(x.hg, x.k, x.lmax, x.part, perfect=x.perfect, rounds=5, subrounds=m["subrounds"],
                             revert=m["revert"], rollback=m["rollback"], zero_gain=m["rebalancing"])
        assert np.array_equal(part[off[i]:off[i + 1]], ref), f"instance {i}"


@pytest.mark.parametrize("tuning", [dict(ctas_per_sm=1, unroll=4, order=0), dict(ctas_per_sm=2, unroll=8, order=1),
                                    dict(ctas_per_sm=2, unroll=4, order=0), dict(ctas_per_sm=1, unroll=8, order=1)])
def test_tuning_variants_give_identical_results(lp, tuning):
    insts = _instances(5, 40, hubs=True)
    base = _run(lp, insts, lp.default_config(rounds=4, flags=lp.FLAG_MULTI_LAUNCH))
    tuned = _run(lp, insts, lp.default_config(rounds=4), tuning=dict(mode=lp.MODE_PERSISTENT, **tuning))
    _same(base, tuned)


def test_single_instance_session_persistent(lp, orc):
    """A plain session runs as one instance of the persistent round (one CTA)."""
    from lpgpu import gen
    inst = gen.plain_small(seed=3)
    out = []
    for flags in (lp.FLAG_PERSISTENT, lp.FLAG_MULTI_LAUNCH):
        with lp.Session(0) as s:
            s.upload(inst.hg)
            s.set_partition(inst.k, inst.part, lmax=inst.lmax, perfect=inst.perfect)
            r = s.refine(lp.default_config(rounds=inst.rounds, flags=flags))
            out.append((r, s.partition(), s.round_stats(), np.array(s.metrics()[:1]), s.block_weights()))
    _same(out[0], out[1])
    ref, _ = orc.lp_sync(inst.hg, inst.k, inst.lmax, inst.part, perfect=inst.perfect, rounds=inst.rounds,
                         subrounds=7, revert=1, rollback=1, zero_gain=1)
    assert np.array_equal(out[0][1], ref)


def test_graph_replay_and_generated_batch(lp):
    """A batch of the generator's small instances, refined twice from the same
    start through the captured graph, equals the multi-launch pipeline."""
    from lpgpu import gen
    insts = [gen.batch_instance(0, i) for i in range(48)]
    cfg = lp.default_config(rounds=5, flags=lp.FLAG_PERSISTENT)
    with lp.Session(0) as s:
        s.upload_batch([x.hg for x in insts])
        s.set_partition_batch([x.k for x in insts], [x.part for x in insts], eps=0.03)
        s.save_partition()
        r1 = s.refine(cfg)
        p1 = s.partition()
        s.restore_partition()
        r2 = s.refine(cfg)
        p2 = s.partition()
        assert np.array_equal(p1, p2) and r1.km1_after == r2.km1_after
        km = s.instance_km1()
    mul = _run(lp, insts, lp.default_config(rounds=5, flags=lp.FLAG_MULTI_LAUNCH))
    assert np.array_equal(p1, mul[1]) and np.array_equal(km, mul[3])


def test_persistent_limits(lp):
    """k above 64: the forced form is rejected, a tuned one falls back to the
    multi-launch pipeline with the same result; refinement node lists too."""
    insts = _instances(9, 6, ks=(70, 3))
    assert max(x.k for x in insts) > lp.PERSISTENT_MAX_K
    with lp.Session(0) as s:
        s.upload_batch([x.hg for x in insts])
        s.set_partition_batch([x.k for x in insts], [x.part for x in insts], eps=0.03)
        with pytest.raises(lp.LpgpuError) as e:
            s.refine(lp.default_config(rounds=2, flags=lp.FLAG_PERSISTENT))
        assert e.value.status == lp.ERR_INVALID_ARG
    tuned = _run(lp, insts, lp.default_config(rounds=3), tuning=dict(mode=lp.MODE_PERSISTENT))
    base = _run(lp, insts, lp.default_config(rounds=3, flags=lp.FLAG_MULTI_LAUNCH))
    _same(tuned, base)
    with lp.Session(0) as s:
        x = insts[1]
        s.upload(x.hg)
        s.set_partition(x.k, x.part)
        with pytest.raises(lp.LpgpuError):
            s.refine(lp.default_config(rounds=2, flags=lp.FLAG_PERSISTENT), nodes=np.arange(5, dtype=np.int32))

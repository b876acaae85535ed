"""Batched sessions: many independent hypergraphs refined in the same launches.
Every instance must end exactly as when refined alone (device and oracle)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _instances(seed, count):
    from lpgpu import gen
    out = []
    rng = np.random.default_rng(seed)
    for i in range(count):
        n = int(rng.integers(40, 700))           # sizes not aligned to 32 on purpose
        m = int(n * rng.uniform(0.8, 1.4))
        k = int(rng.choice([2, 3, 4, 7, 16, 33]))
        out.append(gen.random_small(1000 * seed + i, n=n, m=m, k=k, max_size=9, weighted=bool(i % 2)))
    return out


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_batch_equals_instances_alone(lp, orc, seed):
    insts = _instances(seed, 12)
    cfg = lp.default_config(rounds=5, subrounds=4)
    with lp.Session(0) as s:
        s.upload_batch([x.hg for x in insts])
        s.set_partition_batch([x.k for x in insts], [x.part for x in insts], eps=0.03)
        before = s.instance_km1()
        r = s.refine(cfg)
        part = s.partition()
        after = s.instance_km1()
        total_km1 = s.metrics()[0]
    assert r.km1_after == r.km1_before + r.delta == total_km1 == after.sum()
    off = np.cumsum([0] + [x.hg.n for x in insts])
    for i, x in enumerate(insts):
        with lp.Session(0) as one:
            one.upload(x.hg)
            one.set_partition(x.k, x.part, eps=0.03)
            km0 = one.metrics()[0]
            one.refine(cfg)
            alone = one.partition()
            km1 = one.metrics()[0]
        assert np.array_equal(part[off[i]:off[i + 1]], alone), f"instance {i}"
        assert (before[i], after[i]) == (km0, km1)
        ref, _ = orc.lp_sync(x.hg, x.k, x.lmax, x.part, perfect=x.perfect, rounds=5, subrounds=4,
                             revert=1, rollback=1, zero_gain=1)
        assert np.array_equal(alone, ref)


def test_batch_state_and_errors(lp, orc):
    insts = _instances(7, 5)
    with lp.Session(0) as s:
        s.upload_batch([x.hg for x in insts])
        with pytest.raises(lp.LpgpuError) as e:
            s.set_partition(2, np.zeros(s.n, np.int32))
        assert e.value.status == lp.ERR_STATE
        s.set_partition_batch([x.k for x in insts], [x.part for x in insts])
        with pytest.raises(lp.LpgpuError):
            s.best_moves()
        bw = s.block_weights()
        kk = 0
        for x in insts:
            _, _, obw = orc.init_partition(x.hg, x.k, x.part)
            assert np.array_equal(bw[kk:kk + x.k], obw)
            kk += x.k
    with lp.Session(0) as s:
        bad = [insts[0].hg, insts[1].hg]
        from lpgpu import gen
        # a net that reaches into the next instance is rejected
        h = bad[0]
        pins = h.pins.copy()
        pins[0] = h.n  # first vertex of the next instance in union ids
        broken = gen.Hypergraph(h.n, h.m, h.net_off, pins, h.w_v, h.w_e)
        with pytest.raises(lp.LpgpuError) as e:
            s.upload_batch([broken, bad[1]])
        assert e.value.status == lp.ERR_INVALID_ARG


@pytest.mark.parametrize("seed", [3, 4])
def test_instance_buffers_equal_union(lp, seed):
    """lpgpu_session_upload_instances / _set_partition_instances /
    _get_partition_instances give the union API's results."""
    insts = _instances(seed, 9)
    cfg = lp.default_config(rounds=4, subrounds=4)
    with lp.Session(0) as a, lp.Session(0) as b:
        a.upload_batch([x.hg for x in insts])
        a.set_partition_batch([x.k for x in insts], [x.part for x in insts], eps=0.05)
        ra = a.refine(cfg)
        pa = a.partition()
        b.upload_instances([x.hg for x in insts])
        b.set_partition_instances([x.k for x in insts], [x.part for x in insts], eps=0.05)
        rb = b.refine(cfg)
        pb = b.partition_instances()
        assert (ra.km1_before, ra.km1_after, ra.delta) == (rb.km1_before, rb.km1_after, rb.delta)
        assert np.array_equal(np.concatenate(pb), pa)
        assert np.array_equal(a.instance_km1(), b.instance_km1())
        assert np.array_equal(a.pin_counts(), b.pin_counts())


@pytest.mark.parametrize("seed", range(2))
def test_instance_buffers_back_to_back(lp, seed):
    """Instances whose arrays lie back to back in shared buffers (copies that
    the library merges), some of them without nets or weights, give the same
    results as separate buffers; outputs written back to back as well."""
    from lpgpu import gen
    insts = _instances(seed + 20, 7)
    # an instance without nets and one with unit weights (NULL) in the middle
    empty = gen.Hypergraph(5, 0, np.zeros(1, np.int64), np.zeros(0, np.int32), np.ones(5, np.int32),
                           np.zeros(0, np.int32))
    hgs = [x.hg for x in insts[:3]] + [empty] + [x.hg for x in insts[3:]]
    ks = [x.k for x in insts[:3]] + [2] + [x.k for x in insts[3:]]
    parts = [x.part for x in insts[:3]] + [np.array([0, 1, 0, 1, 0], np.int32)] + [x.part for x in insts[3:]]

    def arena(arrays, dtype):
        buf = np.concatenate([np.asarray(a, dtype) for a in arrays]) if arrays else np.zeros(0, dtype)
        views, o = [], 0
        for a in arrays:
            views.append(buf[o:o + len(a)])
            o += len(a)
        return buf, views

    b_off, offs = arena([h.net_off for h in hgs], np.int64)
    b_pin, pins = arena([h.pins for h in hgs], np.int32)
    b_wv, wvs = arena([h.w_v for h in hgs], np.int32)
    b_we, wes = arena([h.w_e for h in hgs], np.int32)
    b_pt, pts = arena(parts, np.int32)
    packed = [gen.Hypergraph(h.n, h.m, offs[i], pins[i], wvs[i], None if i == 5 else wes[i])
              for i, h in enumerate(hgs)]
    loose = [gen.Hypergraph(h.n, h.m, h.net_off.copy(), h.pins.copy(), h.w_v.copy(),
                            None if i == 5 else h.w_e.copy()) for i, h in enumerate(hgs)]
    cfg = lp.default_config(rounds=4)
    with lp.Session(0) as a, lp.Session(0) as b:
        a.upload_instances(packed)
        a.set_partition_instances(ks, pts, eps=0.05)
        ra = a.refine(cfg)
        b_out, outs = arena([np.zeros(h.n, np.int32) for h in hgs], np.int32)
        a.partition_instances(outs)
        b.upload_instances(loose)
        b.set_partition_instances(ks, [p.copy() for p in parts], eps=0.05)
        rb = b.refine(cfg)
        pb = b.partition_instances()
        assert (ra.km1_before, ra.km1_after, ra.delta) == (rb.km1_before, rb.km1_after, rb.delta)
        assert all(np.array_equal(x, y) for x, y in zip(outs, pb))
        assert np.array_equal(a.pin_counts(), b.pin_counts())
        assert np.array_equal(a.instance_km1(), b.instance_km1())


def test_instance_buffers_are_checked(lp):
    from lpgpu import gen
    insts = _instances(5, 4)
    bad = insts[2].hg
    pins = bad.pins.copy()
    pins[3] = bad.n  # one past the instance's own vertices
    broken = gen.Hypergraph(bad.n, bad.m, bad.net_off, pins, bad.w_v, bad.w_e)
    with lp.Session(0) as s:
        with pytest.raises(lp.LpgpuError) as e:
            s.upload_instances([insts[0].hg, insts[1].hg, broken, insts[3].hg])
        assert e.value.status == lp.ERR_INVALID_ARG
        unit = [gen.Hypergraph(x.hg.n, x.hg.m, x.hg.net_off, x.hg.pins, None, None) for x in insts]
        s.upload_instances(unit)
        s.set_partition_instances([x.k for x in insts], [x.part for x in insts])
        bw = s.block_weights()
        assert bw.sum() == sum(x.hg.n for x in insts)


@pytest.mark.parametrize("api", ["union", "instances"])
def test_single_instance_batch(lp, orc, api):
    """A batch of one instance (every vertex belongs to instance 0) behaves like
    a plain session."""
    x = _instances(6, 1)[0]
    cfg = lp.default_config(rounds=4, subrounds=4)
    with lp.Session(0) as s:
        if api == "union":
            s.upload_batch([x.hg])
            s.set_partition_batch([x.k], [x.part], eps=0.03)
        else:
            s.upload_instances([x.hg])
            s.set_partition_instances([x.k], [x.part], eps=0.03)
        s.refine(cfg)
        got = s.partition()
    ref, _ = orc.lp_sync(x.hg, x.k, x.lmax, x.part, perfect=x.perfect, rounds=4, subrounds=4,
                         revert=1, rollback=1, zero_gain=1)
    assert np.array_equal(got, ref)

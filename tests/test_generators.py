"""Synthetic workload generators: shapes, ranges, determinism (CPU)."""
import numpy as np

from lpgpu import gen


def _check_csr(hg, min_size, max_size):
    sizes = np.diff(hg.net_off)
    assert hg.net_off[0] == 0 and hg.net_off[-1] == len(hg.pins)
    assert sizes.min() >= min_size and sizes.max() <= max_size
    assert hg.pins.min() >= 0 and hg.pins.max() < hg.n
    for e in range(0, hg.m, max(1, hg.m // 200)):
        p = hg.pins[hg.net_off[e]:hg.net_off[e + 1]]
        assert len(np.unique(p)) == len(p)
    deg = np.diff(hg.vtx_off)
    assert deg.sum() == len(hg.pins)
    # stable incidence: incident nets ascending per vertex
    for v in range(0, hg.n, max(1, hg.n // 200)):
        seg = hg.inets[hg.vtx_off[v]:hg.vtx_off[v + 1]]
        assert (np.diff(seg) > 0).all()


def test_plain_small_shape_and_determinism():
    a = gen.plain_small(seed=3)
    b = gen.plain_small(seed=3)
    assert a.hg.n == 16384 and a.hg.m == 16384 and a.k == 2
    _check_csr(a.hg, 2, 64)
    assert np.array_equal(a.hg.pins, b.hg.pins) and np.array_equal(a.part, b.part)
    sizes = np.diff(a.hg.net_off)
    assert 3.0 < sizes.mean() < 4.2
    assert np.bincount(a.part).tolist() == [8192, 8192]
    assert a.lmax[0] == 8437 and a.perfect[0] == 8192


def test_part_weights_formula():
    perfect, lmax = gen.part_weights(4194304, 128, 0.03)
    assert perfect[0] == 32768 and lmax[0] == 33751


def test_small_batch_and_served_instances():
    for i in range(3):
        bi = gen.batch_instance(1, i)
        assert 1024 <= bi.hg.n <= 65536 and bi.k in (2, 4, 8, 16)
        _check_csr(bi.hg, 2, 256)
    si = gen.served_request(1, 0, hi=8192)
    assert si.k in (2, 4, 8, 16, 32, 64)
    _check_csr(si.hg, 2, 4096)

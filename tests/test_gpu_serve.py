"""Served refinement on the device: requests refined in continuous batches end
exactly as when each is refined alone (plain loop and oracle)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests(serve, gen, count, seed, rate=4000.0):
    arr = serve.poisson_arrivals(count, rate, seed)
    out = []
    for i in range(count):
        x = gen.served_request(seed, i, lo=512, hi=20000, ks=(2, 3, 8, 33), rounds=4)
        out.append(serve.Request(i, x.hg, x.k, x.eps, x.part, x.rounds, float(arr[i])))
    return out


@pytest.mark.parametrize("slots", [1, 2])
def test_served_equals_plain_loop(lp, orc, slots):
    from lpgpu import gen, serve
    rs = _requests(serve, gen, 24, 3 + slots)
    rp = _requests(serve, gen, 24, 3 + slots)
    srv = serve.RefineServer(slots=slots, subrounds=8)
    st = serve.replay(srv, rs)
    assert not srv.errors
    serve.plain_loop(rp, subrounds=8)
    assert st.summary()["requests"] == 24
    assert max(st.batch_sizes) > 1  # requests were batched
    for a, b in zip(rs, rp):
        assert a.km1 == b.km1
        assert np.array_equal(a.result, b.result), f"request {a.rid}"
    for a in rs[:4]:
        x = gen.served_request(3 + slots, a.rid, lo=512, hi=20000, ks=(2, 3, 8, 33), rounds=4)
        ref, _ = orc.lp_sync(x.hg, x.k, x.lmax, x.part, perfect=x.perfect, rounds=4, subrounds=8,
                             revert=1, rollback=1, zero_gain=1)
        assert np.array_equal(a.result, ref)


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

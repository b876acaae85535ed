"""The allocation-free metrics entry point (lpgpu_partition_metrics_noalloc)
against the session path and the CPU oracle, through the C ABI.

It is meant for callers that must not allocate device memory (externally
owned memory pools or memory plans, latency-bound loops), so the test hands it
device buffers it owns itself (torch tensors) and compares block weights, km1
and cut with lpgpu_session_get_block_weights / lpgpu_session_metrics and with
the oracle's initializePartition block weights and metrics::km1 / cut,
exactly, on two calls in a row with different partitions (the shared scratch
array must be cleared between calls). This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _reference(lp, hg, k, part):
    with lp.Session(0) as s:
        s.upload(hg)
        s.set_partition(k, part)
        km1, cut, _ = s.metrics()
        return s.block_weights(), km1, cut


def test_noalloc_metrics_match_session_twice(lp, orc):
    torch = pytest.importorskip("torch")
    from lpgpu import gen
    inst = gen.random_small(3, n=3000, m=3600, k=37, max_size=14)
    hg, k = inst.hg, inst.k
    dev = torch.device("cuda:0")
    d_off = torch.from_numpy(np.ascontiguousarray(hg.net_off)).to(dev)
    d_pins = torch.from_numpy(np.ascontiguousarray(hg.pins)).to(dev)
    d_wv = torch.from_numpy(np.ascontiguousarray(hg.w_v)).to(dev)
    d_we = torch.from_numpy(np.ascontiguousarray(hg.w_e)).to(dev)
    L = lp.lib()
    fn = L.lpgpu_partition_metrics_noalloc
    fn.argtypes = [ctypes.c_int64, ctypes.c_int64] + [ctypes.c_void_p] * 5 + [ctypes.c_int32] + \
                  [ctypes.c_void_p] * 4
    fn.restype = ctypes.c_int
    rng = np.random.default_rng(11)
    parts = [inst.part, rng.integers(0, k, size=hg.n).astype(np.int32)]
    for part in parts:
        d_part = torch.from_numpy(np.ascontiguousarray(part)).to(dev)
        d_bw = torch.full((k,), -1, dtype=torch.int64, device=dev)
        d_km1 = torch.full((1,), -1, dtype=torch.int64, device=dev)
        d_cut = torch.full((1,), -1, dtype=torch.int64, device=dev)
        torch.cuda.synchronize()
        st = fn(hg.n, hg.m, d_off.data_ptr(), d_pins.data_ptr(), d_wv.data_ptr(), d_we.data_ptr(),
                d_part.data_ptr(), k, d_bw.data_ptr(), d_km1.data_ptr(), d_cut.data_ptr(), None)
        assert st == lp.OK, L.lpgpu_last_error()
        torch.cuda.synchronize()
        bw, km1, cut = _reference(lp, hg, k, part)
        assert np.array_equal(d_bw.cpu().numpy(), bw)
        assert int(d_km1.item()) == km1 and int(d_cut.item()) == cut
        _, conn, obw = orc.init_partition(hg, k, part)
        okm1, ocut = orc.metrics(hg, k, conn)
        assert np.array_equal(d_bw.cpu().numpy(), obw)
        assert (int(d_km1.item()), int(d_cut.item())) == (okm1, ocut)


def test_noalloc_rejects_k_beyond_scratch(lp):
    L = lp.lib()
    fn = L.lpgpu_partition_metrics_noalloc
    fn.argtypes = [ctypes.c_int64, ctypes.c_int64] + [ctypes.c_void_p] * 5 + [ctypes.c_int32] + \
                  [ctypes.c_void_p] * 4
    fn.restype = ctypes.c_int
    st = fn(0, 0, None, None, None, None, None, lp.MAX_K + 1, None, None, None, None)
    assert st == lp.ERR_INVALID_ARG
    assert b"1024" in L.lpgpu_last_error()


def test_noalloc_rejects_nets_without_vertices(lp):
    """Host-side checks only: no pointer is dereferenced for a rejected call."""
    L = lp.lib()
    fn = L.lpgpu_partition_metrics_noalloc
    fn.argtypes = [ctypes.c_int64, ctypes.c_int64] + [ctypes.c_void_p] * 5 + [ctypes.c_int32] + \
                  [ctypes.c_void_p] * 4
    fn.restype = ctypes.c_int
    dummy = ctypes.c_void_p(16)
    st = fn(0, 3, dummy, dummy, None, None, None, 2, dummy, dummy, dummy, None)
    assert st == lp.ERR_INVALID_ARG
    assert b"nets without vertices" in L.lpgpu_last_error()

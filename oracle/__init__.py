"""ctypes front end of the CPU oracle (test infrastructure only).

Only the test suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this package, always as the checker / baseline, never as
the measured or shipped path.
"""
import ctypes
import os

import numpy as np

from .build import SO, build_oracle

_lib = None

I64P = ctypes.POINTER(ctypes.c_int64)
I32P = ctypes.POINTER(ctypes.c_int32)
U32P = ctypes.POINTER(ctypes.c_uint32)
U8P = ctypes.POINTER(ctypes.c_uint8)


class RoundStats(ctypes.Structure):
    _fields_ = [("active", ctypes.c_int64), ("pins", ctypes.c_int64),
                ("candidates", ctypes.c_int64), ("moved", ctypes.c_int64),
                ("reverted", ctypes.c_int64), ("delta", ctypes.c_int64),
                ("km1_after", ctypes.c_int64), ("seconds", ctypes.c_double)]


class LpCfg(ctypes.Structure):
    _fields_ = [("rounds", ctypes.c_int32), ("activation_threshold", ctypes.c_int32),
                ("subrounds", ctypes.c_int32), ("revert", ctypes.c_int32),
                ("rollback", ctypes.c_int32), ("threads", ctypes.c_int32),
                ("zero_gain", ctypes.c_int32), ("seed", ctypes.c_int64)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(SO):
            build_oracle()
        _lib = ctypes.CDLL(SO)
    return _lib


def _p(a, t):
    return a.ctypes.data_as(t)


def transpose(n, net_off, pins):
    m = len(net_off) - 1
    vtx_off = np.zeros(n + 1, np.int64)
    inets = np.zeros(len(pins), np.int32)
    lib().orc_transpose(ctypes.c_int64(n), ctypes.c_int64(m), _p(net_off, I64P), _p(pins, I32P),
                        _p(vtx_off, I64P), _p(inets, I32P))
    return vtx_off, inets


def init_partition(hg, k, part):
    m = hg.m
    W = (k + 31) // 32
    phi = np.zeros(m * k, np.int32)
    conn = np.zeros(m * W, np.uint32)
    bw = np.zeros(k, np.int64)
    lib().orc_init_partition(ctypes.c_int64(hg.n), ctypes.c_int64(m), _p(hg.net_off, I64P),
                             _p(hg.pins, I32P), _p(hg.w_v, I32P), ctypes.c_int32(k),
                             _p(np.ascontiguousarray(part, np.int32), I32P),
                             _p(phi, I32P), _p(conn, U32P), _p(bw, I64P))
    return phi.reshape(m, k), conn.reshape(m, W), bw


def metrics(hg, k, conn):
    km1 = ctypes.c_int64()
    cut = ctypes.c_int64()
    c = np.ascontiguousarray(conn, np.uint32)
    lib().orc_metrics(ctypes.c_int64(hg.m), _p(hg.w_e, I32P), ctypes.c_int32(k), _p(c, U32P),
                      ctypes.byref(km1), ctypes.byref(cut))
    return km1.value, cut.value


def _hg_args(hg):
    return (ctypes.c_int64(hg.n), ctypes.c_int64(hg.m), _p(hg.net_off, I64P), _p(hg.pins, I32P),
            _p(hg.vtx_off, I64P), _p(hg.inets, I32P), _p(hg.w_v, I32P), _p(hg.w_e, I32P))


def best_moves(hg, k, part, lmax):
    n = hg.n
    to = np.zeros(n, np.int32)
    gain = np.zeros(n, np.int32)
    border = np.zeros(n, np.uint8)
    lm = np.ascontiguousarray(lmax, np.int64)
    lib().orc_best_moves(*_hg_args(hg), ctypes.c_int32(k),
                         _p(np.ascontiguousarray(part, np.int32), I32P), _p(lm, I64P),
                         _p(to, I32P), _p(gain, I32P), _p(border, U8P))
    return to, gain, border.astype(bool)


def gain_cache(hg, k, part):
    n = hg.n
    benefit = np.zeros(n, np.int32)
    penalty = np.zeros(n * k, np.int32)
    lib().orc_gain_cache(*_hg_args(hg), ctypes.c_int32(k),
                         _p(np.ascontiguousarray(part, np.int32), I32P),
                         _p(benefit, I32P), _p(penalty, I32P))
    return benefit, penalty.reshape(n, k)


def _cfg(rounds=5, activation_threshold=100, subrounds=1, revert=0, rollback=0, threads=1,
         zero_gain=0, seed=0):
    return LpCfg(rounds, activation_threshold, subrounds, revert, rollback, threads, zero_gain, seed)


def lp_sync(hg, k, lmax, part, perfect=None, **cfg):
    c = _cfg(**cfg)
    p = np.array(part, np.int32, copy=True)
    stats = (RoundStats * max(1, c.rounds))()
    lm = np.ascontiguousarray(lmax, np.int64)
    pf = None if perfect is None else np.ascontiguousarray(perfect, np.int64)
    r = lib().orc_lp_sync(*_hg_args(hg), ctypes.c_int32(k), _p(lm, I64P),
                          None if pf is None else _p(pf, I64P), _p(p, I32P),
                          ctypes.byref(c), stats)
    return p, [_stat_dict(stats[i]) for i in range(r)]


def rebalance(hg, k, lmax, part, max_rounds=16):
    """Deterministic rebalancer (orc_rebalance): partition and per-round stats."""
    p = np.array(part, np.int32, copy=True)
    stats = (RoundStats * (max_rounds + 1))()
    lm = np.ascontiguousarray(lmax, np.int64)
    r = lib().orc_rebalance(*_hg_args(hg), ctypes.c_int32(k), _p(lm, I64P), _p(p, I32P),
                            ctypes.c_int32(max_rounds), stats)
    return p, [_stat_dict(stats[i]) for i in range(r)]


def repair_empty_blocks(hg, k, lmax, part):
    """Moves of repairEmptyBlocks (orc_repair_empty_blocks): (vertex, from, to, gain) per
    empty block that received one, in block order; gain is km1Gain (positive = better)."""
    out = [np.zeros(max(1, k), np.int32) for _ in range(4)]
    lm = np.ascontiguousarray(lmax, np.int64)
    c = lib().orc_repair_empty_blocks(*_hg_args(hg), ctypes.c_int32(k), _p(lm, I64P),
                                      _p(np.ascontiguousarray(part, np.int32), I32P),
                                      *[_p(a, I32P) for a in out])
    return [tuple(int(a[i]) for a in out) for i in range(c)]


def lp_async(hg, k, lmax, perfect, part, **cfg):
    c = _cfg(**cfg)
    p = np.array(part, np.int32, copy=True)
    stats = (RoundStats * max(1, c.rounds))()
    lm = np.ascontiguousarray(lmax, np.int64)
    pf = np.ascontiguousarray(perfect, np.int64)
    r = lib().orc_lp_async(*_hg_args(hg), ctypes.c_int32(k), _p(lm, I64P), _p(pf, I64P),
                           _p(p, I32P), ctypes.byref(c), stats)
    return p, [_stat_dict(stats[i]) for i in range(r)]


def _stat_dict(s):
    return {f: getattr(s, f) for f, _ in RoundStats._fields_}

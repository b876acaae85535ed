"""Seeded synthetic hypergraphs and initial partitions for the LP refinement workloads.

Every generator is deterministic in its seed (numpy PCG64). Nets are stored as
CSR (``net_off`` int64[m+1], ``pins`` int32[P]); duplicate pins inside a net are
removed and a net that falls below the minimum size after removal is redrawn.

Workloads (all ids int32):

* ``plain_small``  -- 16,384 vertices and nets, geometric net sizes (mean 3.5,
  clipped to [2, 64]), pins uniform in a +-512 window of an anchor vertex, unit
  weights, k = 2, eps = 0.03, random balanced initial partition.
* ``plain_large``  -- 1,048,576 vertices, 1,258,291 nets, Zipf(2.2) net sizes on
  [2, 4096], 80 % of pins in a +-4096 window and 20 % uniform, vertex weights
  U[1, 4], net weights U[1, 8], k = 32, eps = 0.03, weight-balanced greedy
  initial partition.
* ``rownet``       -- row-net model of a 4,194,304 x 4,194,304 sparse pattern
  with ~32M nonzeros: power-law row degrees on [1, 8192] (exponent calibrated
  from 2.0 so that the expected nonzero count is 32M), column ids 50 % in a
  +-16,384 band around the diagonal and 50 % uniform, unit weights, k = 128,
  eps = 0.03, contiguous blocks with 10 % of vertices reassigned at random.
* ``batch``        -- many small instances: vertex counts log-uniform in
  [1,024, 65,536], nets = 1.1 x vertices, geometric net sizes (mean 4, [2, 256]),
  +-512 window pins, k uniform in {2, 4, 8, 16}.
* ``served``       -- request sizes log-uniform in [1,024, 2,097,152] vertices,
  nets = 1.2 x vertices, Zipf(2.2) net sizes on [2, 4096] as in plain_large,
  k uniform in {2, 4, 8, 16, 32, 64}.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Hypergraph:
    n: int
    m: int
    net_off: np.ndarray      # int64[m+1]
    pins: np.ndarray         # int32[P]
    w_v: np.ndarray          # int32[n]
    w_e: np.ndarray          # int32[m]
    vtx_off: np.ndarray = None  # int64[n+1] (filled by with_incidence)
    inets: np.ndarray = None    # int32[P]
    meta: dict = field(default_factory=dict)

    @property
    def num_pins(self) -> int:
        return int(self.net_off[-1])

    def with_incidence(self) -> "Hypergraph":
        """Stable vertex -> incident-net transpose (incident nets in increasing id)."""
        if self.vtx_off is None:
            deg = np.bincount(self.pins, minlength=self.n).astype(np.int64)
            vtx_off = np.zeros(self.n + 1, np.int64)
            np.cumsum(deg, out=vtx_off[1:])
            net_of_pin = np.repeat(np.arange(self.m, dtype=np.int32),
                                   np.diff(self.net_off).astype(np.int64))
            order = np.argsort(self.pins, kind="stable")
            self.vtx_off = vtx_off
            self.inets = np.ascontiguousarray(net_of_pin[order], np.int32)
        return self


def part_weights(total_weight: int, k: int, eps: float):
    """Perfect and maximum block weights (context.cpp:237-250 of the reference):
    perfect = ceil(W / k) and max = (HypernodeWeight)((1 + eps) * perfect)."""
    perfect = int(math.ceil(total_weight / float(k)))
    lmax = int((1.0 + eps) * perfect)
    return np.full(k, perfect, np.int64), np.full(k, lmax, np.int64)


# --------------------------------------------------------------------------- nets

def _sorted_unique(a):
    a = np.sort(a, kind="stable")
    if len(a) == 0:
        return a
    keep = np.empty(len(a), bool)
    keep[0] = True
    np.not_equal(a[1:], a[:-1], out=keep[1:])
    return a[keep]


def _build_csr(n, sizes, draw_pins, rng, min_size):
    """Draw pins for every net, remove duplicates, redraw nets below min_size."""
    m = len(sizes)
    sizes = np.asarray(sizes, np.int64)
    net_ids = np.repeat(np.arange(m, dtype=np.int64), sizes)
    pins = draw_pins(net_ids, rng)
    keys = _sorted_unique(net_ids * n + pins)
    counts = np.bincount(keys // n, minlength=m)
    bad = np.nonzero(counts < min_size)[0]
    tries = 0
    while len(bad) > 0:
        tries += 1
        if tries > 64:
            raise RuntimeError("net redraw did not converge")
        keep = counts[keys // n] >= min_size
        keys = keys[keep]
        bad_ids = np.repeat(bad.astype(np.int64), sizes[bad])
        new = _sorted_unique(bad_ids * n + draw_pins(bad_ids, rng))
        keys = _sorted_unique(np.concatenate([keys, new]))
        counts = np.bincount(keys // n, minlength=m)
        bad = np.nonzero(counts < min_size)[0]
    net_off = np.zeros(m + 1, np.int64)
    np.cumsum(counts, out=net_off[1:])
    return net_off, (keys % n).astype(np.int32)


def _window_pins(n, anchors, window, uniform_frac=0.0):
    def draw(net_ids, rng):
        a = anchors[net_ids]
        p = a + rng.integers(-window, window + 1, size=len(net_ids))
        if uniform_frac > 0:
            u = rng.random(len(net_ids)) < uniform_frac
            p = np.where(u, rng.integers(0, n, size=len(net_ids)), p)
        return np.clip(p, 0, n - 1).astype(np.int64)
    return draw


def _zipf_sizes(rng, count, alpha, lo, hi):
    d = np.arange(lo, hi + 1, dtype=np.float64)
    cdf = np.cumsum(d ** -alpha)
    cdf /= cdf[-1]
    return (lo + np.searchsorted(cdf, rng.random(count), side="right")).astype(np.int64).clip(lo, hi)


def _geom_sizes(rng, count, mean, lo, hi):
    return np.clip(rng.geometric(1.0 / mean, size=count), lo, hi).astype(np.int64)


def _powerlaw_alpha_for_mean(target_mean, lo, hi):
    """Exponent of a power law on [lo, hi] whose mean equals target_mean (bisection)."""
    d = np.arange(lo, hi + 1, dtype=np.float64)

    def mean(a):
        p = d ** -a
        return float((d * p).sum() / p.sum())

    a_lo, a_hi = 1.0, 3.0
    for _ in range(100):
        mid = 0.5 * (a_lo + a_hi)
        if mean(mid) > target_mean:
            a_lo = mid
        else:
            a_hi = mid
    return 0.5 * (a_lo + a_hi)


# ----------------------------------------------------------------- partitions

def random_balanced_partition(n, k, rng):
    """Random permutation; the vertex at rank i goes to block i mod k."""
    part = np.empty(n, np.int32)
    part[rng.permutation(n)] = (np.arange(n) % k).astype(np.int32)
    return part


def greedy_weight_partition(w_v, k, rng):
    """Random permutation, each vertex to the currently lightest block (lowest id on ties)."""
    import heapq
    n = len(w_v)
    order = rng.permutation(n)
    heap = [(0, b) for b in range(k)]
    part = np.empty(n, np.int32)
    wl = w_v.tolist()
    for v in order.tolist():
        w, b = heap[0]
        part[v] = b
        heapq.heapreplace(heap, (w + wl[v], b))
    return part


def contiguous_perturbed_partition(n, k, frac, rng):
    part = (np.arange(n, dtype=np.int64) * k // n).astype(np.int32)
    sel = rng.choice(n, size=int(round(frac * n)), replace=False)
    part[sel] = rng.integers(0, k, size=len(sel)).astype(np.int32)
    return part


# ------------------------------------------------------------------ workloads

@dataclass
class Instance:
    name: str
    hg: Hypergraph
    k: int
    eps: float
    part: np.ndarray
    rounds: int
    perfect: np.ndarray = None
    lmax: np.ndarray = None

    def __post_init__(self):
        total = int(self.hg.w_v.sum())
        self.perfect, self.lmax = part_weights(total, self.k, self.eps)


def plain_small(seed=0, n=16384, m=16384, k=2, eps=0.03, rounds=5) -> Instance:
    rng = np.random.default_rng([seed, 1])
    sizes = _geom_sizes(rng, m, 3.5, 2, 64)
    anchors = rng.integers(0, n, size=m)
    net_off, pins = _build_csr(n, sizes, _window_pins(n, anchors, 512), rng, 2)
    hg = Hypergraph(n, m, net_off, pins, np.ones(n, np.int32), np.ones(m, np.int32)).with_incidence()
    part = random_balanced_partition(n, k, np.random.default_rng([seed, 2]))
    return Instance("plain_small", hg, k, eps, part, rounds)


def plain_large(seed=0, n=1048576, m=1258291, k=32, eps=0.03, rounds=10) -> Instance:
    rng = np.random.default_rng([seed, 11])
    sizes = _zipf_sizes(rng, m, 2.2, 2, 4096)
    anchors = rng.integers(0, n, size=m)
    net_off, pins = _build_csr(n, sizes, _window_pins(n, anchors, 4096, 0.2), rng, 2)
    w_v = rng.integers(1, 5, size=n).astype(np.int32)
    w_e = rng.integers(1, 9, size=m).astype(np.int32)
    hg = Hypergraph(n, m, net_off, pins, w_v, w_e).with_incidence()
    part = greedy_weight_partition(w_v, k, np.random.default_rng([seed, 12]))
    return Instance("plain_large", hg, k, eps, part, rounds)


ROWNET_TARGET_NNZ = 32 * 1024 * 1024


def rownet(seed=0, n=4194304, k=128, eps=0.03, rounds=10, target_nnz=None) -> Instance:
    """Row-net model: each row is a net, each column a vertex (square pattern)."""
    m = n
    target = ROWNET_TARGET_NNZ * n / 4194304 if target_nnz is None else target_nnz
    hi = 8192
    alpha = _powerlaw_alpha_for_mean(target / m, 1, hi)
    rng = np.random.default_rng([seed, 21])
    d = np.arange(1, hi + 1, dtype=np.float64)
    cdf = np.cumsum(d ** -alpha)
    cdf /= cdf[-1]
    sizes = (1 + np.searchsorted(cdf, rng.random(m), side="right")).astype(np.int64).clip(1, hi)
    band = min(16384, n // 2)
    diag = (np.arange(m, dtype=np.int64) * n) // m
    net_off, pins = _build_csr(n, sizes, _window_pins(n, diag, band, 0.5), rng, 1)
    hg = Hypergraph(n, m, net_off, pins, np.ones(n, np.int32), np.ones(m, np.int32)).with_incidence()
    hg.meta["alpha"] = alpha
    part = contiguous_perturbed_partition(n, k, 0.10, np.random.default_rng([seed, 22]))
    return Instance("rownet", hg, k, eps, part, rounds)


def seed_partition(inst: Instance, seed: int) -> np.ndarray:
    """The initial partition of a plain workload drawn with another seed (the
    workload's own rule: random balanced for plain_small, weight-balanced greedy
    for plain_large, contiguous blocks with 10 % reassigned for rownet), for
    runs over several seeds on one hypergraph."""
    hg = inst.hg
    if inst.name == "plain_small":
        return random_balanced_partition(hg.n, inst.k, np.random.default_rng([seed, 2]))
    if inst.name == "plain_large":
        return greedy_weight_partition(hg.w_v, inst.k, np.random.default_rng([seed, 12]))
    if inst.name == "rownet":
        return contiguous_perturbed_partition(hg.n, inst.k, 0.10, np.random.default_rng([seed, 22]))
    raise ValueError(f"no seed partition rule for {inst.name}")


def batch_instance(seed, idx, lo=1024, hi=65536, ks=(2, 4, 8, 16), eps=0.03, rounds=5,
                   incidence=True) -> Instance:
    rng = np.random.default_rng([seed, 31, idx])
    n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
    m = int(round(1.1 * n))
    k = int(rng.choice(ks))
    sizes = _geom_sizes(rng, m, 4.0, 2, 256)
    anchors = rng.integers(0, n, size=m)
    net_off, pins = _build_csr(n, sizes, _window_pins(n, anchors, 512), rng, 2)
    hg = Hypergraph(n, m, net_off, pins, np.ones(n, np.int32), np.ones(m, np.int32))
    if incidence:
        hg.with_incidence()
    part = random_balanced_partition(n, k, rng)
    return Instance(f"batch[{idx}]", hg, k, eps, part, rounds)


def served_request(seed, idx, lo=1024, hi=2097152, ks=(2, 4, 8, 16, 32, 64), eps=0.03,
                   rounds=8, incidence=True) -> Instance:
    rng = np.random.default_rng([seed, 41, idx])
    n = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
    m = int(round(1.2 * n))
    k = int(rng.choice(ks))
    sizes = _zipf_sizes(rng, m, 2.2, 2, min(4096, n))
    anchors = rng.integers(0, n, size=m)
    net_off, pins = _build_csr(n, sizes, _window_pins(n, anchors, 4096, 0.2), rng, 2)
    w_v = rng.integers(1, 5, size=n).astype(np.int32)
    w_e = rng.integers(1, 9, size=m).astype(np.int32)
    hg = Hypergraph(n, m, net_off, pins, w_v, w_e)
    if incidence:
        hg.with_incidence()
    part = random_balanced_partition(n, k, rng)
    return Instance(f"served[{idx}]", hg, k, eps, part, rounds)


def random_small(seed, n=200, m=240, k=4, max_size=8, weighted=True, eps=0.03, rounds=5, hubs=0,
                 hub_frac=0.2, vw_hi=5) -> Instance:
    """Small random hypergraph for property tests (includes degree-0 vertices).

    `hubs` > 0 sends a fraction `hub_frac` of the pins to `hubs` high-degree
    vertices (ids spaced n / hubs apart); vertex weights are drawn from
    [1, vw_hi)."""
    rng = np.random.default_rng([seed, 51])
    sizes = rng.integers(2, max_size + 1, size=m)

    def pick(ids, r):
        x = r.integers(0, n, size=len(ids))
        if hubs:
            h = r.random(len(ids)) < hub_frac
            x[h] = r.integers(0, hubs, size=int(h.sum())) * (n // hubs)
        return x

    net_off, pins = _build_csr(n, sizes, pick, rng, 2)
    w_v = rng.integers(1, vw_hi, size=n).astype(np.int32) if weighted else np.ones(n, np.int32)
    w_e = rng.integers(1, 9, size=m).astype(np.int32) if weighted else np.ones(m, np.int32)
    hg = Hypergraph(n, m, net_off, pins, w_v, w_e).with_incidence()
    part = random_balanced_partition(n, k, rng)
    return Instance(f"random[{seed}]", hg, k, eps, part, rounds)


def _one(name, seed, idx, kw=None):
    return globals()[name](seed, idx, incidence=False, **(kw or {}))


def generate_many(name, seed, count, processes=None, **kw):
    """Instances idx = 0..count-1 of `batch_instance` / `served_request` (extra
    keyword arguments passed on), built in a spawn-context process pool (safe
    after a CUDA context exists; the calling script needs a main guard)."""
    import multiprocessing as mp
    import os
    procs = processes or min(count, os.cpu_count() or 1)
    if procs <= 1:
        return [_one(name, seed, i, kw) for i in range(count)]
    with mp.get_context("spawn").Pool(procs) as pool:
        return pool.starmap(_one, [(name, seed, i, kw) for i in range(count)],
                            chunksize=max(1, count // (4 * procs)))


WORKLOADS = {
    "plain_small": plain_small,
    "plain_large": plain_large,
    "rownet": rownet,
}

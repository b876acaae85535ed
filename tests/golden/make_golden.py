"""Generates the committed golden fixtures under tests/golden/.

Inputs are the reference's own hMetis test instances (tests/instances/*.hgr of
the Mt-KaHyPar source tree). They are parsed with the reference reader's rules
(mt-kahypar/io/hypergraph_io.cpp:95-333: '%' comment lines, header
"nets vertices [type]", type 1 = net weights, 10 = vertex weights, 11 = both,
1-based pins, single-pin nets dropped) and stored as CSR .npz files, so the
test suite needs no access to the reference tree. For every fixture the
CPU oracle's outputs (Φ, Λ, km1, best moves, gain cache, a synchronous LP run)
are stored beside the input as golden vectors.

Run from the repository root:  python tests/golden/make_golden.py <reference_root>
(the Mt-KaHyPar source tree; MTK_REFERENCE_ROOT is read when no argument is given)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "mt-kahypar_gb300"))

from lpgpu import gen  # noqa: E402
import oracle  # noqa: E402

INSTANCES = ["twocenters.hgr", "contracted_unweighted_ibm01.hgr", "contracted_ibm01.hgr",
             "hypergraph_with_node_and_edge_weights.hgr", "karate_club.graph.hgr",
             "test_instance.hgr", "powersim.mtx.hgr"]


def read_hgr(path):
    with open(path) as f:
        lines = [ln for ln in f.read().split("\n")]
    it = iter(ln for ln in lines if not ln.startswith("%"))
    header = next(it).split()
    m_file, n = int(header[0]), int(header[1])
    typ = int(header[2]) if len(header) > 2 else 0
    has_ew = typ in (1, 11)
    has_vw = typ in (10, 11)
    offs = [0]
    pins = []
    wts = []
    for _ in range(m_file):
        tok = [int(t) for t in next(it).split()]
        w = 1
        if has_ew:
            w, tok = tok[0], tok[1:]
        if len(tok) < 2:      # single-pin net: dropped by the reference reader
            continue
        pins.extend(p - 1 for p in tok)
        offs.append(len(pins))
        wts.append(w)
    vw = np.ones(n, np.int32)
    if has_vw:
        for v in range(n):
            vw[v] = int(next(it).split()[0])
    hg = gen.Hypergraph(n, len(wts), np.array(offs, np.int64), np.array(pins, np.int32),
                        vw, np.array(wts, np.int32))
    return hg.with_incidence()


def main(ref_root):
    inst_dir = os.path.join(ref_root, "tests", "instances")
    for name in INSTANCES:
        hg = read_hgr(os.path.join(inst_dir, name))
        out = {"n": hg.n, "m": hg.m, "net_off": hg.net_off, "pins": hg.pins, "w_v": hg.w_v, "w_e": hg.w_e}
        for k in (2, 3, 8):
            part = gen.random_balanced_partition(hg.n, k, np.random.default_rng([7, k]))
            perfect, lmax = gen.part_weights(int(hg.w_v.sum()), k, 0.25)
            phi, conn, bw = oracle.init_partition(hg, k, part)
            km1, cut = oracle.metrics(hg, k, conn)
            to, gain, border = oracle.best_moves(hg, k, part, lmax)
            ben, pen = oracle.gain_cache(hg, k, part)
            p_lp, stats = oracle.lp_sync(hg, k, lmax, part, perfect=perfect, rounds=5, subrounds=4,
                                         revert=1, rollback=1, zero_gain=1)
            out.update({f"k{k}_part": part, f"k{k}_lmax": lmax, f"k{k}_perfect": perfect,
                        f"k{k}_phi": phi, f"k{k}_conn": conn, f"k{k}_bw": bw,
                        f"k{k}_km1": km1, f"k{k}_cut": cut, f"k{k}_to": to, f"k{k}_gain": gain,
                        f"k{k}_border": border, f"k{k}_benefit": ben, f"k{k}_penalty": pen,
                        f"k{k}_lp_part": p_lp,
                        f"k{k}_lp_delta": np.array([s["delta"] for s in stats], np.int64)})
        np.savez_compressed(os.path.join(HERE, name.replace(".hgr", ".npz")), **out)
        print(name, hg.n, hg.m, hg.num_pins)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MTK_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: make_golden.py <reference_root>  (or set MTK_REFERENCE_ROOT)")
    main(root)

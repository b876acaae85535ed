"""Autotuner of the batched refinement: times every variant on this GPU and
writes the tuning table the library loads at start-up.

Search space (lpgpu_tuning):
  * mode: the multi-launch sub-round pipeline over the union hypergraph, or
    persistent rounds (one launch per round, instances as work items);
  * persistent: resident CTAs per SM (1: up to 128 registers, 2: up to 64),
    sweep unroll (4 or 8 incidences per lane step), work order (largest
    instance first, or instance order).

Workloads: batches drawn like the batched benchmark (geometric net sizes of
mean 4, locality-window pins, k in {2, 4, 8, 16}, 5 rounds), one batch per
instance-size class, plus an instance-count sweep of the mixed class. Each
variant is timed on the device (CUDA events around refine only, the start
partition restored between repetitions) and must give the same per-instance
km1 as the multi-launch pipeline; a variant that does not is an error.

Table: for every class the fastest variant, valid up to the geometric mean of
this class's and the next class's mean instance size, and from the smallest
instance count at which persistent rounds won the count sweep.

  python -m lpgpu.autotune [--out PATH] [--quick]
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time

import numpy as np

# (name, smallest vertex count, largest vertex count, instances)
CLASSES = [
    ("tiny", 1024, 4096, 4096),
    ("small", 4096, 16384, 2048),
    ("medium", 16384, 65536, 512),
    ("large", 65536, 262144, 128),
]
COUNTS = [38, 76, 152, 304, 608, 1216, 4096]  # instance-count sweep on the mixed class


def _batch(lo, hi, count, seed):
    from . import gen
    return gen.generate_many("batch_instance", seed, count, lo=lo, hi=hi)


def _variants(lp):
    out = [("multi-launch", None)]
    for c in (1, 2):
        for u in (4, 8):
            for o in (0, 1):
                out.append((f"persistent c{c} u{u} o{o}",
                            dict(mode=lp.MODE_PERSISTENT, ctas_per_sm=c, unroll=u, order=o)))
    return out


def time_batch(lp, insts, reps=3, rounds=5, variants=None):
    """Device ms per refine of every variant on one batch; checks identical km1."""
    res = []
    with lp.Session(0) as s:
        s.upload_instances([x.hg for x in insts])
        s.set_partition_instances([x.k for x in insts], [x.part for x in insts], eps=0.03)
        s.save_partition()
        base = None
        for name, tu in (variants or _variants(lp)):
            if tu:
                s.set_tuning(**tu)
                cfg = lp.default_config(rounds=rounds)
            else:
                s.set_tuning(None)
                cfg = lp.default_config(rounds=rounds, flags=lp.FLAG_MULTI_LAUNCH)
            s.restore_partition()
            s.refine(cfg)  # warm-up (graph capture)
            ms = 0.0
            for _ in range(reps):
                s.restore_partition()
                s.synchronize()
                s.record(0)
                s.refine(cfg)
                s.record(1)
                ms += s.elapsed_ms(0, 1)
            km = s.instance_km1()
            if base is None:
                base = km
            elif not np.array_equal(km, base):
                raise RuntimeError(f"variant {name} changed the result")
            res.append({"variant": name, "tuning": tu, "ms": ms / reps})
    return res


def build_table(class_results, count_results):
    """Rows in increasing class size; see the module docstring."""
    # smallest count from which persistent rounds win at every larger count of the sweep
    min_inst = None
    for row in sorted(count_results, key=lambda r: -r["count"]):
        best = min(row["results"], key=lambda r: r["ms"])
        if best["tuning"] is None:
            break
        min_inst = row["count"]
    if min_inst is None:
        min_inst = 1 << 30  # persistent rounds never won: the table keeps the multi-launch form
    rows = []
    for i, cr in enumerate(class_results):
        best = min(cr["results"], key=lambda r: r["ms"])
        nxt = class_results[i + 1]["mean_pins"] if i + 1 < len(class_results) else 2 * cr["mean_pins"]
        bound = int(math.sqrt(cr["mean_pins"] * nxt))
        tu = best["tuning"] or {"mode": 0, "ctas_per_sm": 2, "unroll": 8, "order": 0}
        rows.append({"class": cr["class"], "max_mean_pins": bound, "min_instances": int(min_inst), **tu})
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=None, help="table path (default: the package's tuning_gb300.json)")
    ap.add_argument("--quick", action="store_true", help="quarter-size batches, one repetition")
    args = ap.parse_args(argv)
    import lpgpu as lp
    # every instance is drawn before the first CUDA call (spawn pool)
    scale = 4 if args.quick else 1
    reps = 1 if args.quick else 3
    batches = [(name, _batch(lo, hi, max(8, cnt // scale), 100 + i))
               for i, (name, lo, hi, cnt) in enumerate(CLASSES)]
    mixed = _batch(1024, 65536, max(COUNTS) // scale, 7)
    lp.build()
    t0 = time.time()
    class_results = []
    for name, insts in batches:
        res = time_batch(lp, insts, reps=reps)
        mean_pins = int(np.mean([x.hg.num_pins for x in insts]))
        class_results.append({"class": name, "instances": len(insts), "mean_pins": mean_pins, "results": res})
        best = min(res, key=lambda r: r["ms"])
        print(f"{name}: {len(insts)} instances, mean {mean_pins} pins: best {best['variant']} "
              f"{best['ms']:.2f} ms (multi-launch {res[0]['ms']:.2f} ms)", flush=True)
    count_results = []
    for cnt in COUNTS:
        cnt = min(cnt, len(mixed))
        res = time_batch(lp, mixed[:cnt], reps=reps)
        count_results.append({"count": cnt, "results": res})
        best = min(res, key=lambda r: r["ms"])
        print(f"mixed x{cnt}: best {best['variant']} {best['ms']:.2f} ms (multi-launch {res[0]['ms']:.2f} ms)",
              flush=True)
    rows = build_table(class_results, count_results)
    out = {"what": "tuning table of liblpgpu's batched refinement, written by lpgpu.autotune",
           "device": _device_name(), "seconds": round(time.time() - t0, 1),
           "entries": rows, "classes": class_results, "count_sweep": count_results}
    path = args.out or lp.TUNING_PATH
    with open(path, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", path, json.dumps(rows))
    return 0


def _device_name():
    import subprocess
    try:
        return subprocess.run(["nvidia-smi", "--query-gpu=name", "--format=csv,noheader", "-i", "0"],
                              capture_output=True, text=True, timeout=20).stdout.strip()
    except (OSError, subprocess.SubprocessError):
        return "unknown"


if __name__ == "__main__":
    sys.exit(main())

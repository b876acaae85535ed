"""The autotuner's table construction (lpgpu.autotune.build_table) and the
committed GB300 table: rows in increasing size classes, each with the fastest
variant of its class, a size bound between neighbouring classes and the
instance count from which persistent rounds won the count sweep; the library
accepts the committed table."""
import json
import os

import pytest

from conftest import PKG


def _res(ms_multi, ms_px):
    return [{"variant": "multi-launch", "tuning": None, "ms": ms_multi},
            {"variant": "persistent", "tuning": {"mode": 1, "ctas_per_sm": 2, "unroll": 8, "order": 0}, "ms": ms_px}]


def test_build_table_rows():
    from lpgpu import autotune
    classes = [{"class": "a", "mean_pins": 100, "results": _res(5, 2)},
               {"class": "b", "mean_pins": 400, "results": _res(5, 4)},
               {"class": "c", "mean_pins": 1600, "results": _res(3, 9)}]
    counts = [{"count": c, "results": _res(m, p)} for c, m, p in
              [(10, 1, 5), (100, 4, 6), (1000, 20, 10), (5000, 90, 40)]]
    rows = autotune.build_table(classes, counts)
    assert [r["class"] for r in rows] == ["a", "b", "c"]
    assert [r["mode"] for r in rows] == [1, 1, 0]
    assert rows[0]["max_mean_pins"] == 200 and rows[1]["max_mean_pins"] == 800
    assert rows[2]["max_mean_pins"] == 2262  # sqrt(1600 * 3200)
    assert all(r["min_instances"] == 1000 for r in rows)


def test_build_table_without_a_persistent_win():
    from lpgpu import autotune
    classes = [{"class": "a", "mean_pins": 100, "results": _res(1, 2)}]
    counts = [{"count": 10, "results": _res(1, 2)}]
    rows = autotune.build_table(classes, counts)
    assert rows[0]["mode"] == 0 and rows[0]["min_instances"] > 10 ** 8


def test_committed_table_loads(lp):
    path = os.path.join(PKG, "lpgpu", "tuning_gb300.json")
    if not os.path.exists(path):
        pytest.skip("no committed table")
    d = json.load(open(path))
    rows = d["entries"]
    assert rows and all(a["max_mean_pins"] < b["max_mean_pins"] for a, b in zip(rows, rows[1:]))
    lp.load_tuning(path)
    with pytest.raises(lp.LpgpuError):
        lp.set_tuning_table([dict(rows[0], unroll=3)])
    lp.load_tuning(path)

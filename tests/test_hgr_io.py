"""hMetis file reading and partition files (host code of liblpgpu; no GPU)."""
import os

import numpy as np
import pytest

from conftest import load_golden

GOLDEN = ["twocenters", "contracted_unweighted_ibm01", "contracted_ibm01",
          "hypergraph_with_node_and_edge_weights", "karate_club.graph", "test_instance", "powersim.mtx"]


def write_hgr(path, hg, typ, extra_single=()):
    """Writes hg in hMetis format with type `typ`; `extra_single` adds single-pin
    net lines (dropped by the reader) at the given net positions."""
    ew, vw = typ in (1, 11), typ in (10, 11)
    lines = ["% written by the test", f"{hg.m + len(extra_single)} {hg.n}" + (f" {typ}" if typ else "")]
    for e in range(hg.m):
        if e in extra_single:
            lines.append(("7 " if ew else "") + "1")
            lines.append("% a comment between nets")
        pins = [str(p + 1) for p in hg.pins[hg.net_off[e]:hg.net_off[e + 1]]]
        lines.append(" ".join(([str(hg.w_e[e])] if ew else []) + pins))
    if vw:
        lines += [str(w) for w in hg.w_v]
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


@pytest.mark.parametrize("name", GOLDEN)
@pytest.mark.parametrize("typ", [0, 1, 10, 11])
def test_round_trip_of_golden_hypergraphs(lp, tmp_path, name, typ):
    hg, _ = load_golden(name)
    path = str(tmp_path / "h.hgr")
    write_hgr(path, hg, typ, extra_single={0, hg.m // 2})
    got, removed = lp.read_hgr(path)
    assert removed == 2
    assert (got.n, got.m) == (hg.n, hg.m)
    assert np.array_equal(got.net_off, hg.net_off) and np.array_equal(got.pins, hg.pins)
    assert np.array_equal(got.w_e, hg.w_e if typ in (1, 11) else np.ones(hg.m, np.int32))
    assert np.array_equal(got.w_v, hg.w_v if typ in (10, 11) else np.ones(hg.n, np.int32))


def test_reference_instances_match_fixtures(lp):
    """The reader gives the fixtures' CSR for the reference's own test instances
    (when MTK_REFERENCE_ROOT names a Mt-KaHyPar source tree)."""
    root = os.environ.get("MTK_REFERENCE_ROOT")
    inst = os.path.join(root, "tests", "instances") if root else None
    if not inst or not os.path.isdir(inst):
        pytest.skip("MTK_REFERENCE_ROOT does not name a tree with tests/instances")
    for name in GOLDEN:
        hg, _ = load_golden(name)
        got, _ = lp.read_hgr(os.path.join(inst, name + ".hgr"))
        assert np.array_equal(got.net_off, hg.net_off) and np.array_equal(got.pins, hg.pins), name
        assert np.array_equal(got.w_e, hg.w_e) and np.array_equal(got.w_v, hg.w_v), name


@pytest.mark.parametrize("text,why", [
    ("", "missing header"),
    ("2 3\n1 2\n", "expected 2 net lines"),
    ("1 3\n1 4\n", "outside"),
    ("1 3\n0 2\n", "outside"),
    ("1 3 5\n1 2\n", "type"),
    ("1 3\n1 x\n", "unsigned"),
    ("1 3 10\n1 2\n1\n1\n", "vertex weights"),
])
def test_malformed_files_are_rejected(lp, tmp_path, text, why):
    path = tmp_path / "bad.hgr"
    path.write_text(text)
    with pytest.raises(lp.LpgpuError) as e:
        lp.read_hgr(str(path))
    assert e.value.status == lp.ERR_INVALID_ARG
    assert why in str(e.value)


def test_missing_file(lp, tmp_path):
    with pytest.raises(lp.LpgpuError):
        lp.read_hgr(str(tmp_path / "nope.hgr"))


def test_partition_files(lp, tmp_path):
    part = np.random.default_rng(3).integers(0, 17, size=1000).astype(np.int32)
    path = str(tmp_path / "p.part")
    lp.write_partition(path, part)
    assert open(path).read().split("\n")[:3] == [str(x) for x in part[:3]]
    assert np.array_equal(lp.read_partition(path, 1000), part)
    with pytest.raises(lp.LpgpuError):
        lp.read_partition(path, 1001)

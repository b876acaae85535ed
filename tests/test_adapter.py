"""The IRefiner adapter (mt-kahypar_gb300/adapter/gpu_label_propagation_refiner.h)
compiled against the stand-in Mt-KaHyPar headers and linked with liblpgpu.

CPU: it compiles and links; the write-back of a device partition into the
PartitionedHypergraph (changeNodePart with retries, else a rebuild) keeps pin
counts, block weights and the km1 delta exact; without a GPU it fails loudly
instead of falling back. GPU: the driver program refines an hMetis instance
through IRefiner::initialize / refine and ends with the partition and km1 of
a direct session refine and of the oracle."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT, load_golden

ADAPTER = os.path.join(ROOT, "mt-kahypar_gb300", "adapter")


@pytest.fixture(scope="module")
def driver(lp, tmp_path_factory):
    if not shutil.which("g++"):
        pytest.skip("g++ not found")
    exe = tmp_path_factory.mktemp("adapter") / "refine_hgr"
    libdir = os.path.dirname(lp.LIB_PATH)
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(ADAPTER, "shim"), "-I", ADAPTER, "-I", os.path.join(ROOT, "include"),
                        os.path.join(ADAPTER, "refine_hgr.cpp"), "-L", libdir, "-llpgpu",
                        "-Wl,-rpath," + libdir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return str(exe)


def write_hgr(path, hg):
    """hMetis file with net and vertex weights (type 11), 1-based pins."""
    with open(path, "w") as f:
        f.write(f"{hg.m} {hg.n} 11\n")
        for e in range(hg.m):
            pins = hg.pins[hg.net_off[e]:hg.net_off[e + 1]] + 1
            f.write(" ".join(map(str, [int(hg.w_e[e])] + pins.tolist())) + "\n")
        for v in range(hg.n):
            f.write(f"{int(hg.w_v[v])}\n")


def test_writeback_keeps_state_exact(driver):
    r = subprocess.run([driver, "--writeback-selftest"], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "selftest ok" in r.stdout


def test_fails_loudly_without_a_device(driver, tmp_path):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    hg, _ = load_golden("twocenters")
    write_hgr(tmp_path / "g.hgr", hg)
    (tmp_path / "p").write_text("\n".join(str(v % 2) for v in range(hg.n)) + "\n")
    r = subprocess.run([driver, str(tmp_path / "g.hgr"), "2", "0.03", "3", str(tmp_path / "p"),
                        str(tmp_path / "out")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 2 and "refiner error" in r.stderr
    assert not (tmp_path / "out").exists()


@pytest.mark.gpu
@pytest.mark.parametrize("name,k", [("contracted_ibm01", 8), ("powersim.mtx", 4), ("test_instance", 3)])
def test_adapter_refine_equals_session_and_oracle(lp, orc, driver, tmp_path, name, k):
    from lpgpu import gen
    hg, _ = load_golden(name)
    part = gen.random_balanced_partition(hg.n, k, np.random.default_rng([k, 5]))
    write_hgr(tmp_path / "g.hgr", hg)
    np.savetxt(tmp_path / "p", part, fmt="%d")
    r = subprocess.run([driver, str(tmp_path / "g.hgr"), str(k), "0.03", "5", str(tmp_path / "p"),
                        str(tmp_path / "out")], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    out = np.loadtxt(tmp_path / "out", dtype=np.int32)
    fields = r.stdout.split()
    vals = dict(zip(fields[0::2], fields[1::2]))
    perfect, lmax = gen.part_weights(int(hg.w_v.sum()), k, 0.03)
    cfg = lp.default_config(rounds=5)  # the preset: threshold 100, rebalancing, 7 sub-rounds
    with lp.Session(0) as s:
        s.upload(hg)
        s.set_partition(k, part, lmax=lmax, perfect=perfect)
        res = s.refine(cfg)
        direct = s.partition()
    assert np.array_equal(out, direct)
    assert int(vals["km1_before"]) == res.km1_before and int(vals["km1_after"]) == res.km1_after
    assert int(vals["reported"]) == res.km1_after and int(vals["improved"]) == int(res.km1_after < res.km1_before)
    ref, _ = orc.lp_sync(hg, k, lmax, part, perfect=perfect, rounds=5, subrounds=7, revert=1, rollback=1,
                         zero_gain=1)
    assert np.array_equal(out, ref)

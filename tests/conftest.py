import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "mt-kahypar_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build_oracle()
    return oracle


@pytest.fixture(scope="session")
def lp():
    """The product library, built in-tree; GPU tests fail loudly if it is missing."""
    import lpgpu
    lpgpu.build()
    lpgpu.lib()
    return lpgpu


def load_golden(name):
    from lpgpu import gen
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    hg = gen.Hypergraph(int(d["n"]), int(d["m"]), d["net_off"], d["pins"], d["w_v"], d["w_e"]).with_incidence()
    return hg, d


def seven_vertex_fixture():
    """The 7-vertex / 4-net hypergraph of the reference's data-structure tests
    {0,2},{0,1,3,4},{3,4,6},{2,5,6} (partitioned_hypergraph_test.cc:58-61,
    gain_policy_test.cc:37-38)."""
    from lpgpu import gen
    nets = [[0, 2], [0, 1, 3, 4], [3, 4, 6], [2, 5, 6]]
    off = np.zeros(len(nets) + 1, np.int64)
    off[1:] = np.cumsum([len(e) for e in nets])
    pins = np.array([p for e in nets for p in e], np.int32)
    return gen.Hypergraph(7, 4, off, pins, np.ones(7, np.int32), np.ones(4, np.int32)).with_incidence()

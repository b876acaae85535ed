"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/lp_oracle.cpp`` into ``oracle/_build/liblp_oracle.so`` with the
host C++ compiler. The reference implementation itself is not built: its
label-propagation sources need TBB's legacy task API, hwloc, Boost and an
un-vendored submodule, none of which exist on either machine.
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
SO = os.path.join(OUT_DIR, "liblp_oracle.so")


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "lp_oracle.cpp")
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(SO) and os.path.getmtime(SO) >= os.path.getmtime(src):
        return SO
    tmp = SO + ".tmp"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread",
                           src, "-o", tmp])
    os.replace(tmp, SO)
    return SO


if __name__ == "__main__":
    print(build_oracle(force=True))

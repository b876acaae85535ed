"""Build recipe of liblpgpu.so (sm_103a only, no CMake).

Every ``csrc/*.cu`` translation unit is compiled in parallel with
``nvcc -gencode arch=compute_103a,code=sm_103a`` and linked into
``lpgpu/liblpgpu.so`` (CUDA runtime linked statically). Objects go to
``_build/``; both are git-ignored and rebuilt on each machine.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "lpgpu", "liblpgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "-I" + INCLUDE, "-I" + CSRC]
# LPGPU_SPLIT_COMPILE=1 optimizes a file's functions in parallel: a faster
# build, but the sub-round kernels measured about 8 % slower, so it is off
if os.environ.get("LPGPU_SPLIT_COMPILE", "0") == "1":
    NVCC_FLAGS += ["--split-compile", "0"]
# extra nvcc flags, e.g. "-DLPGPU_LV_UNROLL=8" to build a tuning variant
NVCC_FLAGS += os.environ.get("LPGPU_NVCC_EXTRA", "").split()


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    cc = nvcc()
    jobs = []
    objs = []
    for src in srcs:
        obj = os.path.join(BUILD, os.path.splitext(os.path.basename(src))[0] + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([cc] + ARCH + NVCC_FLAGS + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose and r.stderr:
                    print(r.stderr)
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(j), r.stderr))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + ".tmp"
        r = subprocess.run([cc] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"],
                           capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))

"""The C-ABI library builds, loads and exports every entry point declared in
include/*.h; without a GPU the device entry points fail with a status code
instead of falling back to the CPU."""
import ctypes
import glob
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        for m in re.finditer(r"LPGPU_API\s+[\w\s\*]+?\b(lpgpu_\w+)\s*\(", txt):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "lpgpu_refine_km1" in names and "lpgpu_session_refine" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(lp):
    L = lp.lib()
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing
    assert set(declared_symbols()) <= set(lp.SYMBOLS) | set(declared_symbols())


def test_config_defaults_match_preset(lp):
    c = lp.default_config()
    # config/fast_preset.ini:57-61 of the reference
    assert c.rounds == 5 and c.activation_threshold == 100 and c.rebalancing == 1
    assert c.subrounds >= 1


def test_instance_descriptor_layout(lp):
    """The numpy record the binding fills for lpgpu_session_upload_instances has
    the field offsets of the C struct (ctypes mirror), and the pointer arrays
    hold the arrays' addresses (0 for a missing one)."""
    import numpy as np
    dt = lp._INSTANCE_DTYPE
    assert dt.itemsize == ctypes.sizeof(lp.InstanceDesc)
    for name, _ in lp.InstanceDesc._fields_:
        assert dt.fields[name][1] == getattr(lp.InstanceDesc, name).offset, name
    a, b = np.arange(5, dtype=np.int32), np.arange(3, dtype=np.int64)
    ptrs = lp._addresses([a, None, b])
    assert ptrs.dtype == np.uintp and list(ptrs) == [a.ctypes.data, 0, b.ctypes.data]


def test_status_strings(lp):
    L = lp.lib()
    for s in range(8):
        assert L.lpgpu_status_string(s)


def test_footprint_estimate_monotone(lp):
    a = lp.estimate_footprint(1000, 1000, 4000, 2)
    b = lp.estimate_footprint(2000, 2000, 8000, 2)
    c = lp.estimate_footprint(1000, 1000, 4000, 128)
    assert 0 < a < b and a < c


def test_no_device_is_an_error_not_a_fallback(lp):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = ctypes.c_void_p()
    st = lp.lib().lpgpu_session_create(0, ctypes.byref(h))
    assert st == lp.ERR_NO_DEVICE
    with pytest.raises(lp.LpgpuError):
        lp.Session(0)


C_PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "lpgpu.h"
int main(int argc, char** argv) {
  lpgpu_config c;
  lpgpu_config_default(&c);
  if (c.rounds != 5 || c.activation_threshold != 100) return 2;
  int64_t n, m, removed; int64_t* off; int32_t *pins, *vw, *ew;
  if (lpgpu_read_hgr(argv[1], &n, &m, &off, &pins, &vw, &ew, &removed) != LPGPU_OK) {
    fprintf(stderr, "%s\n", lpgpu_last_error());
    return 3;
  }
  printf("%lld %lld %lld %lld %d\n", (long long)n, (long long)m, (long long)off[m], (long long)removed, pins[0]);
  lpgpu_free(off); lpgpu_free(pins); lpgpu_free(vw); lpgpu_free(ew);
  lpgpu_session* s = 0;
  lpgpu_status st = lpgpu_session_create(0, &s);  /* no device here: an error, never a fallback */
  if (st == LPGPU_OK) lpgpu_session_destroy(s);
  printf("%s\n", lpgpu_status_string(st));
  return 0;
}
"""


@pytest.mark.parametrize("compiler,ext", [("gcc", "c"), ("g++", "cpp")])
def test_header_compiles_and_links_from_c_and_cpp(lp, tmp_path, compiler, ext):
    """include/lpgpu.h is plain C and C++: a program built with the host
    compiler links liblpgpu.so and calls it (file reader, no GPU needed)."""
    import shutil
    import subprocess
    if not shutil.which(compiler):
        pytest.skip(compiler + " not found")
    src = tmp_path / f"prog.{ext}"
    src.write_text(C_PROGRAM)
    hgr = tmp_path / "t.hgr"
    hgr.write_text("% tiny\n3 4\n1 2\n3\n2 3 4\n")
    libdir = os.path.dirname(lp.LIB_PATH)
    exe = tmp_path / "prog"
    r = subprocess.run([compiler, str(src), "-I", os.path.join(ROOT, "include"), "-L", libdir, "-llpgpu",
                        "-Wl,-rpath," + libdir, "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(hgr)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    first, second = r.stdout.strip().split("\n")
    assert first == "4 2 5 1 0"
    assert second  # status text of session_create (ok on a GPU machine, an error here)

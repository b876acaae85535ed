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

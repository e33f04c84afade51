"""The C-ABI library loads on a machine without a GPU and exports every entry
point include/xg.h declares (no compute calls)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = []
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names += re.findall(r"\b(?:int|const char\*)\s+(xg_\w+)\s*\(", src)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from ngsxfem_gb300 import build
    build.build()
    return ctypes.CDLL(build.LIB)


def test_header_declares_entry_points():
    names = declared()
    assert "xg_cutinfo_update" in names and "xg_form_assemble" in names and "xg_cutfem_step" in names


def test_exports(lib):
    from ngsxfem_gb300 import _lib
    names = declared()
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert sorted(_lib.EXPORTS) == names


def test_status_strings(lib):
    lib.xg_status_string.restype = ctypes.c_char_p
    assert lib.xg_status_string(0) == b"ok"
    assert b"capacity" in lib.xg_status_string(3)


def test_rule_sizes(lib):
    # rule family: tet order 2 -> 4 points, order 4 -> 14, order 6 -> 64 (conical),
    # trig order 4 -> 6, order 5 -> 7, segment order 4 -> 3
    assert lib.xg_base_rule_size(3, 2) == 4
    assert lib.xg_base_rule_size(3, 4) == 14
    assert lib.xg_base_rule_size(3, 6) == 64
    assert lib.xg_base_rule_size(2, 4) == 6
    assert lib.xg_base_rule_size(2, 5) == 7
    assert lib.xg_base_rule_size(1, 4) == 3


def test_no_device_reports_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a device is present")
    ok = ctypes.c_int(-1)
    assert lib.xg_device_ok(ctypes.byref(ok)) == 8
    assert ok.value == 0


def test_rule_family_matches_oracle(lib):
    """Host rule tables of the product equal the oracle's rule family (built by
    a different algorithm) to the last bit or so."""
    import numpy as np
    from oracle import oracle as orc
    orc.build()
    P = ctypes.c_void_p
    lib.xg_base_rule.argtypes = [ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int]
    for d in (1, 2, 3):
        for p in range(0, 9):
            pts = np.zeros((512, 3))
            w = np.zeros(512)
            n = lib.xg_base_rule(d, p, pts.ctypes.data_as(P), w.ctypes.data_as(P), 512)
            rp, rw = orc.base_rule(d, p)
            assert n == len(rw)
            assert np.max(np.abs(pts[:n] - rp)) <= 4e-16, (d, p)
            assert np.max(np.abs(w[:n] - rw)) <= 4e-16, (d, p)

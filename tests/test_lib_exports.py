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
            names += re.findall(r"\b(?:int|int64_t|const char\*)\s+(xg_\w+)\s*\(", src)
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


def declared_arity():
    """Number of parameters of every xg_* function the headers declare."""
    out = {}
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(?:int|const char\*)\s+(xg_\w+)\s*\(([^)]*)\)\s*;", src, flags=re.S):
            params = m.group(2).strip()
            out[m.group(1)] = 0 if params in ("", "void") else params.count(",") + 1
    return out


def test_ctypes_signatures_match_the_header():
    """The ctypes argument lists in ngsxfem_gb300/_lib.py have the arity the
    header declares (a mismatch would only show on a GPU)."""
    from ngsxfem_gb300 import _lib
    arity = declared_arity()
    sigs = _lib.SIGNATURES if hasattr(_lib, "SIGNATURES") else None
    if sigs is None:
        L = _lib.load()
        sigs = {n: (None, getattr(L, n).argtypes) for n in _lib.EXPORTS}
    bad = [(n, len(a), arity[n]) for n, (_, a) in sigs.items() if a is not None and n in arity and len(a) != arity[n]]
    assert not bad, bad


def test_call_sites_pass_the_declared_number_of_arguments():
    """Every _lib.call("xg_...", ...) in the package, bench.py and the smoke
    check passes as many arguments as the entry point takes."""
    import ast
    arity = declared_arity()
    files = [os.path.join(ROOT, "ngsxfem_gb300", f) for f in os.listdir(os.path.join(ROOT, "ngsxfem_gb300"))
             if f.endswith(".py")] + [os.path.join(ROOT, "bench.py"), os.path.join(ROOT, "__graft_entry__.py")]
    checked, bad = 0, []
    for path in files:
        for node in ast.walk(ast.parse(open(path).read())):
            if not (isinstance(node, ast.Call) and isinstance(node.func, ast.Attribute) and node.func.attr == "call"):
                continue
            if not node.args or not isinstance(node.args[0], ast.Constant) or not isinstance(node.args[0].value, str):
                continue
            name = node.args[0].value
            if name not in arity or any(isinstance(a, ast.Starred) for a in node.args):
                continue
            checked += 1
            if len(node.args) - 1 != arity[name]:
                bad.append((os.path.basename(path), node.lineno, name, len(node.args) - 1, arity[name]))
    assert checked > 40
    assert not bad, bad

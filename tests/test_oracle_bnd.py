"""Boundary cut integrals dCut(lset, dt, vb=BND): the oracle
(orc_integrate_bnd, oracle/xg_oracle_mlset.cpp) against the closed forms of
ngsxfem's tests/pytests/test_bndcut.py, and the product's boundary rule
(csrc/xg_mlset.cuh ml::bnd_rule) against the oracle per element (host build,
tests/native/mlset_rule_check.cu, run by test_oracle_mlset.py).  CPU only."""
import json
import os

import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))


def test_boundary_measures_2d(orc):
    ref = KA["bnd2d"]
    m = MakeStructured2DMesh(9, 9)
    for cut in ref["cuts"]:
        l = orc.interpolate_p1_perturb(m.coords[:, 0] - cut)
        neg, st = orc.integrate_bnd(m, l, orc.NEG, 2)
        pos, _ = orc.integrate_bnd(m, l, orc.POS, 2)
        npts, _ = orc.integrate_bnd(m, l, orc.IF, 0)
        assert st == 0
        assert abs(neg - (2 * cut + 1)) < ref["tol"]
        assert abs(neg + pos - ref["perimeter"]) < ref["tol"]
        assert abs(npts - ref["IF_points"]) < ref["tol"]
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - 0.5)
    assert abs(orc.integrate_bnd(m, l, orc.IF, 0, (1, 0, 0))[0] - ref["if_x_at_half"]) < ref["tol"]
    assert abs(orc.integrate_bnd(m, l, orc.IF, 0, (0, 1, 0))[0] - ref["if_y_at_half"]) < ref["tol"]


def test_boundary_measures_3d(orc):
    ref = KA["bnd3d"]
    m = MakeStructured3DMesh(7)
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - ref["cut"])
    neg, st = orc.integrate_bnd(m, l, orc.NEG, 2)
    assert st == 0 and abs(neg - ref["NEG"]) < ref["tol"]
    # the interface on boundary triangles (codimension 2) is not supported
    assert orc.integrate_bnd(m, l, orc.IF, 2)[1] == 6


def test_boundary_regions_2d(orc):
    """definedon=mesh.Boundaries(side): the oracle restricted to the BND
    elements of one side of the square (test_bndcut.py:51-59, 203-217)."""
    ref = KA["bnd2d_definedon"]
    m = MakeStructured2DMesh(9, 9)
    bottom, left = m.Boundaries("bottom").Mask(), m.Boundaries("left").Mask()
    assert bottom.sum() == 9 and left.sum() == 9 and m.Boundaries("bottom|top|left|right").Mask().all()
    for cut in ref["cuts"]:
        l = orc.interpolate_p1_perturb(m.coords[:, 0] - cut)
        assert abs(orc.integrate_bnd(m, l, orc.NEG, 2, defined_on=bottom)[0] - cut) < ref["tol"]
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - 0.5)
    assert abs(orc.integrate_bnd(m, l, orc.IF, 0, defined_on=bottom)[0] - ref["bottom_IF_at_half"]) < ref["tol"]
    assert abs(orc.integrate_bnd(m, l, orc.IF, 0, defined_on=left)[0] - ref["left_IF_at_half"]) < ref["tol"]
    # an all-true mask equals no restriction; the sides add up to the whole boundary
    full = orc.integrate_bnd(m, l, orc.NEG, 2)[0]
    assert orc.integrate_bnd(m, l, orc.NEG, 2, defined_on=np.ones(len(bottom), bool))[0] == full
    sides = sum(orc.integrate_bnd(m, l, orc.NEG, 2, defined_on=m.Boundaries(s).Mask())[0]
                for s in ("bottom", "right", "top", "left"))
    assert abs(sides - full) < 1e-14


def test_boundary_elements_order():
    """Mesh.boundary_elements: the facets of one element, vertices ascending,
    lexicographic (the BND element order of libxg and of the oracle)."""
    m = MakeStructured3DMesh(3)
    b = m.boundary_elements()
    assert len(b) == 6 * 2 * 3 * 3 and (np.diff(b, axis=1) > 0).all()
    keys = [tuple(r) for r in b]
    assert keys == sorted(keys)
    sides = ["left", "right", "front", "back", "bottom", "top"]
    masks = np.array([m.Boundaries(s).Mask() for s in sides])
    assert (masks.sum(axis=0) == 1).all() and (masks.sum(axis=1) == 18).all()
    x = m.coords[b]
    assert np.all(x[masks[2]][..., 1] == 0.0) and np.all(x[masks[5]][..., 2] == 1.0)


def bnd_bits(mask):
    """A boolean mask over the BND elements as the oracle's uint64 bit words."""
    b = np.packbits(np.asarray(mask, bool), bitorder="little")
    return np.concatenate([b, np.zeros((-b.size) % 8, np.uint8)]).view(np.uint64)


def test_boundary_linear_form(orc):
    """v * dCut(lset, dt, vb=BND) (the reference's boundary linear forms,
    test_bndcut.py:123-165): with c1 / cx the coefficients of the functions
    1 and x (vertex dofs 1 / x, the others 0), b.c1 is the measure of the
    domain part of the boundary and b.cx the integral of x over it."""
    m = MakeStructured2DMesh(9, 9)
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - 0.4)
    bottom = bnd_bits(m.Boundaries("bottom").Mask())
    for k in (1, 2, 3):
        sp = orc.Space(m, k)
        b = sp.linear_form(l, [dict(kind=2, domain=orc.NEG)])
        c1, cx = np.zeros(len(b)), np.zeros(len(b))
        c1[:m.nv], cx[:m.nv] = 1.0, m.coords[:, 0]
        assert abs(b @ c1 - 1.8) < 1e-13 and abs(b @ cx - 0.16) < 1e-13
        if k == 1:
            assert abs(b.sum() - 1.8) < 1e-13  # partition of unity
        bb = sp.linear_form(l, [dict(kind=2, domain=orc.NEG, defined_on=bottom)])
        assert abs(bb @ c1 - 0.4) < 1e-13
        bi = sp.linear_form(l, [dict(kind=2, domain=orc.IF, order=0, e=(0, 1, 0))])
        assert abs(bi @ c1 - 1.0) < 1e-13  # y at the interface points (0.4, 0) and (0.4, 1)
        # volume and boundary terms add
        bv = sp.linear_form(l, [dict(kind=0, domain=orc.NEG)])
        both = sp.linear_form(l, [dict(kind=0, domain=orc.NEG), dict(kind=2, domain=orc.NEG)])
        assert np.allclose(both, bv + b, rtol=0, atol=1e-15)
    m3 = MakeStructured3DMesh(4)
    l3 = orc.interpolate_p1_perturb(m3.coords[:, 0] - 0.3)
    sp = orc.Space(m3, 2)
    b = sp.linear_form(l3, [dict(kind=2, domain=orc.NEG)])
    c1 = np.zeros(len(b))
    c1[:m3.nv] = 1.0
    assert abs(b @ c1 - 2.2) < 1e-13
    with pytest.raises(RuntimeError):
        sp.linear_form(l3, [dict(kind=2, domain=orc.IF)])


def owners(m):
    """The element each BND element (Mesh.boundary_elements order) belongs to."""
    own = {}
    d = m.dim
    for e, el in enumerate(m.elements):
        for s in range(d + 1):
            own[tuple(sorted(np.delete(el, s)))] = e
    return np.array([own[tuple(r)] for r in m.boundary_elements()], dtype=np.int64)


def test_boundary_linear_form_device_code(orc, tmp_path):
    """csrc/xg_lfbnd.cuh (the body of the GPU kernel k_lf_bnd) compiled as
    host code (tests/native/lf_bnd_check.cu): its element vectors, gathered
    with the oracle space's dofs, equal orc_linear_form within 1e-13."""
    import ctypes
    import shutil
    import subprocess

    from ngsxfem_gb300 import _lib
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    root = os.path.dirname(HERE)
    libdir = os.path.dirname(orc.LIB)
    so = str(tmp_path / "liblfb.so")
    subprocess.check_call([nvcc, "-x", "cu", "-std=c++17", "-O1", "-shared", "-Xcompiler", "-fPIC", "-Xcompiler",
                           "-ffp-contract=off", "-diag-suppress", "20011,20014",
                           "-I", os.path.join(root, "ngsxfem_gb300", "csrc"), "-I", os.path.join(root, "include"),
                           os.path.join(HERE, "native", "lf_bnd_check.cu"), "-L", libdir, "-loracle",
                           "-Xlinker", "-rpath", "-Xlinker", libdir, "-o", so])
    L = ctypes.CDLL(so)
    P = ctypes.c_void_p
    L.lfb_element_vectors.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int64, P, P, P, P, P, ctypes.c_int, P]
    p = lambda a: a.ctypes.data_as(P)  # noqa: E731
    cases = [(MakeStructured2DMesh(9, 7), lambda c: c[:, 0] - 0.4 + 0.1 * c[:, 1], (1, 2, 3)),
             (MakeStructured3DMesh(3), lambda c: c[:, 0] - 0.3 + 0.2 * c[:, 2], (1, 2, 3))]
    worst = 0.0
    for m, f, ks in cases:
        D = m.dim
        l = orc.interpolate_p1_perturb(f(m.coords))
        bnd, own = m.boundary_elements(), owners(m)
        nb = len(bnd)
        xv = np.zeros((nb, D + 1, 3))
        xv[..., :D] = m.coords[m.elements[own]]
        gv = np.ascontiguousarray(m.elements[own], dtype=np.int32)
        xb = np.zeros((nb, D, 3))
        xb[..., :D] = m.coords[bnd]
        lb = np.ascontiguousarray(l[bnd])
        bottom = m.Boundaries("bottom").Mask()
        term_sets = [[dict(kind=2, domain=orc.NEG)],
                     [dict(kind=2, domain=orc.POS, e=(1, 0, 1), coef=-1.5, defined_on=bottom, order=3)],
                     [dict(kind=2, domain=orc.NEG, e=(0, 2, 0)), dict(kind=2, domain=orc.POS, order=1)]]
        if D == 2:
            term_sets.append([dict(kind=2, domain=orc.IF, order=0, e=(0, 1, 0), coef=2.0)])
        for k in ks:
            sp = orc.Space(m, k)
            dofs = sp.el_dofs()
            for terms in term_sets:
                arr = (_lib.LTerm * len(terms))()
                keep = []
                for i, t in enumerate(terms):
                    arr[i].kind, arr[i].domain, arr[i].order = 2, t["domain"], t.get("order", -1)
                    arr[i].coef = t.get("coef", 1.0)
                    for j in range(3):
                        arr[i].e[j] = t.get("e", (0, 0, 0))[j]
                    if t.get("defined_on") is not None:
                        bits = bnd_bits(t["defined_on"])
                        keep.append(bits)
                        arr[i].d_defined_on = bits.ctypes.data
                n = dofs.shape[1]
                vec = np.zeros((nb, n))
                st = L.lfb_element_vectors(D, k, nb, p(xv), p(gv), p(xb), p(lb), ctypes.cast(arr, P), len(terms),
                                           p(vec))
                assert st == 0
                got = np.zeros(sp.ndof)
                np.add.at(got, dofs[own], vec)
                oterms = [dict(t, kind=2, defined_on=None if t.get("defined_on") is None else
                               bnd_bits(t["defined_on"])) for t in terms]
                ref = sp.linear_form(l, oterms)
                err = np.max(np.abs(got - ref)) / max(1.0, np.max(np.abs(ref)))
                worst = max(worst, err)
                assert err < 1e-13, (D, k, terms, err)
    assert worst < 1e-13

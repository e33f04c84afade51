"""Boundary cut integrals on the GPU (xg_integrate_bnd, Integrate(f *
dCut(lset, dt, vb=BND), mesh)) against the oracle and the closed forms of
ngsxfem's tests/pytests/test_bndcut.py.  Bar: 1e-12 relative to the oracle."""
import json
import os

import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))


def gf_of(xg, m, vals):
    g = xg.GridFunction(xg.H1(m, order=1))
    g.vec.copy_(torch.from_numpy(np.ascontiguousarray(vals)))
    return g


def test_boundary_integrals(xg, orc):
    ref = KA["bnd2d"]
    m = MakeStructured2DMesh(9, 9)
    for cut in ref["cuts"]:
        l = orc.interpolate_p1_perturb(m.coords[:, 0] - cut)
        g = gf_of(xg, m, l)
        neg = xg.Integrate(xg.dCut(g, xg.NEG, vb=xg.BND, order=2), m)
        assert abs(neg - (2 * cut + 1)) < ref["tol"]
        assert abs(xg.Integrate(xg.dCut(g, xg.IF, vb=xg.BND, order=0), m) - ref["IF_points"]) < ref["tol"]
        for dt in (xg.NEG, xg.POS, xg.IF):
            for e in ((0, 0, 0), (1, 0, 0), (0, 2, 0)):
                r, st = orc.integrate_bnd(m, l, dt, 2, e)
                cf = xg.x ** e[0] * xg.y ** e[1]
                got = xg.Integrate(cf * xg.dCut(g, dt, vb=xg.BND, order=2), m)
                assert st == 0 and abs(got - r) <= 1e-12 * max(1.0, abs(r)), (cut, dt, e, got, r)
    m3 = MakeStructured3DMesh(7)
    l3 = orc.interpolate_p1_perturb(m3.coords[:, 0] - KA["bnd3d"]["cut"])
    g3 = gf_of(xg, m3, l3)
    assert abs(xg.Integrate(xg.dCut(g3, xg.NEG, vb=xg.BND, order=2), m3) - KA["bnd3d"]["NEG"]) < KA["bnd3d"]["tol"]
    with pytest.raises(RuntimeError):
        xg.Integrate(xg.dCut(g3, xg.IF, vb=xg.BND, order=2), m3)


def test_boundary_element_order(xg):
    """The device's BND elements (xg_mesh_boundary facet numbers into the
    lexicographic facet list) are Mesh.boundary_elements, row for row."""
    import ctypes

    from ngsxfem_gb300 import _lib
    for m in (MakeStructured2DMesh(5, 4), MakeStructured3DMesh(3)):
        dm = xg.device_mesh(m)
        nb = np.zeros(1, dtype=np.int64)
        _lib.call("xg_mesh_boundary", dm.h, nb.ctypes.data_as(ctypes.c_void_p), None)
        fac = np.zeros(int(nb[0]), dtype=np.int32)
        _lib.call("xg_mesh_boundary", dm.h, nb.ctypes.data_as(ctypes.c_void_p), fac.ctypes.data_as(ctypes.c_void_p))
        d = m.dim
        allf = np.unique(np.sort(np.concatenate([np.delete(m.elements, s, axis=1) for s in range(d + 1)]), axis=1),
                         axis=0)
        assert np.array_equal(allf[fac], m.boundary_elements())


def test_boundary_regions(xg, orc):
    """definedon=mesh.Boundaries(side) and definedonelements (a BND BitArray)
    against the oracle with the same mask and the closed forms of
    test_bndcut.py:51-59, 203-217."""
    ref = KA["bnd2d_definedon"]
    m = MakeStructured2DMesh(9, 9)
    for cut in ref["cuts"]:
        l = orc.interpolate_p1_perturb(m.coords[:, 0] - cut)
        g = gf_of(xg, m, l)
        bottom = m.Boundaries("bottom")
        got = xg.Integrate(xg.dCut(g, xg.NEG, vb=xg.BND, order=2, definedon=bottom), m)
        assert abs(got - cut) < ref["tol"]
        for side in ("bottom", "right|top", "left"):
            mask = m.Boundaries(side).Mask()
            for dt, e in ((xg.NEG, (1, 0, 0)), (xg.POS, (0, 1, 0)), (xg.IF, (0, 0, 0))):
                r, st = orc.integrate_bnd(m, l, dt, 2, e, defined_on=mask)
                cf = xg.x ** e[0] * xg.y ** e[1]
                got = xg.Integrate(cf * xg.dCut(g, dt, vb=xg.BND, order=2, definedon=m.Boundaries(side)), m)
                assert st == 0 and abs(got - r) <= 1e-12 * max(1.0, abs(r)), (cut, side, dt, got, r)
        # definedonelements: CutInfo's BND HASNEG elements give the unrestricted NEG part
        ci = xg.CutInfo(m, g)
        hasneg = ci.GetElementsOfType(xg.HASNEG, xg.BND)
        full = xg.Integrate(xg.dCut(g, xg.NEG, vb=xg.BND, order=2), m)
        part = xg.Integrate(xg.dCut(g, xg.NEG, vb=xg.BND, order=2, definedonelements=hasneg), m)
        assert abs(part - full) < 1e-14
        both = xg.Integrate(xg.dCut(g, xg.NEG, vb=xg.BND, order=2, definedonelements=hasneg, definedon=bottom), m)
        assert abs(both - cut) < ref["tol"]
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - 0.5)
    g = gf_of(xg, m, l)
    for side, key in (("bottom", "bottom_IF_at_half"), ("left", "left_IF_at_half")):
        got = xg.Integrate(xg.dCut(g, xg.IF, vb=xg.BND, order=0, definedon=m.Boundaries(side)), m)
        assert abs(got - ref[key]) < ref["tol"]
    with pytest.raises(ValueError):
        xg.Integrate(xg.dCut(g, xg.NEG, vb=xg.BND, definedonelements=xg.BitArray(m.ne)), m)


def bnd_bits(mask):
    b = np.packbits(np.asarray(mask, bool), bitorder="little")
    return np.concatenate([b, np.zeros((-b.size) % 8, np.uint8)]).view(np.uint64)


def test_boundary_linear_form(xg, orc):
    """LinearForm with v * dCut(lset, dt, vb=BND[, definedon]) against the
    oracle's vector (1e-12 relative to its largest entry) and the closed
    forms of test_bndcut.py:123-165."""
    m = MakeStructured2DMesh(9, 9)
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - 0.4)
    g = gf_of(xg, m, l)
    bottom = m.Boundaries("bottom")
    for k in (1, 2, 3):
        V = xg.H1(m, order=k)
        v = V.TestFunction()
        sp = orc.Space(m, k)
        cases = [
            (v * xg.dCut(g, xg.NEG, vb=xg.BND), [dict(kind=2, domain=orc.NEG)]),
            (xg.x * v * xg.dCut(g, xg.POS, vb=xg.BND, definedon=bottom),
             [dict(kind=2, domain=orc.POS, e=(1, 0, 0), defined_on=bnd_bits(bottom.Mask()))]),
            (2.0 * xg.y * v * xg.dCut(g, xg.IF, vb=xg.BND, order=0),
             [dict(kind=2, domain=orc.IF, order=0, e=(0, 1, 0), coef=2.0)]),
            (v * xg.dCut(g, xg.NEG) + v * xg.dCut(g, xg.NEG, vb=xg.BND),
             [dict(kind=0, domain=orc.NEG), dict(kind=2, domain=orc.NEG)]),
        ]
        for integral, terms in cases:
            f = xg.LinearForm(V)
            f += integral
            f.Assemble()
            got = f.vec.cpu().numpy()
            ref = sp.linear_form(l, terms)
            assert np.max(np.abs(got - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref))), (k, terms)
        f = xg.LinearForm(V)
        f += v * xg.dCut(g, xg.NEG, vb=xg.BND, definedon=bottom)
        f.Assemble()
        c1 = np.zeros(V.ndof)
        c1[:m.nv] = 1.0
        assert abs(f.vec.cpu().numpy() @ c1 - 0.4) < 1e-12
    m3 = MakeStructured3DMesh(4)
    g3 = gf_of(xg, m3, orc.interpolate_p1_perturb(m3.coords[:, 0] - 0.3))
    V3 = xg.H1(m3, order=2)
    f = xg.LinearForm(V3)
    f += V3.TestFunction() * xg.dCut(g3, xg.IF, vb=xg.BND)
    with pytest.raises(RuntimeError):
        f.Assemble()


@pytest.mark.gpu
def test_boundary_linear_form_3d(xg, orc):
    """Boundary terms on tetrahedral meshes: NEG and POS traces of P1-P3 test
    functions on the boundary triangles (the owner's basis at the physical
    points of the boundary rule), with and without definedon=bottom, against
    the oracle's vector within 1e-12 of its largest entry."""
    m = MakeStructured3DMesh(4)
    c = m.coords
    l = orc.interpolate_p1_perturb(c[:, 0] + 0.5 * c[:, 1] - 0.3 * c[:, 2] - 0.45)
    g = gf_of(xg, m, l)
    bottom = m.Boundaries("bottom")
    for k in (1, 2, 3):
        V = xg.H1(m, order=k)
        v = V.TestFunction()
        sp = orc.Space(m, k)
        for dt in (xg.NEG, xg.POS):
            cases = [
                (v * xg.dCut(g, dt, vb=xg.BND), [dict(kind=2, domain=dt)]),
                (xg.y * v * xg.dCut(g, dt, vb=xg.BND, definedon=bottom),
                 [dict(kind=2, domain=dt, e=(0, 1, 0), defined_on=bnd_bits(bottom.Mask()))]),
                (xg.z * v * xg.dCut(g, dt, vb=xg.BND),
                 [dict(kind=2, domain=dt, e=(0, 0, 1))]),
            ]
            for integral, terms in cases:
                f = xg.LinearForm(V)
                f += integral
                f.Assemble()
                got = f.vec.cpu().numpy()
                ref = sp.linear_form(l, terms)
                assert np.max(np.abs(ref)) > 0
                assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref)), (k, dt, terms)

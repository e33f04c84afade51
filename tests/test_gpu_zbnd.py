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

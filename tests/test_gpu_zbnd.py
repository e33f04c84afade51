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

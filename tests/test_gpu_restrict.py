"""The dof restrictions of the reference's fictdom demos on the GPU:
GetDofsOfElements (the dofs of the HASNEG elements), Restrict(V, hasneg)
.FreeDofs(), Compress, RestrictedBilinearForm (the same matrix as the
BilinearForm: every pattern is already that of the active elements and
facets), and the assembled matrix's rows lie in the free dofs."""
import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("D,k", [(2, 2), (3, 1), (3, 3)])
def test_restricted_fictdom_form(xg, orc, D, k):
    m = MakeStructured2DMesh(10, 10) if D == 2 else MakeStructured3DMesh(4)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.45) ** 2).sum(axis=1) - 0.3 ** 2)
    g = xg.GridFunction(xg.H1(m, order=1))
    xg.InterpolateToP1(l, g)
    ci = xg.CutInfo(m, g)
    hasneg, ifb = ci.GetElementsOfType(xg.HASNEG), ci.GetElementsOfType(xg.IF)
    gp = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=ifb, use_and=True)
    Vbase = xg.H1(m, order=k)
    free = xg.GetDofsOfElements(Vbase, hasneg)
    el = Vbase.element_dofs()
    want = np.zeros(Vbase.ndof, dtype=bool)
    want[el[hasneg.numpy()].reshape(-1)] = True
    assert np.array_equal(free.numpy(), want)
    V = xg.Restrict(Vbase, hasneg)
    assert V.ndof == Vbase.ndof and np.array_equal(V.FreeDofs().numpy(), want)
    assert xg.Compress(Vbase, free).FreeDofs() is free
    assert Vbase.FreeDofs().numpy().all()
    u, v = V.TnT()
    h = xg.specialcf.mesh_size
    n = xg.Normalize(xg.grad(g))
    mats = []
    for a in (xg.BilinearForm(Vbase), xg.RestrictedBilinearForm(V, "a", hasneg, gp, check_unused=False)):
        a += xg.grad(u) * xg.grad(v) * xg.dCut(g, xg.NEG, definedonelements=hasneg)
        a += (-xg.grad(u) * n * v - xg.grad(v) * n * u + (10.0 * k * k / h) * u * v) * \
            xg.dCut(g, xg.IF, definedonelements=ifb)
        a += 0.1 / h ** 2 * (u - u.Other()) * (v - v.Other()) * xg.dFacetPatch(definedonelements=gp)
        a.Assemble()
        mats.append(a.mat.global_coo())
    for p, q in zip(*mats):
        assert np.array_equal(p, q)
    rows = np.unique(mats[0][0])
    assert want[rows].all() and len(rows) == want.sum()
    # the view keeps the base space alive and does not free its handle
    del V
    gfu = xg.GridFunction(Vbase)
    assert gfu.vec.numel() == Vbase.ndof and torch.isfinite(gfu.vec).all()

"""The fictitious-domain workflow of the reference's demos end to end: the
bilinear form (stiffness + mass on NEG, ghost penalty) and the linear form
(source on NEG, Neumann data on the interface) assembled on the GPU through
the Python mirror, the system solved on the free dofs of Restrict(V, hasneg)
(scipy, in this test only), and the L2 error measured by Integrate((gfu -
uex) ** 2 * dCut(lset, NEG)) on the GPU.  The problem: -lap u + u = f on
{x + y/2 < 0.6} in the unit square, u = cos(pi x) cos(pi y) (zero normal
derivative on the square's sides, the interface's Neumann data grad u . n);
the planar interface is exact, so the error converges at order k + 1."""
import math

import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh

pytestmark = pytest.mark.gpu

PI = math.pi
NRM = np.array([1.0, 0.5]) / math.sqrt(1.25)


def solve(xg, N, k):
    import scipy.sparse.linalg as sla

    m = MakeStructured2DMesh(N, N)
    g = xg.GridFunction(xg.H1(m, order=1))
    xg.InterpolateToP1(lambda x, y: x + 0.5 * y - 0.6, g)
    ci = xg.CutInfo(m, g)
    hasneg, ifb = ci.GetElementsOfType(xg.HASNEG), ci.GetElementsOfType(xg.IF)
    gp = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=ifb, use_and=True)
    Vb = xg.H1(m, order=k)
    V = xg.Restrict(Vb, hasneg)
    # the data in the form's space (the linear form's GridFunction sources),
    # the exact solution at order 3 for the error
    uex = xg.GridFunction(xg.H1(m, order=3)).Set(lambda x, y: np.cos(PI * x) * np.cos(PI * y))
    f = xg.GridFunction(Vb).Set(lambda x, y: (2 * PI * PI + 1) * np.cos(PI * x) * np.cos(PI * y))
    gn = xg.GridFunction(Vb).Set(lambda x, y: -PI * (np.sin(PI * x) * np.cos(PI * y) * NRM[0] +
                                                     np.cos(PI * x) * np.sin(PI * y) * NRM[1]))
    u, v = V.TnT()
    h = xg.specialcf.mesh_size
    a = xg.RestrictedBilinearForm(V, "a", hasneg, gp, check_unused=False)
    a += (xg.grad(u) * xg.grad(v) + u * v) * xg.dCut(g, xg.NEG, definedonelements=hasneg)
    a += 0.1 / h ** 2 * (u - u.Other()) * (v - v.Other()) * xg.dFacetPatch(definedonelements=gp)
    a.Assemble()
    rhs = xg.LinearForm(V)
    rhs += f * v * xg.dCut(g, xg.NEG, definedonelements=hasneg)
    rhs += gn * v * xg.dCut(g, xg.IF, definedonelements=ifb)
    rhs.Assemble()
    free = np.flatnonzero(V.FreeDofs().numpy())
    A = a.mat.to_scipy()[free][:, free].tocsc()
    b = rhs.vec.cpu().numpy()[free]
    x = np.zeros(V.ndof)
    x[free] = sla.spsolve(A, b)
    gfu = xg.GridFunction(V)
    gfu.vec.copy_(torch.from_numpy(x))
    err = xg.Integrate((gfu - uex) ** 2 * xg.dCut(g, xg.NEG, order=2 * k + 4), m)
    h1 = xg.Integrate((xg.grad(gfu) - xg.grad(uex)) ** 2 * xg.dCut(g, xg.NEG, order=2 * k + 2), m)
    return math.sqrt(err), math.sqrt(h1)


@pytest.mark.parametrize("k", [1, 2])
def test_fictdom_converges(xg, k):
    errs = [solve(xg, N, k) for N in (8, 16, 32)]
    l2 = [e[0] for e in errs]
    h1 = [e[1] for e in errs]
    # the rate over the whole range and on the finest pair (the coarsest
    # mesh, h = 1/8, is preasymptotic for P2)
    eoc_l2 = [math.log2(l2[0] / l2[-1]) / 2, math.log2(l2[-2] / l2[-1])]
    eoc_h1 = [math.log2(h1[0] / h1[-1]) / 2, math.log2(h1[-2] / h1[-1])]
    assert min(eoc_l2) > k + 1 - 0.3, (l2, eoc_l2)
    assert min(eoc_h1) > k - 0.3, (h1, eoc_h1)
    assert l2[-1] < (1e-2 if k == 1 else 1e-3), l2

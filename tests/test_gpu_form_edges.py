"""Edge cases and determinism of the form families built on the generic
kernels (boundary terms, coefficient fields, the deformed mesh, Q1 on
quad/hex meshes): a level set without a zero in the mesh (all NEG: every
element uncut and active; all POS: nothing active, an empty matrix), a
level set with exact zeros at vertices (the +1e-14 perturbation of
InterpolateToP1), and repeated assemblies bit-identical."""
import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


def gf_of(xg, m, vals):
    g = xg.GridFunction(xg.H1(m, order=1))
    g.vec.copy_(torch.from_numpy(np.ascontiguousarray(vals, dtype=np.float64)))
    return g


def assemble_vals(a):
    a.Assemble()
    r, c, v = a.mat.global_coo()
    return r.copy(), c.copy(), v.copy()


def forms(xg, m, g, V, adap=None):
    u, v = V.TnT()
    h = xg.specialcf.mesh_size
    fx = xg.GridFunction(xg.H1(m, order=1)).Set(lambda *x: 1.0 + x[0])
    out = []
    a = xg.BilinearForm(V)
    a += fx * xg.grad(u) * xg.grad(v) * xg.dCut(g, xg.NEG)
    a += (10.0 / h) * u * v * xg.dCut(g, xg.NEG, vb=xg.BND)
    out.append(a)
    if adap is not None:
        b = xg.BilinearForm(V)
        b += xg.grad(u) * xg.grad(v) * xg.dCut(g, xg.NEG, deformation=adap)
        out.append(b)
    return out


@pytest.mark.parametrize("D", [2, 3])
def test_uncut_level_sets(xg, D):
    m = MakeStructured2DMesh(6, 6) if D == 2 else MakeStructured3DMesh(3)
    V = xg.H1(m, order=2)
    one = np.zeros(V.ndof)
    one[: m.nv] = 1.0
    # all NEG: the whole domain; the BND mass is the boundary measure / h
    g = gf_of(xg, m, -np.ones(m.nv))
    a = forms(xg, m, g, V)[0]
    a.Assemble()
    A = a.mat.to_scipy()
    assert a.mat.nrows == V.ndof
    h = 1.0 / 6 if D == 2 else 1.0 / 3
    K = A @ one  # the stiffness annihilates constants: the boundary mass remains
    assert abs(one @ K - 10.0 / h * (4.0 if D == 2 else 6.0)) < 1e-10 * (one @ K)
    # all POS: nothing active
    g2 = gf_of(xg, m, np.ones(m.nv))
    b = forms(xg, m, g2, V)[0]
    b.Assemble()
    assert b.mat.nrows == 0 and b.mat.nnz == 0


def test_vertex_zeros_and_determinism(xg, orc):
    m = MakeStructured2DMesh(8, 8)
    X, Y = m.coords.T
    lset = xg.GridFunction(xg.H1(m, order=1))
    xg.InterpolateToP1(lambda x, y: x - 0.5, lset)  # zeros on the mesh line x = 0.5
    V = xg.H1(m, order=2)
    adap = xg.LevelSetMeshAdaptation(m, order=2, threshold=0.2)
    adap.CalcDeformation(lambda x, y: (x - 0.5) + 0.3 * (y - 0.5) ** 2)
    for a in forms(xg, m, lset, V) + forms(xg, m, adap.lset_p1, V, adap)[1:]:
        first = assemble_vals(a)
        again = assemble_vals(a)
        for p, q in zip(first, again):
            assert np.array_equal(p, q)
        assert np.isfinite(first[2]).all()
    # quad mesh, a level set through vertices
    mq = MakeStructured2DMesh(6, 6, quads=True)
    gq = xg.GridFunction(xg.H1(mq, order=1))
    xg.InterpolateToP1(lambda x, y: x - 0.5, gq)
    Vq = xg.H1(mq, order=1)
    u, v = Vq.TnT()
    q = xg.BilinearForm(Vq)
    q += xg.grad(u) * xg.grad(v) * xg.dCut(gq, xg.NEG) + u * v * xg.dCut(gq, xg.IF)
    first = assemble_vals(q)
    again = assemble_vals(q)
    assert all(np.array_equal(p, r) for p, r in zip(first, again))
    one = np.ones(mq.nv)
    Q = q.mat.to_scipy()
    assert abs(one @ (Q @ one) - 1.0) < 1e-12  # the interface x = 0.5 has length 1


@pytest.mark.parametrize("D,k", [(2, 2), (3, 1)])
def test_terms_without_element_sets(xg, orc, D, k):
    """Terms without definedonelements: the elements with a part in the
    term's domain are active (the same set on the GPU and in the oracle)."""
    m = MakeStructured2DMesh(9, 9) if D == 2 else MakeStructured3DMesh(4)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.3) ** 2).sum(axis=1) - 0.36)
    g = gf_of(xg, m, l)
    V = xg.H1(m, order=k)
    u, v = V.TnT()
    a = xg.BilinearForm(V)
    a += xg.grad(u) * xg.grad(v) * xg.dCut(g, xg.NEG) + 3.0 * u * v * xg.dCut(g, xg.IF)
    a.Assemble()
    sp = orc.Space(m, k)
    rp, cols, vals = sp.assemble(l, [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG),
                                     dict(kind=orc.TERM_MASS, domain=orc.IF, coef=3.0)])
    r, cc, vv = a.mat.global_coo()
    ref = {(int(p), int(q)): float(x) for p, q, x in zip(np.repeat(np.arange(sp.ndof), np.diff(rp)), cols, vals)}
    got = {(int(p), int(q)): float(x) for p, q, x in zip(r, cc, vv)}
    assert set(ref) == set(got)
    scale = max(abs(x) for x in ref.values())
    assert max(abs(got[q] - ref[q]) for q in ref) < 1e-12 * scale

"""Boundary terms of bilinear forms on the GPU (xg_form_set_bnd_terms,
csrc/xg_bform.cu; `a += c * u * v * dCut(lset, dt, vb=BND, ...)` in a
BilinearForm) against the oracle (orc_assemble_bnd) and against ngsxfem's
tests/pytests/test_bndcut.py::test_bfi_assembly_2d.  Bars: the same
pattern, FP64 within 1e-12 of the largest entry, mixed within 1e-5."""
import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


def gf_of(xg, m, vals):
    g = xg.GridFunction(xg.H1(m, order=1))
    g.vec.copy_(torch.from_numpy(np.ascontiguousarray(vals)))
    return g


def compare(sp, ref_csr, mat, tol):
    rp, cols, vals = ref_csr
    r, c, v = mat.global_coo()
    ref_rows = np.repeat(np.arange(sp.ndof), np.diff(rp))
    ref = {(int(a), int(b)): float(x) for a, b, x in zip(ref_rows, cols, vals)}
    got = {(int(a), int(b)): float(x) for a, b, x in zip(r, c, v)}
    assert set(ref) == set(got)
    scale = max(abs(x) for x in ref.values())
    err = max(abs(got[q] - ref[q]) for q in ref) / scale
    assert err < tol, err


def bits_words(b):
    return b.words.cpu().numpy()


@pytest.mark.parametrize("D,k,n", [(2, 1, 9), (2, 2, 7), (2, 3, 5), (3, 1, 4), (3, 2, 3)])
def test_nitsche_form_with_boundary_terms(xg, orc, D, k, n):
    """Laplace on HASNEG, ghost penalty, and boundary penalties 10/h u v on
    the NEG part and 0.5 u v on the POS part of the boundary, the circle /
    sphere |x - 0.3| = 0.6 crossing the boundary of the unit square / cube."""
    m = MakeStructured2DMesh(n, n) if D == 2 else MakeStructured3DMesh(n)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.3) ** 2).sum(axis=1) - 0.36)
    g = gf_of(xg, m, l)
    ci = xg.CutInfo(m, g)
    hasneg, ifb = ci.GetElementsOfType(xg.HASNEG), ci.GetElementsOfType(xg.IF)
    gp = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=ifb, use_and=True)
    V = xg.H1(m, order=k)
    u, v = V.TnT()
    h = xg.specialcf.mesh_size
    sp = orc.Space(m, k)
    ref = sp.assemble(l, [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, defined_on=bits_words(hasneg)),
                          dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2, defined_on=bits_words(gp))],
                      bterms=[dict(domain=orc.NEG, coef=10.0, hpow=-1), dict(domain=orc.POS, coef=0.5)])
    for prec, tol in ((xg.PREC_FP64, 1e-12), (xg.PREC_MIXED, 1e-5)):
        a = xg.BilinearForm(V, precision=prec)
        a += xg.grad(u) * xg.grad(v) * xg.dCut(g, xg.NEG, definedonelements=hasneg)
        a += 0.1 / h ** 2 * (u - u.Other()) * (v - v.Other()) * xg.dFacetPatch(definedonelements=gp)
        a += (10.0 / h) * u * v * xg.dCut(g, xg.NEG, vb=xg.BND)
        a += 0.5 * u * v * xg.dCut(g, xg.POS, vb=xg.BND)
        a.Assemble()
        compare(sp, ref, a.mat, tol)


def test_boundary_only_forms_2d(xg, orc):
    """Forms of boundary terms alone: the cut points (IF, 2D), a side
    (definedon=mesh.Boundaries), a bitset over the BND elements; x + y/2 =
    0.6 on the unit square: NEG length 1.7, two IF points, bottom NEG 0.6."""
    m = MakeStructured2DMesh(9, 9)
    X, Y = m.coords.T
    l = X + 0.5 * Y - 0.6
    g = gf_of(xg, m, l)
    V = xg.H1(m, order=2)
    u, v = V.TnT()
    sp = orc.Space(m, 2)
    bottom = m.Boundaries("bottom")
    nb = len(bottom.Mask())
    sel = np.zeros(nb, bool)
    sel[::3] = True
    cases = [(xg.dCut(g, xg.NEG, vb=xg.BND), dict(domain=orc.NEG), 1.7),
             (xg.dCut(g, xg.IF, vb=xg.BND, order=0), dict(domain=orc.IF, order=0), 2.0),
             (xg.dCut(g, xg.NEG, vb=xg.BND, definedon=bottom), dict(domain=orc.NEG, defined_on=bottom.Mask()), 0.6),
             (xg.dCut(g, xg.POS, vb=xg.BND, definedonelements=xg.BitArray.from_numpy(sel)),
              dict(domain=orc.POS, defined_on=sel), None)]
    one = np.zeros(sp.ndof)
    one[: m.nv] = 1.0
    for meas, bt, val in cases:
        a = xg.BilinearForm(V)
        a += u * v * meas
        a.Assemble()
        d = bt.get("defined_on")
        if d is not None:
            w = np.zeros((nb + 63) // 64, dtype=np.uint64)
            for i in np.nonzero(d)[0]:
                w[i >> 6] |= np.uint64(1) << np.uint64(i & 63)
            bt = dict(bt, defined_on=w)
        compare(sp, sp.assemble(l, [], bterms=[bt]), a.mat, 1e-12)
        if val is not None:
            A = a.mat.to_scipy()
            assert abs(one @ (A @ one) - val) < 1e-12 * val


def test_bfi_assembly_2d(xg):
    """test_bndcut.py::test_bfi_assembly_2d: cut x = 0.4, u v dCut(NEG,
    vb=BND, definedon=left) times the interpolant of sin(x) cos(y) equals the
    P1 boundary mass matrix of the left side times it."""
    m = MakeStructured2DMesh(9, 9)
    X, Y = m.coords.T
    g = gf_of(xg, m, X - 0.4)
    V = xg.H1(m, order=1)
    u, v = V.TnT()
    a = xg.BilinearForm(V)
    a += u * v * xg.dCut(g, xg.NEG, vb=xg.BND, definedon=m.Boundaries("left"))
    a.Assemble()
    w = np.sin(X) * np.cos(Y)
    left = np.nonzero(X == 0.0)[0]
    left = left[np.argsort(Y[left])]
    ref = np.zeros(m.nv)
    for p, q in zip(left[:-1], left[1:]):
        hh = Y[q] - Y[p]
        ref[[p, q]] += hh / 6 * np.array([[2.0, 1.0], [1.0, 2.0]]) @ w[[p, q]]
    assert np.abs(a.mat.to_scipy() @ w - ref).max() < 1e-14


def test_boundary_terms_rejected_where_unsupported(xg):
    """IF on boundary triangles (3D) and integrands other than c u v raise."""
    m = MakeStructured3DMesh(3)
    g = gf_of(xg, m, m.coords[:, 0] - 0.4)
    V = xg.H1(m, order=1)
    u, v = V.TnT()
    a = xg.BilinearForm(V)
    a += u * v * xg.dCut(g, xg.IF, vb=xg.BND)
    with pytest.raises(RuntimeError):
        a.Assemble()
    b = xg.BilinearForm(V)
    b += xg.grad(u) * xg.grad(v) * xg.dCut(g, xg.NEG, vb=xg.BND)
    with pytest.raises(NotImplementedError):
        b.Assemble()

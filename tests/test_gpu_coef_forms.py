"""Volume terms with a coefficient field on the GPU (xg_form_set_coef_terms,
csrc/xg_cform.cu; `a += gf * grad(u) * grad(v) * dCut(...)`, `x * u * v *
dCut(...)` in a BilinearForm) against the oracle (orc_assemble_full).  Bars:
the same pattern, FP64 within 1e-12 of the largest entry, mixed within
1e-5; the planar closed form of the oracle's test through the Python API."""
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


def words(b):
    return b.words.cpu().numpy()


@pytest.mark.parametrize("D,k,kg,n", [(2, 1, 1, 9), (2, 2, 2, 7), (2, 3, 2, 5), (3, 1, 2, 4), (3, 2, 1, 3)])
def test_coefficient_terms_parity(xg, orc, D, k, kg, n):
    """Laplace with a field on HASNEG, x y u v on HASNEG, a field times the
    Nitsche terms and the penalty on IF, plain Laplace and ghost penalty."""
    m = MakeStructured2DMesh(n, n) if D == 2 else MakeStructured3DMesh(n)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.3) ** 2).sum(axis=1) - 0.36)
    g = gf_of(xg, m, l)
    ci = xg.CutInfo(m, g)
    hasneg, ifb = ci.GetElementsOfType(xg.HASNEG), ci.GetElementsOfType(xg.IF)
    gp = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=ifb, use_and=True)
    Vg = xg.H1(m, order=kg)
    if D == 2:
        kap = xg.GridFunction(Vg).Set(lambda x, y: 1.0 + x * x + 0.5 * y)
    else:
        kap = xg.GridFunction(Vg).Set(lambda x, y, z: 1.0 + x * x + 0.5 * y * z)
    V = xg.H1(m, order=k)
    u, v = V.TnT()
    h = xg.specialcf.mesh_size
    nrm = xg.Normalize(xg.grad(g))
    sp, spg = orc.Space(m, k), orc.Space(m, kg)
    gel = kap.vec.cpu().numpy()[spg.el_dofs()]
    ref = sp.assemble(l, [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, defined_on=words(hasneg)),
                          dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2, defined_on=words(gp))],
                      cterms=[dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, coef=2.0, gf_order=kg, gf_el=gel,
                                   defined_on=words(hasneg)),
                              dict(kind=orc.TERM_MASS, domain=orc.NEG, e=(1, 1, 0), defined_on=words(hasneg)),
                              dict(kind=orc.TERM_NGRADU_V, domain=orc.IF, coef=-1.0, gf_order=kg, gf_el=gel,
                                   defined_on=words(ifb)),
                              dict(kind=orc.TERM_U_NGRADV, domain=orc.IF, coef=-1.0, gf_order=kg, gf_el=gel,
                                   defined_on=words(ifb)),
                              dict(kind=orc.TERM_MASS, domain=orc.IF, coef=10.0 * k * k, hpow=-1, gf_order=kg,
                                   gf_el=gel, defined_on=words(ifb))])
    for prec, tol in ((xg.PREC_FP64, 1e-12), (xg.PREC_MIXED, 1e-5)):
        a = xg.BilinearForm(V, precision=prec)
        a += xg.grad(u) * xg.grad(v) * xg.dCut(g, xg.NEG, definedonelements=hasneg)
        a += 2.0 * kap * xg.grad(u) * xg.grad(v) * xg.dCut(g, xg.NEG, definedonelements=hasneg)
        a += xg.x * xg.y * u * v * xg.dCut(g, xg.NEG, definedonelements=hasneg)
        a += kap * (-xg.grad(u) * nrm * v - xg.grad(v) * nrm * u + (10.0 * k * k / h) * u * v) * \
            xg.dCut(g, xg.IF, definedonelements=ifb)
        a += 0.1 / h ** 2 * (u - u.Other()) * (v - v.Other()) * xg.dFacetPatch(definedonelements=gp)
        a.Assemble()
        compare(sp, ref, a.mat, tol)


def test_planar_field_integrals(xg):
    """x + y/2 = 0.6 on the unit square: with the field gf = x,
    1^T M_gf 1 = the NEG part's first moment 0.0716666..., and with the
    field 1 + x in the Laplacian x^T K x = area + first moment."""
    m = MakeStructured2DMesh(9, 9)
    X, Y = m.coords.T
    g = gf_of(xg, m, X + 0.5 * Y - 0.6)
    V = xg.H1(m, order=2)
    u, v = V.TnT()
    fx = xg.GridFunction(xg.H1(m, order=1)).Set(lambda x, y: x)
    one = np.zeros(V.ndof)
    one[: m.nv] = 1.0
    xv = np.zeros(V.ndof)
    xv[: m.nv] = X
    mx = 0.5 * (0.36 - 0.3 + 0.25 / 3)
    a = xg.BilinearForm(V)
    a += fx * u * v * xg.dCut(g, xg.NEG)
    a.Assemble()
    A = a.mat.to_scipy()
    assert abs(one @ (A @ one) - mx) < 1e-13
    b = xg.BilinearForm(V)
    b += (xg.grad(u) * xg.grad(v) + fx * xg.grad(u) * xg.grad(v)) * xg.dCut(g, xg.NEG, order=3)
    b.Assemble()
    B = b.mat.to_scipy()
    assert abs(xv @ (B @ xv) - (0.35 + mx)) < 1e-13


@pytest.mark.parametrize("D,k", [(2, 2), (3, 1), (3, 2)])
def test_vector_field_convection_parity(xg, orc, D, k):
    """CoefficientFunction((b_x, b_y[, b_z])) * grad(u) * v with GridFunction
    components (and a constant one in 3D): one convection term per component,
    with the unit vector and the component's field, the constant components as
    one plain convection term."""
    m = MakeStructured2DMesh(8, 8) if D == 2 else MakeStructured3DMesh(4)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.3) ** 2).sum(axis=1) - 0.36)
    g = gf_of(xg, m, l)
    hasneg = xg.CutInfo(m, g).GetElementsOfType(xg.HASNEG)
    Vg = xg.H1(m, order=1)
    bx = xg.GridFunction(Vg).Set(lambda *p: 1.0 + p[1])
    by = xg.GridFunction(Vg).Set(lambda *p: -0.5 * p[0])
    comps = (bx, by) if D == 2 else (bx, by, 0.25)
    V = xg.H1(m, order=k)
    u, v = V.TnT()
    sp, spg = orc.Space(m, k), orc.Space(m, 1)
    w = words(hasneg)
    cterms = [dict(kind=orc.TERM_CONV, domain=orc.NEG, b=tuple(1.0 if j == i else 0.0 for j in range(3)),
                   gf_order=1, gf_el=f.vec.cpu().numpy()[spg.el_dofs()], defined_on=w)
              for i, f in enumerate((bx, by))]
    terms = [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, defined_on=w)]
    if D == 3:
        terms.append(dict(kind=orc.TERM_CONV, domain=orc.NEG, b=(0.0, 0.0, 0.25), defined_on=w))
    ref = sp.assemble(l, terms, cterms=cterms)
    a = xg.BilinearForm(V)
    a += xg.grad(u) * xg.grad(v) * xg.dCut(g, xg.NEG, definedonelements=hasneg)
    a += xg.CoefficientFunction(comps) * xg.grad(u) * v * xg.dCut(g, xg.NEG, definedonelements=hasneg)
    a.Assemble()
    compare(sp, ref, a.mat, 1e-12)

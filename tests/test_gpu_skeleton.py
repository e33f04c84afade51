"""Skeleton terms on the GPU (xg_skel.cu through the C ABI) against the oracle:
cut-facet discontinuous-Galerkin forms (SymbolicCutFacetBilinearFormIntegrator,
xfem/symboliccutbfi.cpp:886-1572) and the derivative-jump ghost penalty on
whole facets (SymbolicFacetBilinearFormIntegrator2 with DiffOpDuDnk normal
derivatives, :1574-1735, xfem/ghostpenalty.cpp:221-365), on H1 and L2
spaces of orders 1..3, in the CutFEM step of demos/fictdom_dg.py.

Bars: the same sparsity pattern, FP64 values within 1e-12 of the largest
entry, mixed precision within 1e-5, bit-identical repeated steps."""
import numpy as np
import pytest
import torch

from test_gpu_parity import CASES, run_cutfem_step, setup_case

pytestmark = pytest.mark.gpu


def dg_form(orc, order):
    # fictdom_dg.py:125-135: volume stiffness, Nitsche on the interface, the
    # interior-penalty skeleton on the cut facets, the patch ghost penalty
    return [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG),
            dict(kind=orc.TERM_NGRADU_V, domain=orc.IF, coef=-1.0),
            dict(kind=orc.TERM_U_NGRADV, domain=orc.IF, coef=-1.0),
            dict(kind=orc.TERM_MASS, domain=orc.IF, coef=40.0, hpow=-1),
            dict(kind=orc.TERM_SKEL_JUMP, domain=orc.NEG, coef=20.0 * order ** 2, hpow=-1),
            dict(kind=orc.TERM_SKEL_FLUX, domain=orc.NEG, coef=-0.5),
            dict(kind=orc.TERM_SKEL_FLUX_T, domain=orc.NEG, coef=-0.5),
            dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2)]


def dn_form(orc, order):
    # derivative-jump ghost penalty sum_k gamma_k h^(2k-1) [d^k_n u][d^k_n v]
    # on the ghost facets (no patch terms: the skeleton kernel writes)
    t = [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG),
         dict(kind=orc.TERM_MASS, domain=orc.IF, coef=40.0, hpow=-1)]
    for k in range(1, order + 1):
        t.append(dict(kind=orc.TERM_SKEL_DN1 + k - 1, domain=orc.WHOLE, coef=0.1 ** k, hpow=2 * k - 1))
    return t


def dn_patch_form(orc, order):
    # both ghost penalties on the same facets: the skeleton kernel adds
    return dn_form(orc, order)[:2] + [dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2),
                                      dict(kind=orc.TERM_SKEL_DN1, domain=orc.WHOLE, coef=0.3, hpow=1),
                                      dict(kind=orc.TERM_SKEL_JUMP, domain=orc.POS, coef=2.0)]


FORMS = {"dg": dg_form, "dn": dn_form, "dn_patch": dn_patch_form}


def oracle_step(orc, m, l, order, terms, l2):
    """The CutFEM step of the oracle with the skeleton facet sets of
    fictdom_dg.py: NEG skeleton on (HASNEG, HASNEG) facets, POS on (HASPOS,
    HASPOS), whole-facet terms and the patch terms on the ghost facets."""
    sp = orc.Space(m, order, l2=l2)
    dom, ratio, bits = sp.cutinfo(l)
    ghost = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
    fneg = sp.facets_with_neighbor_types(bits[5], bits[5], True, True, True)
    fpos = sp.facets_with_neighbor_types(bits[6], bits[6], True, True, True)
    t2 = []
    for t in terms:
        t = dict(t)
        if t["kind"] == orc.TERM_GHOST_MASS:
            t["defined_on"] = ghost
        elif t["kind"] >= orc.TERM_SKEL_JUMP:
            t["defined_on"] = {orc.NEG: fneg, orc.POS: fpos, orc.WHOLE: ghost}[t["domain"]]
        else:
            t["defined_on"] = {orc.NEG: bits[5], orc.IF: bits[4], orc.POS: bits[6]}[t["domain"]]
        t2.append(t)
    return sp, sp.assemble(l, t2)


def compare(sp, ref_csr, mat, tol):
    rp, cols, vals = ref_csr
    r, c, v = mat.global_coo()
    ref_rows = np.repeat(np.arange(sp.ndof), np.diff(rp))
    ref = {(int(a), int(b)): float(x) for a, b, x in zip(ref_rows, cols, vals)}
    got = {(int(a), int(b)): float(x) for a, b, x in zip(r, c, v)}
    assert set(ref) == set(got)
    scale = max(1e-300, max(abs(x) for x in ref.values()))
    err = max(abs(got[k] - ref[k]) for k in ref) / scale
    assert err < tol, err


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("form", list(FORMS))
@pytest.mark.parametrize("l2", [True, False])
def test_skeleton_step_parity(xg, orc, case, order, form, l2):
    m, l, gf = setup_case(xg, orc, case)
    terms = FORMS[form](orc, order)
    sp, ref = oracle_step(orc, m, l, order, terms, l2)
    V = xg.L2(m, order=order) if l2 else xg.H1(m, order=order)
    assert np.array_equal(V.element_dofs(), sp.el_dofs())
    mat = run_cutfem_step(xg, V, gf, terms, xg.PREC_FP64)
    compare(sp, ref, mat, 1e-12)


@pytest.mark.parametrize("case", ["circle2d", "sphere3d"])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_skeleton_mixed_and_deterministic(xg, orc, case, order):
    m, l, gf = setup_case(xg, orc, case)
    V = xg.L2(m, order=order)
    terms = dg_form(orc, order) + dn_form(orc, order)[2:]
    a = run_cutfem_step(xg, V, gf, terms, xg.PREC_FP64)
    va = a.vals[: a.nnz].clone()
    b = run_cutfem_step(xg, V, gf, terms, xg.PREC_FP64)
    assert torch.equal(va, b.vals[: b.nnz])
    c = run_cutfem_step(xg, V, gf, terms, xg.PREC_MIXED)
    assert c.nnz == a.nnz and torch.equal(a.cols[: a.nnz], c.cols[: c.nnz])
    rel = float((va - c.vals[: c.nnz]).abs().max() / va.abs().max())
    assert rel < 1e-5, rel


def test_python_dg_script(xg, orc):
    """demos/fictdom_dg.py:100-135 through the Python mirror on an L2 P2
    space (dCut(..., skeleton=True), specialcf.normal, .Other(), dn jumps on
    dx(skeleton=True)) equals the oracle's assembly on the same sets."""
    m, l, gf = setup_case(xg, orc, "circle2d")
    order = 2
    V = xg.L2(m, order=order, dgjumps=True)
    ci = xg.CutInfo(m, gf)
    hasneg, hasif = ci.GetElementsOfType(xg.HASNEG), ci.GetElementsOfType(xg.IF)
    ba_gp = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=hasif)
    ba_fd = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=hasneg)
    u, v = V.TnT()
    h = xg.specialcf.mesh_size
    nh = xg.Normalize(xg.grad(gf))
    nF = xg.specialcf.normal(2)
    flux_u = -0.5 * (xg.grad(u) + xg.grad(u.Other())) * nF
    flux_v = -0.5 * (xg.grad(v) + xg.grad(v.Other())) * nF
    jump_u, jump_v = u - u.Other(), v - v.Other()
    a = xg.BilinearForm(V)
    a += xg.grad(u) * xg.grad(v) * xg.dCut(gf, xg.NEG, definedonelements=hasneg)
    a += (10.0 / h * jump_u * jump_v + flux_u * jump_v + flux_v * jump_u) * \
        xg.dCut(gf, xg.NEG, skeleton=True, definedonelements=ba_fd)
    a += (-xg.grad(u) * nh * v - xg.grad(v) * nh * u + 20.0 / h * u * v) * xg.dCut(gf, xg.IF, definedonelements=hasif)
    a += 0.1 / h ** 2 * (u - u.Other()) * (v - v.Other()) * xg.dFacetPatch(definedonelements=ba_gp)
    a += 0.01 * h ** 3 * (xg.dn(u, 2) - xg.dn(u.Other(), 2)) * (xg.dn(v, 2) - xg.dn(v.Other(), 2)) * \
        xg.dx(skeleton=True, definedonelements=ba_gp)
    a.Assemble(ci)
    sp = orc.Space(m, order, l2=True)
    dom, ratio, bits = sp.cutinfo(l)
    gpb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
    fdb = sp.facets_with_neighbor_types(bits[5], bits[5], True, True, True)
    assert np.array_equal(ba_gp.words.cpu().numpy().view(np.uint64), gpb)
    assert np.array_equal(ba_fd.words.cpu().numpy().view(np.uint64), fdb)
    terms = [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, defined_on=bits[5]),
             dict(kind=orc.TERM_SKEL_JUMP, domain=orc.NEG, coef=10.0, hpow=-1, defined_on=fdb),
             dict(kind=orc.TERM_SKEL_FLUX, domain=orc.NEG, coef=-0.5, defined_on=fdb),
             dict(kind=orc.TERM_SKEL_FLUX_T, domain=orc.NEG, coef=-0.5, defined_on=fdb),
             dict(kind=orc.TERM_NGRADU_V, domain=orc.IF, coef=-1.0, defined_on=bits[4]),
             dict(kind=orc.TERM_U_NGRADV, domain=orc.IF, coef=-1.0, defined_on=bits[4]),
             dict(kind=orc.TERM_MASS, domain=orc.IF, coef=20.0, hpow=-1, defined_on=bits[4]),
             dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2, defined_on=gpb),
             dict(kind=orc.TERM_SKEL_DN2, domain=orc.WHOLE, coef=0.01, hpow=3, defined_on=gpb)]
    compare(sp, sp.assemble(l, terms), a.mat, 1e-12)


def quadratic_coefs(mesh, el_dofs, ndof, order, p):
    """Coefficients of a quadratic polynomial in the element basis: vertex
    values, 4 p(mid) - 2 (p_a + p_b) on the quadratic edge functions, 0 on the
    cubic edge and face functions."""
    D = mesh.dim
    edges = [(0, 1), (0, 2), (1, 2)] if D == 2 else [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    out = np.zeros(ndof)
    for e in range(mesh.ne):
        X = mesh.coords[mesh.elements[e]]
        loc = [p(X[i]) for i in range(D + 1)]
        if order >= 2:
            for a_, b_ in edges:
                loc.append(4 * p(0.5 * (X[a_] + X[b_])) - 2 * (p(X[a_]) + p(X[b_])))
                if order == 3:
                    loc.append(0.0)
        loc += [0.0] * (el_dofs.shape[1] - len(loc))
        out[el_dofs[e]] = loc
    return out


@pytest.mark.parametrize("dim,order", [(2, 2), (2, 3), (3, 2)])
def test_unfitted_dg_solve_reproduces_quadratic(xg, dim, order):
    """Unfitted symmetric interior-penalty DG (the fictdom_dg form) on L2 P2 /
    P3 with the planar boundary x = c: u = x^2 - c^2 solves -laplace u = -2
    with u = 0 on the cut and homogeneous Neumann data on the box sides.  The
    method is consistent and u lies in the space, so the solution of the
    assembled system is u itself."""
    import scipy.sparse as sps
    import scipy.sparse.linalg as spla
    from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh
    c = 0.537
    m = MakeStructured2DMesh(8, 7) if dim == 2 else MakeStructured3DMesh(4)
    V1 = xg.H1(m, order=1)
    gf = xg.GridFunction(V1)
    xg.InterpolateToP1(m.coords[:, 0] - c, gf)
    ci = xg.CutInfo(m, gf)
    hasneg, hasif = ci.GetElementsOfType(xg.HASNEG), ci.GetElementsOfType(xg.IF)
    ba_gp = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=hasif)
    ba_fd = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=hasneg)
    V = xg.L2(m, order=order, dgjumps=True)
    u, v = V.TnT()
    h = xg.specialcf.mesh_size
    nh = xg.Normalize(xg.grad(gf))
    nF = xg.specialcf.normal(dim)
    lam = 20.0 * order ** 2
    flux_u = -0.5 * (xg.grad(u) + xg.grad(u.Other())) * nF
    flux_v = -0.5 * (xg.grad(v) + xg.grad(v.Other())) * nF
    jump_u, jump_v = u - u.Other(), v - v.Other()
    a = xg.BilinearForm(V)
    a += xg.grad(u) * xg.grad(v) * xg.dCut(gf, xg.NEG, definedonelements=hasneg)
    a += (lam / h * jump_u * jump_v + flux_u * jump_v + flux_v * jump_u) * \
        xg.dCut(gf, xg.NEG, skeleton=True, definedonelements=ba_fd)
    a += (-xg.grad(u) * nh * v - xg.grad(v) * nh * u + lam / h * u * v) * xg.dCut(gf, xg.IF, definedonelements=hasif)
    a += 0.1 / h ** 2 * (u - u.Other()) * (v - v.Other()) * xg.dFacetPatch(definedonelements=ba_gp)
    a.Assemble(ci)
    f = xg.LinearForm(V)
    f += -2.0 * v * xg.dCut(gf, xg.NEG, definedonelements=hasneg)
    f.Assemble(ci)
    A = a.mat.to_scipy().tocsr()
    act = a.mat.row_dof[: a.mat.nrows].cpu().numpy()
    Aa = A[act][:, act]
    x = spla.spsolve(sps.csc_matrix(Aa), f.vec.cpu().numpy()[act])
    ue = quadratic_coefs(m, V.element_dofs(), V.ndof, order, lambda X: X[0] ** 2 - c * c)[act]
    assert np.abs(x - ue).max() < 1e-9 * max(1.0, np.abs(ue).max()), np.abs(x - ue).max()

"""Bilinear forms on regions of several level sets on the GPU
(xg_mlset_form_create / xg_mlset_form_assemble; csrc/xg_mlform.cu) against
the oracle (orc_mlset_assemble): the form of ngsxfem's
tests/pytests/test_mlset_poisson.py (the unit square / cube as the region of
four / six level sets, stiffness on the region, Nitsche on every boundary
piece with its outer normal, ghost penalty), written through the Python
mirror, on H1 spaces of orders 1..3.  Bars: the same pattern, FP64 within
1e-12 of the largest entry, mixed within 1e-5; and the Poisson problem of
that test solved with the assembled matrix converges at the expected rate."""
import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


def setup(xg, D, n):
    from ngsxfem_gb300.mlset import DomainTypeArray, MultiLevelsetCutInfo
    if D == 2:
        m = MakeStructured2DMesh(n, n, -0.2, 1.2, -0.2, 1.2)
        X, Y = m.coords.T
        vals = [-Y, X - 1, Y - 1, -X]
    else:
        m = MakeStructured3DMesh(n, box=((-0.2, 1.2),) * 3)
        X, Y, Z = m.coords.T
        vals = [-Y, X - 1, Y - 1, -X, -Z, Z - 1]
    V1 = xg.H1(m, order=1)
    lsets = []
    for v in vals:
        g = xg.GridFunction(V1)
        xg.InterpolateToP1(v, g)
        lsets.append(g)
    lsets = tuple(lsets)
    region = DomainTypeArray([(xg.NEG,) * len(vals)])
    region.Compress(lsets)
    mlci = MultiLevelsetCutInfo(m, lsets)
    hasneg = mlci.GetElementsWithContribution(region)
    els_if = hasneg & ~mlci.GetElementsOfType(region)
    facets_gp = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=els_if, use_and=True)
    # the elements with a contribution to each boundary piece (els_if_singe of
    # test_mlset_poisson.py)
    region.els_bnd = {piece: mlci.GetElementsWithContribution(piece) for piece in region.Boundary()}
    return m, lsets, region, hasneg, facets_gp


def poisson_form(xg, V, lsets, region, hasneg, facets_gp, k, mass=False):
    u, v = V.TnT()
    h = xg.specialcf.mesh_size
    a = xg.BilinearForm(V)
    if mass:
        a += u * v * xg.dCut(lsets, region, definedonelements=hasneg)
        return a
    a += xg.grad(u) * xg.grad(v) * xg.dCut(lsets, region, definedonelements=hasneg)
    for piece, n in region.GetOuterNormals(lsets).items():
        a += (-xg.grad(u) * n * v - xg.grad(v) * n * u + (10.0 * k * k / h) * u * v) * \
            xg.dCut(lsets, piece, definedonelements=region.els_bnd[piece])
    a += 0.1 / h ** 2 * (u - u.Other()) * (v - v.Other()) * xg.dFacetPatch(definedonelements=facets_gp)
    return a


def oracle_terms(orc, region, lsets, hasneg, k):
    """The same form as oracle terms."""
    M = len(lsets)
    terms = [dict(kind=orc.TERM_LAPLACE, tuples=region.as_list, defined_on=hasneg.words.cpu().numpy())]
    for piece, n in region.GetOuterNormals(lsets).items():
        i = piece.index(orc.IF)
        sign = n.monos[0].c
        bits = region.els_bnd[piece].words.cpu().numpy()
        terms += [dict(kind=orc.TERM_NGRADU_V, tuples=[piece], coef=-sign, normal_lset=i, defined_on=bits),
                  dict(kind=orc.TERM_U_NGRADV, tuples=[piece], coef=-sign, normal_lset=i, defined_on=bits),
                  dict(kind=orc.TERM_MASS, tuples=[piece], coef=10.0 * k * k, hpow=-1, defined_on=bits)]
    assert all(len(t["tuples"][0]) == M for t in terms)
    return terms


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


@pytest.mark.parametrize("D,k,n", [(2, 1, 9), (2, 2, 7), (2, 3, 5), (3, 1, 4), (3, 2, 3)])
def test_mlset_poisson_form_parity(xg, orc, D, k, n):
    m, lsets, region, hasneg, facets_gp = setup(xg, D, n)
    V = xg.H1(m, order=k)
    a = poisson_form(xg, V, lsets, region, hasneg, facets_gp, k)
    a.Assemble()
    sp = orc.Space(m, k)
    L = np.stack([g.vec.cpu().numpy() for g in lsets])
    ref = sp.mlset_assemble(L, oracle_terms(orc, region, lsets, hasneg, k),
                            [dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2,
                                  defined_on=facets_gp.words.cpu().numpy())])
    compare(sp, ref, a.mat, 1e-12)
    b = poisson_form(xg, V, lsets, region, hasneg, facets_gp, k)
    b.precision = xg.PREC_MIXED
    b.Assemble()
    compare(sp, ref, b.mat, 1e-5)


@pytest.mark.parametrize("k", [1, 2])
def test_mlset_poisson_converges(xg, k):
    """tests/pytests/test_mlset_poisson.py's problem: -laplace u = f on the unit
    square given by four level sets, u = 16 x (1-x) y (1-y) (zero on the
    boundary, imposed by Nitsche).  Load vector M f_h (the region's mass matrix
    times the interpolant), error |u_h - I u|_M in the region's mass norm on
    four meshes: as in the reference's convergence study, the first rate is
    left out and the mean of the others is >= k + 1 - 1/4."""
    import scipy.sparse.linalg as spla
    errs = []
    for n in (6, 12, 24, 48):
        m, lsets, region, hasneg, facets_gp = setup(xg, 2, n)
        V = xg.H1(m, order=k)
        a = poisson_form(xg, V, lsets, region, hasneg, facets_gp, k)
        a.Assemble()
        mm = poisson_form(xg, V, lsets, region, hasneg, facets_gp, k, mass=True)
        mm.Assemble()
        uex = xg.GridFunction(V).Set(lambda x, y: 16 * x * (1 - x) * y * (1 - y))
        f = xg.GridFunction(V).Set(lambda x, y: 32 * (y * (1 - y) + x * (1 - x)))
        A = a.mat.to_scipy().tocsc()
        Mm = mm.mat.to_scipy().tocsr()
        act = a.mat.row_dof[: a.mat.nrows].cpu().numpy()
        rhs = Mm @ f.vec.cpu().numpy()
        x = spla.spsolve(A[act][:, act], rhs[act])
        e = np.zeros(V.ndof)
        e[act] = x - uex.vec.cpu().numpy()[act]
        errs.append(np.sqrt(e @ (Mm @ e)))
    rates = [np.log2(errs[i] / errs[i + 1]) for i in range(3)]
    assert np.mean(rates[1:]) > k + 1 - 0.25, (errs, rates)

"""Bilinear forms on the deformed (isoparametric) mesh on the GPU: ngsxfem's P2
workflow `deformation = LevelSetMeshAdaptation(mesh, order=2).CalcDeformation
(lset_p2)`, `a += ... * dCut(lsetp1, NEG, deformation=deformation)`
(python/lsetcurv.py:281-356), here xg_iso_deformation + xg_cterm.d_deform
(csrc/xg_cform.cu) against the oracle (orc_assemble_full with
orc_iso_theta_mesh).  The two deformations come from separate Newton
searches (GPU and CPU), so the bar is 1e-10 of the largest entry (mixed
1e-5); the deformed mass converges to the circle's area."""
import math

import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


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


@pytest.mark.parametrize("D,k,N,dpatch", [(2, 1, 8, False), (2, 2, 8, True), (3, 1, 4, True), (3, 2, 4, False),
                                          (2, 3, 6, True)])
def test_deformed_nitsche_form_parity(xg, orc, D, k, N, dpatch):
    """The form of demos/fictdom.py on the deformed mesh (the ghost penalty
    deformed too when dpatch)."""
    if D == 2:
        m = MakeStructured2DMesh(N, N, -1, 1, -1, 1)
        phi = lambda x, y: np.sqrt(x * x + y * y) - 0.5  # noqa: E731
    else:
        m = MakeStructured3DMesh(N, box=((-1, 1),) * 3)
        phi = lambda x, y, z: np.sqrt(x * x + y * y + z * z) - 0.55  # noqa: E731
    adap = xg.LevelSetMeshAdaptation(m, order=2, threshold=0.2)
    deformation = adap.CalcDeformation(phi)
    lsetp1 = adap.lset_p1
    ci = xg.CutInfo(m, lsetp1)
    hasneg, ifb = ci.GetElementsOfType(xg.HASNEG), ci.GetElementsOfType(xg.IF)
    gp = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=ifb, use_and=True)
    V = xg.H1(m, order=k)
    u, v = V.TnT()
    h = xg.specialcf.mesh_size
    n = xg.Normalize(xg.grad(lsetp1))
    p2 = xg.P2ElementValues(m, phi)
    theta, _ = orc.iso_theta_mesh(m, p2, threshold=0.2)
    l = lsetp1.vec.cpu().numpy()
    sp = orc.Space(m, k)
    dn = dict(theta_el=theta)
    ref = sp.assemble(l, [dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2, defined_on=words(gp))],
                      cterms=[dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, defined_on=words(hasneg), **dn),
                              dict(kind=orc.TERM_NGRADU_V, domain=orc.IF, coef=-1.0, defined_on=words(ifb), **dn),
                              dict(kind=orc.TERM_U_NGRADV, domain=orc.IF, coef=-1.0, defined_on=words(ifb), **dn),
                              dict(kind=orc.TERM_MASS, domain=orc.IF, coef=10.0 * k * k, hpow=-1,
                                   defined_on=words(ifb), **dn)],
                      theta_patch=theta if dpatch else None)
    for prec, tol in ((xg.PREC_FP64, 1e-10), (xg.PREC_MIXED, 1e-5)):
        a = xg.BilinearForm(V, precision=prec)
        a += xg.grad(u) * xg.grad(v) * xg.dCut(lsetp1, xg.NEG, definedonelements=hasneg, deformation=deformation)
        a += (-xg.grad(u) * n * v - xg.grad(v) * n * u + (10.0 * k * k / h) * u * v) * \
            xg.dCut(lsetp1, xg.IF, definedonelements=ifb, deformation=deformation)
        a += 0.1 / h ** 2 * (u - u.Other()) * (v - v.Other()) * \
            xg.dFacetPatch(definedonelements=gp, deformation=deformation if dpatch else None)
        a.Assemble()
        compare(sp, ref, a.mat, tol)


def test_deformed_mass_converges_to_the_area(xg):
    """1^T M 1 of the deformed NEG mass matrix: the circle's area pi/4 at
    third order (the geometry of tests/pytests/test_intcurved.py)."""
    errs = []
    for N in (8, 16, 32):
        m = MakeStructured2DMesh(N, N, -1, 1, -1, 1)
        adap = xg.LevelSetMeshAdaptation(m, order=2, threshold=0.2)
        deformation = adap.CalcDeformation(lambda x, y: np.sqrt(x * x + y * y) - 0.5)
        lsetp1 = adap.lset_p1
        V = xg.H1(m, order=1)
        u, v = V.TnT()
        a = xg.BilinearForm(V)
        a += u * v * xg.dCut(lsetp1, xg.NEG, order=2, deformation=deformation)
        a.Assemble()
        one = np.ones(V.ndof)
        errs.append(abs(one @ (a.mat.to_scipy() @ one) - 0.25 * math.pi))
    eoc = [math.log2(p / q) for p, q in zip(errs[:-1], errs[1:])]
    assert errs[-1] < 1e-5 and min(eoc) > 2.75, (errs, eoc)


@pytest.mark.parametrize("k", [1, 2])
def test_deformed_linear_form(xg, orc, k):
    """LinearForm on the deformed mesh (the right-hand side of
    demos/fictdom.py with `deformation=`): f = x y on NEG and 2 on IF.  With
    the vertex functions summing to 1, b = M_f 1 for the oracle's deformed
    mass matrices with the same coefficients."""
    m = MakeStructured2DMesh(8, 8, -1, 1, -1, 1)
    phi = lambda x, y: np.sqrt(x * x + y * y) - 0.5  # noqa: E731
    adap = xg.LevelSetMeshAdaptation(m, order=2, threshold=0.2)
    deformation = adap.CalcDeformation(phi)
    lsetp1 = adap.lset_p1
    V = xg.H1(m, order=k)
    v = V.TestFunction()
    f = xg.LinearForm(V)
    f += xg.x * xg.y * v * xg.dCut(lsetp1, xg.NEG, deformation=deformation)
    f += 2.0 * v * xg.dCut(lsetp1, xg.IF, deformation=deformation)
    f.Assemble()
    got = f.vec.cpu().numpy()
    theta, _ = orc.iso_theta_mesh(m, xg.P2ElementValues(m, phi), threshold=0.2)
    sp = orc.Space(m, k)
    rp, cols, vals = sp.assemble(lsetp1.vec.cpu().numpy(), [], cterms=[
        dict(kind=orc.TERM_MASS, domain=orc.NEG, e=(1, 1, 0), theta_el=theta),
        dict(kind=orc.TERM_MASS, domain=orc.IF, coef=2.0, theta_el=theta)])
    A = np.zeros((sp.ndof, sp.ndof))
    np.add.at(A, (np.repeat(np.arange(sp.ndof), np.diff(rp)), cols), vals)
    one = np.zeros(sp.ndof)
    one[: m.nv] = 1.0
    ref = A @ one
    assert np.abs(got - ref).max() < 1e-10 * np.abs(ref).max()


def test_integrate_with_deformation(xg):
    m = MakeStructured2DMesh(16, 16, -1, 1, -1, 1)
    adap = xg.LevelSetMeshAdaptation(m, order=2, threshold=0.2)
    deformation = adap.CalcDeformation(lambda x, y: np.sqrt(x * x + y * y) - 0.5)
    lsetp1 = adap.lset_p1
    a = xg.Integrate(xg.dCut(lsetp1, xg.NEG, order=2, deformation=deformation), m)
    assert a == adap.Integrate(xg.NEG, order=2)
    assert abs(a - 0.25 * math.pi) < 5e-4  # third-order geometry error at h = 1/8

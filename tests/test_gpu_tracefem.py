"""The TraceFEM form of the reference's demos/tracefem.py on the GPU: the
Laplace-Beltrami operator P(grad u) . P(grad v) + u v on the interface
(P(w) = w - (w . n) n: the Laplacian minus the normal-normal term,
XG_TERM_NGRADU_NGRADV) and the normal diffusion (1/h) (grad u . n)(grad v . n)
on the whole interface elements (dx(definedonelements=ba_IF), domain
XG_WHOLE), plain and on the deformed mesh, against the oracle
(orc_assemble_full).  Bars: 1e-12 of the largest entry (the deformed form
1e-10: the GPU and the oracle run separate Newton searches)."""
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


def tracefem_form(xg, V, lset, ba_if, deformation=None):
    u, v = V.TnT()
    n = xg.Normalize(xg.grad(lset))
    h = xg.specialcf.mesh_size

    def P(w):
        return w - (w * n) * n

    a = xg.BilinearForm(V)
    a += (P(xg.grad(u)) * P(xg.grad(v)) + u * v) * xg.dCut(lset, xg.IF, definedonelements=ba_if,
                                                           deformation=deformation)
    a += (1.0 / h) * (xg.grad(u) * n) * (xg.grad(v) * n) * xg.dx(definedonelements=ba_if, deformation=deformation)
    a.Assemble()
    return a


@pytest.mark.parametrize("D,k,n", [(2, 1, 10), (2, 2, 8), (3, 1, 4), (3, 2, 4)])
def test_tracefem_form_parity(xg, orc, D, k, n):
    m = MakeStructured2DMesh(n, n) if D == 2 else MakeStructured3DMesh(n)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.45) ** 2).sum(axis=1) - 0.33 ** 2)
    g = xg.GridFunction(xg.H1(m, order=1))
    xg.InterpolateToP1(l, g)
    ba_if = xg.CutInfo(m, g).GetElementsOfType(xg.IF)
    V = xg.H1(m, order=k)
    a = tracefem_form(xg, V, g, ba_if)
    sp = orc.Space(m, k)
    w = words(ba_if)
    NN = orc.TERM_NGRADU_NGRADV
    ref = sp.assemble(g.vec.cpu().numpy(),
                      [dict(kind=orc.TERM_LAPLACE, domain=orc.IF, defined_on=w),
                       dict(kind=orc.TERM_MASS, domain=orc.IF, defined_on=w)],
                      cterms=[dict(kind=NN, domain=orc.IF, coef=-1.0, defined_on=w),
                              dict(kind=NN, domain=orc.WHOLE, hpow=-1, defined_on=w)])
    compare(sp, ref, a.mat, 1e-12)
    # the rows are the dofs of the interface elements only
    assert a.mat.nrows == len(np.unique(sp.el_dofs()[np.asarray(sp.cutinfo(g.vec.cpu().numpy())[0]) == orc.IF]))


@pytest.mark.parametrize("D,k,N", [(2, 2, 8), (3, 1, 4)])
def test_deformed_tracefem_form_parity(xg, orc, D, k, N):
    if D == 2:
        m = MakeStructured2DMesh(N, N, -1, 1, -1, 1)
        phi = lambda x, y: np.sqrt(x * x + y * y) - 0.5  # noqa: E731
    else:
        m = MakeStructured3DMesh(N, box=((-1, 1),) * 3)
        phi = lambda x, y, z: np.sqrt(x * x + y * y + z * z) - 0.55  # noqa: E731
    adap = xg.LevelSetMeshAdaptation(m, order=2, threshold=0.2)
    deformation = adap.CalcDeformation(phi)
    lsetp1 = adap.lset_p1
    ba_if = xg.CutInfo(m, lsetp1).GetElementsOfType(xg.IF)
    V = xg.H1(m, order=k)
    a = tracefem_form(xg, V, lsetp1, ba_if, deformation)
    theta, _ = orc.iso_theta_mesh(m, xg.P2ElementValues(m, phi), threshold=0.2)
    sp = orc.Space(m, k)
    w = words(ba_if)
    dn = dict(theta_el=theta, defined_on=w)
    NN = orc.TERM_NGRADU_NGRADV
    ref = sp.assemble(lsetp1.vec.cpu().numpy(), [],
                      cterms=[dict(kind=orc.TERM_LAPLACE, domain=orc.IF, **dn),
                              dict(kind=orc.TERM_MASS, domain=orc.IF, **dn),
                              dict(kind=NN, domain=orc.IF, coef=-1.0, **dn),
                              dict(kind=NN, domain=orc.WHOLE, hpow=-1, **dn)])
    compare(sp, ref, a.mat, 1e-10)

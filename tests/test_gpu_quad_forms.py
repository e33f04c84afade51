"""Bilinear forms of the Q1 space on quadrilateral and hexahedral meshes on
the GPU (xg_quad_form_*, csrc/xg_qform.cu; `BilinearForm(H1(quad_mesh,
order=1))` with dCut terms) against the oracle (orc_quad_assemble) and the
planar closed forms of tests/test_oracle_quad_forms.py.  Bar: the same
pattern, values within 1e-12 of the largest entry; repeated assemblies
bit-identical."""
import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


def gf_of(xg, m, vals):
    g = xg.GridFunction(xg.H1(m, order=1))
    g.vec.copy_(torch.from_numpy(np.ascontiguousarray(vals)))
    return g


def compare(nv, ref_csr, mat, tol):
    rp, cols, vals = ref_csr
    r, c, v = mat.global_coo()
    ref_rows = np.repeat(np.arange(nv), np.diff(rp))
    ref = {(int(a), int(b)): float(x) for a, b, x in zip(ref_rows, cols, vals)}
    got = {(int(a), int(b)): float(x) for a, b, x in zip(r, c, v)}
    assert set(ref) == set(got)
    scale = max(abs(x) for x in ref.values())
    err = max(abs(got[q] - ref[q]) for q in ref) / scale
    assert err < tol, err


@pytest.mark.parametrize("D,n,pol", [(2, 9, 1), (2, 7, 0), (2, 8, 2), (3, 5, 1), (3, 4, 2)])
def test_quad_nitsche_form_parity(xg, orc, D, n, pol):
    m = MakeStructured2DMesh(n, n, quads=True) if D == 2 else MakeStructured3DMesh(n, hexes=True)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.3) ** 2).sum(axis=1) - 0.36)
    g = gf_of(xg, m, l)
    ci = xg.CutInfo(m, g)
    hasneg, ifb = ci.GetElementsOfType(xg.HASNEG), ci.GetElementsOfType(xg.IF)
    V = xg.H1(m, order=1)
    u, v = V.TnT()
    h = xg.specialcf.mesh_size
    nrm = xg.Normalize(xg.grad(g))
    b = (0.4, -0.3, 0.2)[:D]
    a = xg.BilinearForm(V)
    a += xg.grad(u) * xg.grad(v) * xg.dCut(g, xg.NEG, definedonelements=hasneg, quad_dir_policy=pol)
    a += 0.5 * (xg.grad(u) * b) * v * xg.dCut(g, xg.NEG, definedonelements=hasneg, quad_dir_policy=pol)
    a += (-xg.grad(u) * nrm * v - xg.grad(v) * nrm * u + (10.0 / h) * u * v) * \
        xg.dCut(g, xg.IF, definedonelements=ifb, quad_dir_policy=pol)
    a.Assemble()
    w = lambda bits: bits.words.cpu().numpy()  # noqa: E731
    ref, st = orc.quad_assemble(m, l, [
        dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, defined_on=w(hasneg)),
        dict(kind=orc.TERM_CONV, domain=orc.NEG, coef=0.5, b=tuple(b) + (0.0,) * (3 - D), defined_on=w(hasneg)),
        dict(kind=orc.TERM_NGRADU_V, domain=orc.IF, coef=-1.0, defined_on=w(ifb)),
        dict(kind=orc.TERM_U_NGRADV, domain=orc.IF, coef=-1.0, defined_on=w(ifb)),
        dict(kind=orc.TERM_MASS, domain=orc.IF, coef=10.0, hpow=-1, defined_on=w(ifb))], policy=pol)
    assert st == 0
    compare(m.nv, ref, a.mat, 1e-12)
    first = a.mat.global_coo()[2].copy()
    a.Assemble()
    assert np.array_equal(first, a.mat.global_coo()[2])


@pytest.mark.parametrize("D", [2, 3])
def test_planar_quad_closed_forms(xg, D):
    m = MakeStructured2DMesh(7, 7, quads=True) if D == 2 else MakeStructured3DMesh(5, hexes=True)
    X, Y = m.coords[:, 0], m.coords[:, 1]
    g = gf_of(xg, m, X + 0.5 * Y - 0.6)
    V = xg.H1(m, order=1)
    u, v = V.TnT()
    one = np.ones(m.nv)
    area, mx, length = 0.35, 0.5 * (0.36 - 0.3 + 0.25 / 3), np.sqrt(1.25)
    for integrand, meas, uu, vv, val in [(u * v, xg.NEG, one, one, area), (u * v, xg.NEG, X, one, mx),
                                         (xg.grad(u) * xg.grad(v), xg.NEG, X, X, area),
                                         (u * v, xg.IF, one, one, length), (u * v, xg.POS, one, one, 1 - area)]:
        a = xg.BilinearForm(V)
        a += integrand * xg.dCut(g, meas)
        a.Assemble()
        A = a.mat.to_scipy()
        assert abs(vv @ (A @ uu) - val) < 1e-13, (meas, vv @ (A @ uu), val)

"""Bilinear forms of the Q1 space on quadrilateral and hexahedral meshes in
the oracle (orc_quad_assemble: SymbolicCutBFI on ET_QUAD / ET_HEX,
xfem/symboliccutbfi.cpp:76-486, with the quad rule of
cutint/straightcutrule.cpp:206-501) against closed forms of the planar cut
x + y/2 = 0.6 of the unit square / cube: NEG measure 0.35, its first
moment in x 0.0716666..., the interface's measure sqrt(1.25) (times 1 in
z); Q1 holds 1, x and y exactly, so 1^T M 1, x^T M 1, x^T K x and y^T K y are
those integrals, and K annihilates constants.  CPU only."""
import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh
from oracle import oracle as orc

AREA, MX, LEN = 0.35, 0.5 * (0.36 - 0.3 + 0.25 / 3), np.sqrt(1.25)


def dense(n, csr):
    rp, cols, vals = csr
    A = np.zeros((n, n))
    rows = np.repeat(np.arange(n), np.diff(rp))
    np.add.at(A, (rows, cols), vals)
    return A


@pytest.mark.parametrize("D", [2, 3])
def test_planar_quad_forms(D):
    m = MakeStructured2DMesh(7, 7, quads=True) if D == 2 else MakeStructured3DMesh(5, hexes=True)
    X, Y = m.coords[:, 0], m.coords[:, 1]
    l = X + 0.5 * Y - 0.6
    one = np.ones(m.nv)
    for terms, u, v, val in [([dict(kind=orc.TERM_MASS, domain=orc.NEG)], one, one, AREA),
                             ([dict(kind=orc.TERM_MASS, domain=orc.NEG)], X, one, MX),
                             ([dict(kind=orc.TERM_LAPLACE, domain=orc.NEG)], X, X, AREA),
                             ([dict(kind=orc.TERM_LAPLACE, domain=orc.NEG)], Y, Y, AREA),
                             ([dict(kind=orc.TERM_MASS, domain=orc.POS)], one, one, 1 - AREA),
                             ([dict(kind=orc.TERM_MASS, domain=orc.IF)], one, one, LEN),
                             ([dict(kind=orc.TERM_MASS, domain=orc.NEG, hpow=-1, coef=2.0)], one, one,
                              2 * AREA * (7 if D == 2 else 5))]:
        csr, st = orc.quad_assemble(m, l, terms)
        assert st == 0
        A = dense(m.nv, csr)
        assert abs(v @ A @ u - val) < 1e-13, (terms, v @ A @ u, val)
    K = dense(m.nv, orc.quad_assemble(m, l, [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG)])[0])
    assert np.abs(K @ one).max() < 1e-14 and np.abs(K - K.T).max() < 1e-15


def test_nitsche_terms_and_normal():
    """n.grad(x) on the interface of the planar cut is n_x = 1/sqrt(1.25):
    1^T N x = |IF| n_x with N the (grad(u).n) v matrix; U_NGRADV is its
    transpose; CONV with b = (1, 0) gives x^T C 1 = 0 and 1^T C x = |NEG|."""
    m = MakeStructured2DMesh(6, 6, quads=True)
    X, Y = m.coords[:, 0], m.coords[:, 1]
    l = X + 0.5 * Y - 0.6
    one = np.ones(m.nv)
    Nm = dense(m.nv, orc.quad_assemble(m, l, [dict(kind=orc.TERM_NGRADU_V, domain=orc.IF)])[0])
    Nt = dense(m.nv, orc.quad_assemble(m, l, [dict(kind=orc.TERM_U_NGRADV, domain=orc.IF)])[0])
    assert abs(one @ Nm @ X - LEN / LEN) < 1e-13
    assert np.abs(Nm - Nt.T).max() < 1e-15
    C = dense(m.nv, orc.quad_assemble(m, l, [dict(kind=orc.TERM_CONV, domain=orc.NEG, b=(1.0, 0.0, 0.0))])[0])
    assert abs(one @ C @ X - AREA) < 1e-13 and abs(X @ C @ one) < 1e-15

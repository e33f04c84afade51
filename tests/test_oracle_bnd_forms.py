"""Boundary terms of bilinear forms (u * v * dCut(lset, dt, vb=BND)) in the
oracle (orc_assemble_bnd) against closed forms: ngsxfem's
tests/pytests/test_bndcut.py::test_bfi_assembly_2d (on a boundary side that
is all NEG, dCut equals the plain boundary mass matrix of that side) and the
measures and first moments of the NEG / POS / IF parts of the boundary of a
square and a cube cut by a plane (1^T A 1 and x^T A 1 with the vertex
coefficients, which represent 1 and x exactly at every order).  CPU only."""
import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh


def dense(sp, csr):
    rp, cols, vals = csr
    A = np.zeros((sp.ndof, sp.ndof))
    rows = np.repeat(np.arange(sp.ndof), np.diff(rp))
    np.add.at(A, (rows, cols), vals)
    return A


def vertex_vec(sp, nv, vals):
    u = np.zeros(sp.ndof)
    u[:nv] = vals
    return u


def words(mask):
    mask = np.asarray(mask, dtype=bool)
    w = np.zeros((len(mask) + 63) // 64, dtype=np.uint64)
    for i in np.nonzero(mask)[0]:
        w[i >> 6] |= np.uint64(1) << np.uint64(i & 63)
    return w


def test_left_side_equals_boundary_mass(orc):
    """test_bfi_assembly_2d: cut x = 0.4, NEG on the left side, which lies in
    NEG; A u equals the P1 mass matrix of the left side's segments times u."""
    m = MakeStructured2DMesh(9, 9)
    X, Y = m.coords.T
    sp = orc.Space(m, 1)
    l = X - 0.4
    A = dense(sp, sp.assemble(l, [], bterms=[dict(domain=orc.NEG, defined_on=words(m.Boundaries("left").Mask()))]))
    u = np.sin(X) * np.cos(Y)
    left = np.nonzero(X == 0.0)[0]
    left = left[np.argsort(Y[left])]
    B = np.zeros((m.nv, m.nv))
    for a, b in zip(left[:-1], left[1:]):
        h = Y[b] - Y[a]
        B[np.ix_([a, b], [a, b])] += h / 6 * np.array([[2.0, 1.0], [1.0, 2.0]])
    assert np.abs(A @ u - B @ u).max() < 1e-14


@pytest.mark.parametrize("k", [1, 2, 3])
def test_square_boundary_measures(orc, k):
    """x + y/2 = 0.6 on the unit square: NEG boundary length 1.7 (bottom 0.6,
    left 1, top 0.1), first moment in x 0.185; POS the rest of the perimeter;
    IF the points (0.6, 0) and (0.1, 1).  hpow = -1 divides by the owner's
    h = 1/9; definedon restricts to the bottom side."""
    m = MakeStructured2DMesh(9, 9)
    X, Y = m.coords.T
    sp = orc.Space(m, k)
    l = X + 0.5 * Y - 0.6
    one, x = vertex_vec(sp, m.nv, 1.0), vertex_vec(sp, m.nv, X)
    cases = [(dict(domain=orc.NEG), 1.7, 0.185), (dict(domain=orc.POS), 2.3, 2.0 - 0.185),
             (dict(domain=orc.IF, order=0), 2.0, 0.7), (dict(domain=orc.NEG, hpow=-1, coef=2.0), 2 * 9 * 1.7, 2 * 9 * 0.185),
             (dict(domain=orc.NEG, defined_on=words(m.Boundaries("bottom").Mask())), 0.6, 0.18)]
    for bt, meas, mx in cases:
        A = dense(sp, sp.assemble(l, [], bterms=[bt]))
        assert abs(one @ A @ one - meas) < 1e-12 * max(1, meas), bt
        assert abs(x @ A @ one - mx) < 1e-12 * max(1, meas), bt
        assert np.abs(A - A.T).max() < 1e-15 * np.abs(A).max()


@pytest.mark.parametrize("k", [1, 2])
def test_cube_boundary_measures(orc, k):
    """x + y/2 = 0.6 on the unit cube: NEG boundary area 2.4, first moment in
    x 0.328333...; POS the rest of the surface (6)."""
    m = MakeStructured3DMesh(4)
    X = m.coords[:, 0]
    sp = orc.Space(m, k)
    l = X + 0.5 * m.coords[:, 1] - 0.6
    one, x = vertex_vec(sp, m.nv, 1.0), vertex_vec(sp, m.nv, X)
    mx_neg = 2 * 0.5 * (0.36 - 0.3 + 0.25 / 3) + 0.18 + 0.005
    for bt, meas, mx in [(dict(domain=orc.NEG), 2.4, mx_neg), (dict(domain=orc.POS), 3.6, 3.0 - mx_neg)]:
        A = dense(sp, sp.assemble(l, [], bterms=[bt]))
        assert abs(one @ A @ one - meas) < 1e-12 * meas, bt
        assert abs(x @ A @ one - mx) < 1e-12 * meas, bt


@pytest.mark.parametrize("D,k", [(2, 2), (3, 1)])
def test_volume_plus_boundary_is_the_sum(orc, D, k):
    """The matrix of volume + boundary terms is the sum of the two forms' (the
    owners of BND elements join the active elements)."""
    m = MakeStructured2DMesh(7, 7) if D == 2 else MakeStructured3DMesh(3)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.3) ** 2).sum(axis=1) - 0.36)
    sp = orc.Space(m, k)
    dom, _, bits = sp.cutinfo(l)
    vol = [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, defined_on=bits[5])]  # HASNEG
    bt = [dict(domain=orc.NEG, coef=10.0, hpow=-1), dict(domain=orc.POS, coef=0.5)]
    A = dense(sp, sp.assemble(l, vol, bterms=bt))
    B = dense(sp, sp.assemble(l, vol)) + dense(sp, sp.assemble(l, [], bterms=bt))
    assert np.abs(A - B).max() < 1e-12 * np.abs(A).max()

"""Volume terms with a coefficient field (gf * u * v * dCut, gf * grad(u) *
grad(v) * dCut, x^e factors) in the oracle (orc_assemble_full) against
closed forms on the planar cut x + y/2 = 0.6 of the unit square: the NEG part
has area 0.35, first moment in x 0.0716666..., second 0.0215833...; the
interface runs from (0.6, 0) to (0.1, 1).  With the vertex coefficients of 1
and x (exact at every order) 1^T A 1 and x^T A 1 are these integrals.  A
coefficient field equal to 1 gives the plain terms.  CPU only."""
import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

AREA, MX, MXX = 0.35, 0.5 * (0.36 - 0.3 + 0.25 / 3), (0.6 ** 4 - 0.1 ** 4) / 6
LEN = np.sqrt(0.25 + 1.0)


def dense(sp, csr):
    rp, cols, vals = csr
    A = np.zeros((sp.ndof, sp.ndof))
    rows = np.repeat(np.arange(sp.ndof), np.diff(rp))
    np.add.at(A, (rows, cols), vals)
    return A


def field(orc, m, kg, f, fx=None):
    """Element coefficients [ne][nd] of the interpolant of f in the P_kg
    basis: vertex values, for kg = 2 the edge coefficients 4 f(mid) - 2 (f_a +
    f_b) (vertices, then edges (0,1), (0,2), (1,2) / the six tet edges)."""
    el = m.elements
    X = m.coords
    vals = [f(X[el[:, i]]) for i in range(el.shape[1])]
    if kg == 2:
        edges = [(0, 1), (0, 2), (1, 2)] if m.dim == 2 else [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
        for a, b in edges:
            mid = 0.5 * (X[el[:, a]] + X[el[:, b]])
            vals.append(4 * f(mid) - 2 * (vals[a] + vals[b]))
    return np.stack(vals, 1)


@pytest.mark.parametrize("k", [1, 2])
def test_planar_coefficient_integrals(orc, k):
    m = MakeStructured2DMesh(9, 9)
    X, Y = m.coords.T
    sp = orc.Space(m, k)
    l = X + 0.5 * Y - 0.6
    one = np.zeros(sp.ndof)
    one[: m.nv] = 1.0
    x = np.zeros(sp.ndof)
    x[: m.nv] = X
    y = np.zeros(sp.ndof)
    y[: m.nv] = Y
    gx = field(orc, m, 1, lambda p: p[:, 0])
    gxx = field(orc, m, 2, lambda p: p[:, 0] ** 2)
    g1x = field(orc, m, 1, lambda p: 1.0 + p[:, 0])
    M = orc.TERM_MASS
    cases = [
        (dict(kind=M, gf_order=1, gf_el=gx), one, one, MX),
        (dict(kind=M, gf_order=1, gf_el=gx), x, one, MXX),
        (dict(kind=M, e=(1, 0, 0)), one, one, MX),
        (dict(kind=M, e=(2, 0, 0), order=2 * k + 2), one, one, MXX),
        (dict(kind=M, gf_order=2, gf_el=gxx), one, one, MXX),
        (dict(kind=orc.TERM_LAPLACE, gf_order=1, gf_el=g1x, order=2), x, x, AREA + MX),
        (dict(kind=M, domain=orc.IF, gf_order=1, gf_el=gx, order=2), one, one, LEN * 0.35),
        (dict(kind=M, domain=orc.POS, gf_order=1, gf_el=gx), one, one, 0.5 - MX),
        # a component of a vector field: (gx e_0) . grad(x) = x, (gx e_1) . grad(y) = x
        (dict(kind=orc.TERM_CONV, b=(1.0, 0.0, 0.0), gf_order=1, gf_el=gx, order=2), x, one, MX),
        (dict(kind=orc.TERM_CONV, b=(0.0, 1.0, 0.0), gf_order=1, gf_el=gx, order=2), y, one, MX),
        (dict(kind=orc.TERM_CONV, b=(0.0, 1.0, 0.0), gf_order=1, gf_el=gx, order=2), x, one, 0.0),
    ]
    for ct, u, v, val in cases:
        ct = dict(dict(domain=orc.NEG), **ct)
        A = dense(sp, sp.assemble(l, [], cterms=[ct]))
        got = v @ A @ u
        assert abs(got - val) < 1e-13, (ct["kind"], ct.get("e"), ct.get("gf_order"), got, val)


@pytest.mark.parametrize("D,k", [(2, 1), (2, 3), (3, 2)])
def test_unit_field_gives_the_plain_terms(orc, D, k):
    """gf = 1 (P1 interpolant) and e = 0: each kind equals the plain term."""
    m = MakeStructured2DMesh(7, 7) if D == 2 else MakeStructured3DMesh(3)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.3) ** 2).sum(axis=1) - 0.36)
    sp = orc.Space(m, k)
    dom, _, bits = sp.cutinfo(l)
    g1 = field(orc, m, 1, lambda p: np.ones(len(p)))
    b = (0.3, -0.7, 0.2)
    for kind, domain, bi in [(orc.TERM_MASS, orc.NEG, 5), (orc.TERM_LAPLACE, orc.POS, 6),
                             (orc.TERM_NGRADU_V, orc.IF, 4), (orc.TERM_U_NGRADV, orc.IF, 4),
                             (orc.TERM_CONV, orc.NEG, 5)]:
        t = dict(kind=kind, domain=domain, coef=1.7, hpow=-1, b=b, defined_on=bits[bi])
        A = dense(sp, sp.assemble(l, [t]))
        B = dense(sp, sp.assemble(l, [], cterms=[dict(t, gf_order=1, gf_el=g1)]))
        assert np.abs(A - B).max() < 1e-13 * np.abs(A).max(), kind


@pytest.mark.parametrize("k", [1, 2])
def test_planar_normal_and_whole_element_terms(orc, k):
    """The TraceFEM terms on the planar cut (n = (1, 1/2) / sqrt(1.25)):
    (n . grad x)^2 over NEG = 0.35 * 0.8, n_x n_y over the interface =
    0.4 * |IF|, the tangential Laplacian (Laplace - normal-normal) of x over
    the interface = (1 - 0.8) |IF|; whole elements (dx): the mass of the
    interface elements is their area, without a set the square's."""
    m = MakeStructured2DMesh(9, 9)
    X, Y = m.coords.T
    sp = orc.Space(m, k)
    l = X + 0.5 * Y - 0.6
    one, x, y = np.zeros(sp.ndof), np.zeros(sp.ndof), np.zeros(sp.ndof)
    one[: m.nv], x[: m.nv], y[: m.nv] = 1.0, X, Y
    NN = orc.TERM_NGRADU_NGRADV
    A = dense(sp, sp.assemble(l, [], cterms=[dict(kind=NN, domain=orc.NEG)]))
    assert abs(x @ A @ x - 0.35 * 0.8) < 1e-13
    B = dense(sp, sp.assemble(l, [], cterms=[dict(kind=NN, domain=orc.IF)]))
    assert abs(x @ B @ y - 0.4 * LEN) < 1e-13
    T = dense(sp, sp.assemble(l, [], cterms=[dict(kind=orc.TERM_LAPLACE, domain=orc.IF),
                                             dict(kind=NN, domain=orc.IF, coef=-1.0)]))
    assert abs(x @ T @ x - 0.2 * LEN) < 1e-13
    dom, _, bits = sp.cutinfo(l)
    n_if = int(np.sum(np.asarray(dom) == orc.IF))
    W = dense(sp, sp.assemble(l, [], cterms=[dict(kind=orc.TERM_MASS, domain=orc.WHOLE, defined_on=bits[4])]))
    assert abs(one @ W @ one - n_if / 162.0) < 1e-13
    W1 = dense(sp, sp.assemble(l, [], cterms=[dict(kind=orc.TERM_MASS, domain=orc.WHOLE)]))
    assert abs(one @ W1 @ one - 1.0) < 1e-13
    # the normal-normal term on whole elements: (n . grad x)^2 = 0.8 over them
    Wn = dense(sp, sp.assemble(l, [], cterms=[dict(kind=NN, domain=orc.WHOLE, defined_on=bits[4])]))
    assert abs(x @ Wn @ x - 0.8 * n_if / 162.0) < 1e-13

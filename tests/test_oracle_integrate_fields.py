"""Integrate of polynomials in GridFunctions and x, y, z in the oracle
(orc_integrate_fields): the reference's Integrate with a CoefficientFunction
of GridFunctions evaluated at the points of the straight cut rule
(cutint/cutintegral.cpp:126-212), e.g. the L2 error (gfu - gfex)^2 of its
demos.  Pinned on the planar cut x + y/2 = 0.6 of the unit square (NEG area
0.35, first moment 0.0716666..., second 0.0215833..., the interface from
(0.6, 0) to (0.1, 1)) with fields that interpolate x and x^2 exactly, and on
the oracle's own mass matrices: the integral of f_a f_b equals a^T M b.
CPU only."""
import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh
from oracle import oracle as orc

MX, MXX = 0.5 * (0.36 - 0.3 + 0.25 / 3), (0.6 ** 4 - 0.1 ** 4) / 6
LEN = np.sqrt(1.25)


def field(m, kg, f):
    """Element coefficients [ne][nd] of the P_kg interpolant of f (kg 1, 2)."""
    el, X = m.elements, m.coords
    vals = [f(X[el[:, i]]) for i in range(el.shape[1])]
    if kg == 2:
        edges = [(0, 1), (0, 2), (1, 2)] if m.dim == 2 else [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
        for a, b in edges:
            vals.append(4 * f(0.5 * (X[el[:, a]] + X[el[:, b]])) - 2 * (vals[a] + vals[b]))
    return np.stack(vals, 1)


def test_planar_field_integrals():
    m = MakeStructured2DMesh(9, 9)
    X, Y = m.coords.T
    sp = orc.Space(m, 1)
    l = X + 0.5 * Y - 0.6
    gx = (1, field(m, 1, lambda p: p[:, 0]))
    gxx = (2, field(m, 2, lambda p: p[:, 0] ** 2))
    z = (0, 0, 0)
    cases = [
        (orc.NEG, [gx], [(1.0, z, 0, -1)], MX),
        (orc.NEG, [gx], [(1.0, z, 0, 0)], MXX),
        (orc.NEG, [gxx], [(1.0, z, 0, -1)], MXX),
        (orc.NEG, [gx], [(1.0, (1, 0, 0), 0, -1)], MXX),
        (orc.NEG, [gx, gxx], [(1.0, z, 0, 0), (-1.0, z, 1, -1)], 0.0),  # (x^2 - x^2)
        (orc.NEG, [gx], [(2.0, z, -1, -1)], 0.7),  # constants only: 2 * area
        (orc.POS, [gx], [(1.0, z, 0, -1)], 0.5 - MX),
        (orc.IF, [gx], [(1.0, z, 0, -1)], LEN * 0.35),
    ]
    for dt, fields, monos, val in cases:
        got = sp.integrate_fields(l, dt, 4, fields, monos)
        assert abs(got - val) < 1e-13, (dt, monos, got, val)


@pytest.mark.parametrize("D,k", [(2, 1), (2, 3), (3, 2)])
def test_products_are_the_mass_matrix(D, k):
    """int_dt f_a f_b = a^T M_dt b with M the mass matrix on dt (order 2k)."""
    m = MakeStructured2DMesh(7, 7) if D == 2 else MakeStructured3DMesh(3)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.3) ** 2).sum(axis=1) - 0.36)
    sp = orc.Space(m, k)
    rng = np.random.default_rng(5)
    a, b = rng.standard_normal(sp.ndof), rng.standard_normal(sp.ndof)
    ed = sp.el_dofs()
    for dt in (orc.NEG, orc.POS, orc.IF):
        rp, cols, vals = sp.assemble(l, [dict(kind=orc.TERM_MASS, domain=dt, order=2 * k)])
        M = np.zeros((sp.ndof, sp.ndof))
        np.add.at(M, (np.repeat(np.arange(sp.ndof), np.diff(rp)), cols), vals)
        got = sp.integrate_fields(l, dt, 2 * k, [(k, a[ed]), (k, b[ed])], [(1.0, (0, 0, 0), 0, 1)])
        ref = a @ M @ b
        assert abs(got - ref) < 1e-12 * np.abs(M).sum(), (dt, got, ref)
        # (a - b)^2 = a a - 2 a b + b b
        sq = sp.integrate_fields(l, dt, 2 * k, [(k, a[ed]), (k, b[ed])],
                                 [(1.0, (0, 0, 0), 0, 0), (-2.0, (0, 0, 0), 0, 1), (1.0, (0, 0, 0), 1, 1)])
        assert abs(sq - (a - b) @ M @ (a - b)) < 1e-12 * np.abs(M).sum()


def test_planar_derivative_integrals():
    """d/dx of the field x is 1: int_NEG |grad x|^2 = int_NEG d_x x = the area,
    int_NEG d_y x = 0, int_NEG x d_x(x^2) = 2 int x^2."""
    m = MakeStructured2DMesh(9, 9)
    X, Y = m.coords.T
    sp = orc.Space(m, 1)
    l = X + 0.5 * Y - 0.6
    gx = (1, field(m, 1, lambda p: p[:, 0]))
    gxx = (2, field(m, 2, lambda p: p[:, 0] ** 2))
    z = (0, 0, 0)
    cases = [
        ([gx], [(1.0, z, 0, 0, 0, 0), (1.0, z, 0, 0, 1, 1)], 0.35),
        ([gx], [(1.0, z, 0, -1, 0, -1)], 0.35),
        ([gx], [(1.0, z, 0, -1, 1, -1)], 0.0),
        ([gx, gxx], [(1.0, z, 0, 1, -1, 0)], 2 * MXX),
    ]
    for fields, monos, val in cases:
        got = sp.integrate_fields(l, orc.NEG, 4, fields, monos)
        assert abs(got - val) < 1e-13, (monos, got, val)


@pytest.mark.parametrize("D,k", [(2, 2), (3, 1), (3, 3)])
def test_gradient_products_are_the_stiffness_matrix(D, k):
    """int_dt grad f_a . grad f_b = a^T K_dt b with K the Laplace matrix on dt."""
    m = MakeStructured2DMesh(7, 7) if D == 2 else MakeStructured3DMesh(3)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.3) ** 2).sum(axis=1) - 0.36)
    sp = orc.Space(m, k)
    rng = np.random.default_rng(7)
    a, b = rng.standard_normal(sp.ndof), rng.standard_normal(sp.ndof)
    ed = sp.el_dofs()
    for dt in (orc.NEG, orc.POS, orc.IF):
        rp, cols, vals = sp.assemble(l, [dict(kind=orc.TERM_LAPLACE, domain=dt, order=2 * k)])
        K = np.zeros((sp.ndof, sp.ndof))
        np.add.at(K, (np.repeat(np.arange(sp.ndof), np.diff(rp)), cols), vals)
        got = sp.integrate_fields(l, dt, 2 * k, [(k, a[ed]), (k, b[ed])],
                                  [(1.0, (0, 0, 0), 0, 1, d, d) for d in range(D)])
        assert abs(got - a @ K @ b) < 1e-12 * np.abs(K).sum(), (dt, got, a @ K @ b)


def test_deformed_field_integrals():
    """On the deformed mesh (orc_iso_theta_mesh): a zero deformation gives the
    plain integrals, and the constant field 1 gives the deformed measure of
    orc_iso_integrate_mesh (NEG and IF)."""
    m = MakeStructured2DMesh(8, 8, -1, 1, -1, 1)
    p2 = orc.p2_nodal_values(m, lambda p: np.sqrt(p[..., 0] ** 2 + p[..., 1] ** 2) - 0.5)
    l = np.zeros(m.nv)
    for i in range(3):
        l[m.elements[:, i]] = p2[:, i]
    l = np.where(np.abs(l) < 1e-14, 1e-14, l)
    theta, _ = orc.iso_theta_mesh(m, p2, threshold=0.2)
    sp = orc.Space(m, 2)
    rng = np.random.default_rng(2)
    a = rng.standard_normal(sp.ndof)
    fa = (2, a[sp.el_dofs()])
    one = (1, np.ones((m.ne, 3)))
    z = (0, 0, 0)
    prods = [(1.0, z, 0, 0), (1.0, z, 0, 0, 0, 0), (0.5, (1, 0, 0), 0, -1, 1, -1)]
    for dt in (orc.NEG, orc.IF):
        plain = sp.integrate_fields(l, dt, 4, [fa], prods)
        zero = sp.integrate_fields(l, dt, 4, [fa], prods, theta=np.zeros_like(theta))
        assert abs(plain - zero) < 1e-13 * max(1.0, abs(plain))
        meas, _ = orc.iso_integrate_mesh(m, p2, dt, 4, threshold=0.2)
        got = sp.integrate_fields(l, dt, 4, [one], [(1.0, z, 0, -1)], theta=theta)
        assert abs(got - meas) < 1e-13, (dt, got, meas)

"""The oracle against the closed-form answers ngsxfem's own tests assert
(tests/golden/known_answers.json, from tests/pytests/test_straightcutrule.py)
and against basis-invariant checks of its assembled matrices.  CPU only."""
import json
import math
import os

import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

KA = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "known_answers.json")))


def lset_on(mesh, coef, orc):
    c = mesh.coords
    v = coef[0] + sum(coef[k + 1] * c[:, k] for k in range(mesh.dim))
    return orc.interpolate_p1_perturb(v)


@pytest.mark.parametrize("N", KA["planar2d"]["N"])
@pytest.mark.parametrize("order", KA["planar2d"]["orders"])
def test_planar_2d(orc, N, order):
    m = MakeStructured2DMesh(N, N)
    sp = orc.Space(m, 1)
    l = lset_on(m, KA["planar2d"]["lset"], orc)
    for name, dt in (("NEG", orc.NEG), ("POS", orc.POS), ("IF", orc.IF)):
        val = sp.integrate(l, dt, order)
        assert abs(val - KA["planar2d"]["values"][name]) < 5e-15 * (order + 1) ** 2


@pytest.mark.parametrize("order", KA["planar3d"]["orders"])
def test_planar_3d(orc, order):
    m = MakeStructured3DMesh(1)
    sp = orc.Space(m, 1)
    l = lset_on(m, KA["planar3d"]["lset"], orc)
    for name, dt in (("NEG", orc.NEG), ("POS", orc.POS), ("IF", orc.IF)):
        assert abs(sp.integrate(l, dt, order) - KA["planar3d"]["values"][name]) < 5e-15 * (order + 1) ** 2


@pytest.mark.parametrize("order", [2, 4, 8])
@pytest.mark.parametrize("dim", [0, 1])
def test_monomials_2d(orc, order, dim):
    m = MakeStructured2DMesh(1, 1)
    sp = orc.Space(m, 1)
    l = lset_on(m, KA["planar2d"]["lset"], orc)
    for ref in KA["mono2d"]:
        e = [0, 0, 0]
        e[dim] = ref["alpha"]
        for name, dt in (("POS", orc.POS), ("NEG", orc.NEG)):
            assert abs(sp.integrate(l, dt, order, *e) - ref[name]) < 5e-15 * (order + 1) ** 2


@pytest.mark.parametrize("dim", [0, 1, 2])
def test_monomials_3d(orc, dim):
    m = MakeStructured3DMesh(1)
    sp = orc.Space(m, 1)
    l = lset_on(m, KA["planar3d"]["lset"], orc)
    for ref in KA["mono3d"]:
        e = [0, 0, 0]
        e[dim] = ref["alpha"]
        for name, dt in (("POS", orc.POS), ("NEG", orc.NEG)):
            assert abs(sp.integrate(l, dt, 4, *e) - ref[name]) < 5e-15 * 25


@pytest.mark.parametrize("eps", KA["orth2d"]["eps"])
@pytest.mark.parametrize("axis", [0, 1])
def test_orthogonal_eps_cut(orc, eps, axis):
    m = MakeStructured2DMesh(1, 1)
    sp = orc.Space(m, 1)
    c = m.coords
    if axis == 0:
        v = 1 - 2 * c[:, 0] + eps * (c[:, 1] - 0.5)
    else:
        v = 1 - 2 * c[:, 1] + eps * (c[:, 0] - 0.5)
    l = orc.interpolate_p1_perturb(v)
    assert abs(sp.integrate(l, orc.NEG, 2) - 0.5) < 5e-15 * 9
    assert abs(sp.integrate(l, orc.POS, 2) - 0.5) < 5e-15 * 9
    assert abs(sp.integrate(l, orc.IF, 2) - math.sqrt(1 + eps * eps / 4)) < 5e-15 * 9


@pytest.mark.parametrize("dt", ["NEG", "POS", "IF"])
def test_circle_eoc(orc, dt):
    r = KA["circle_eoc"]["r"]
    errs = []
    for i in range(7):
        m = MakeStructured2DMesh(2 ** i, 2 ** i)
        sp = orc.Space(m, 1)
        l = orc.interpolate_p1_perturb(np.sqrt(m.coords[:, 0] ** 2 + m.coords[:, 1] ** 2) - r)
        errs.append(abs(sp.integrate(l, getattr(orc, dt), 2) - KA["circle_eoc"][dt]))
    eoc = [math.log(errs[i + 1] / errs[i]) / math.log(0.5) for i in range(len(errs) - 1)]
    assert np.mean(eoc[1:]) > KA["circle_eoc"]["min_mean_eoc"]


def test_check_if_straight_cut(orc):
    # straightcutrule.cpp:11-24: both signs or all zero -> IF
    assert orc.check_if_straight_cut([1, -1, 2]) == orc.IF
    assert orc.check_if_straight_cut([0, 0, 0]) == orc.IF
    assert orc.check_if_straight_cut([0, 1, 2]) == orc.POS
    assert orc.check_if_straight_cut([0, -1, -2]) == orc.NEG
    assert orc.check_if_straight_cut([-0.0, 1, 1]) == orc.POS


def test_exact_zero_vertex_raises(orc):
    # a vertex value exactly 0 next to a negative vertex makes the reference throw
    # ("You tried to cut a simplex with a plain geometry", straightcutrule.cpp:43-48)
    elc = np.array([[1.0, 0.0], [0.0, 1.0], [0.0, 0.0]])
    with pytest.raises(RuntimeError):
        orc.straight_cut_rule(elc, [0.0, -1.0, 1.0], orc.NEG, 2)


def test_quadrature_exactness(orc):
    from math import factorial
    for d in (1, 2, 3):
        for p in range(0, 9):
            pts, w = orc.base_rule(d, p)
            for a in range(p + 1):
                for b in range(p + 1 - a if d >= 2 else 1):
                    for c in range(p + 1 - a - b if d >= 3 else 1):
                        val = np.sum(w * pts[:, 0] ** a * pts[:, 1] ** b * pts[:, 2] ** c)
                        exact = factorial(a) * factorial(b) * factorial(c) / factorial(a + b + c + d)
                        assert abs(val - exact) < 2e-15, (d, p, a, b, c)


def p2_interp(mesh, sp, f):
    """Hierarchical coefficients of a quadratic polynomial f: vertex values,
    quadratic edge dof = 4 * (f(mid) - (f(s)+f(e))/2) (lambda_s*lambda_e = 1/4 at
    the midpoint); cubic edge and bubble dofs vanish."""
    ed = sp.el_dofs()
    km = sp.order - 1
    nv = mesh.nv
    coef = np.zeros(sp.ndof)
    coef[:nv] = f(*[mesh.coords[:, k] for k in range(mesh.dim)])
    D = mesh.dim
    edges = [(0, 1), (0, 2), (1, 2)] if D == 2 else [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    for e in range(mesh.ne):
        for j, (a, b) in enumerate(edges):
            va, vb = mesh.elements[e, a], mesh.elements[e, b]
            mid = 0.5 * (mesh.coords[va] + mesh.coords[vb])
            fm = f(*mid)
            coef[ed[e, D + 1 + j * km]] = 4 * (fm - 0.5 * (coef[va] + coef[vb]))
    return coef


def csr_apply(rp, cols, vals, x):
    y = np.zeros(len(rp) - 1)
    for r in range(len(rp) - 1):
        y[r] = np.dot(vals[rp[r]:rp[r + 1]], x[cols[rp[r]:rp[r + 1]]])
    return y


@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("N", [1, 6])
def test_matrix_basis_invariants_2d(orc, order, N):
    """v^T A u on the planar cut against the reference's closed forms:
    1^T M 1 = |NEG| = 7/8, x^T K x = |NEG|, 1^T M_IF 1 = 1/sqrt(2), 1^T M x^2-interp."""
    m = MakeStructured2DMesh(N, N)
    sp = orc.Space(m, order)
    l = lset_on(m, KA["planar2d"]["lset"], orc)
    one = np.zeros(sp.ndof)
    one[: m.nv] = 1
    xs = np.zeros(sp.ndof)
    xs[: m.nv] = m.coords[:, 0]
    M = sp.assemble(l, [dict(kind=orc.TERM_MASS, domain=orc.NEG)])
    K = sp.assemble(l, [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG)])
    S = sp.assemble(l, [dict(kind=orc.TERM_MASS, domain=orc.IF)])
    assert abs(one @ csr_apply(*M, one) - 7 / 8) < 1e-13
    assert abs(xs @ csr_apply(*K, xs) - 7 / 8) < 1e-13
    assert abs(one @ csr_apply(*S, one) - 1 / math.sqrt(2)) < 1e-13
    if order >= 2:
        x2 = p2_interp(m, sp, lambda X, Y: X * X)
        ref = 1 / 3 - KA["mono2d"][2]["POS"]
        assert abs(one @ csr_apply(*M, x2) - ref) < 1e-13


@pytest.mark.parametrize("order", [1, 2])
def test_matrix_basis_invariants_3d(orc, order):
    m = MakeStructured3DMesh(2)
    sp = orc.Space(m, order)
    l = lset_on(m, KA["planar3d"]["lset"], orc)
    one = np.zeros(sp.ndof)
    one[: m.nv] = 1
    ys = np.zeros(sp.ndof)
    ys[: m.nv] = m.coords[:, 1]
    M = sp.assemble(l, [dict(kind=orc.TERM_MASS, domain=orc.POS)])
    K = sp.assemble(l, [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG)])
    S = sp.assemble(l, [dict(kind=orc.TERM_MASS, domain=orc.IF)])
    assert abs(one @ csr_apply(*M, one) - 1 / 48) < 1e-14
    assert abs(ys @ csr_apply(*K, ys) - 47 / 48) < 1e-13
    assert abs(one @ csr_apply(*S, one) - math.sqrt(3) / 8) < 1e-13


def test_ghost_penalty_kills_global_polynomials(orc):
    """The facet-patch jump (u - u.Other()) vanishes for a global polynomial of
    degree <= k, so G p = 0 for its interpolant."""
    m = MakeStructured2DMesh(4, 4)
    sp = orc.Space(m, 2)
    l = orc.interpolate_p1_perturb(np.sqrt((m.coords[:, 0] - .5) ** 2 + (m.coords[:, 1] - .5) ** 2) - 0.3)
    G = sp.assemble(l, [dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2)])
    p = p2_interp(m, sp, lambda X, Y: 1 + X - 2 * Y + X * Y + 3 * Y * Y)
    r = csr_apply(*G, p)
    assert np.max(np.abs(r)) < 1e-11 * np.max(np.abs(G[2]))
    # and it is positive semidefinite: random vector energy >= 0
    rng = np.random.default_rng(1)
    for _ in range(3):
        w = rng.standard_normal(sp.ndof)
        assert w @ csr_apply(*G, w) > -1e-12


def test_cutinfo_config1(orc):
    """[-1,1]^2, 40x40x2 triangles, circle r=0.5: area and perimeter within O(h^2)."""
    m = MakeStructured2DMesh(40, 40, -1, 1, -1, 1)
    sp = orc.Space(m, 1)
    l = orc.interpolate_p1_perturb(np.sqrt(m.coords[:, 0] ** 2 + m.coords[:, 1] ** 2) - 0.5)
    dom, ratio, bits = sp.cutinfo(l)
    h = 0.05
    assert abs(sp.integrate(l, orc.NEG, 2) - math.pi * 0.25) < 2 * h * h
    assert abs(sp.integrate(l, orc.IF, 2) - math.pi) < 2 * h * h
    n_if = int((dom == orc.IF).sum())
    assert 100 < n_if < 300
    # uncut elements have ratio exactly 1 (NEG) / 0 (POS); vertices on the circle
    # carry the +1e-14 perturbation, so some cut elements have slivers whose
    # ratio rounds to 1.0
    assert np.all(ratio[dom == orc.NEG] == 1.0) and np.all(ratio[dom == orc.POS] == 0.0)
    assert np.all((ratio[dom == orc.IF] >= 0) & (ratio[dom == orc.IF] <= 1))


@pytest.mark.parametrize("dt,ref", [(0, 7 / 8), (1, 1 / 8), (2, 0.5)])
def test_spacetime_planar_cut(orc, dt, ref):
    """tests/pytests/test_spacetimecutrule.py:41-69: lset 1-2x-2t, P1 in time,
    order 0 in space and time: POS 1/8, NEG 7/8, IF 1/2 to 5e-15."""
    m = MakeStructured2DMesh(1, 1)
    sp = orc.Space(m, 1)
    X = m.coords[:, 0]
    lst = np.stack([orc.interpolate_p1_perturb(1 - 2 * X), orc.interpolate_p1_perturb(-1 - 2 * X)])
    assert abs(sp.integrate_st(lst, 1, dt, 0, 0) - ref) < 5e-15


def test_spacetime_time_basis(orc):
    for kt in (1, 2):
        nodes = [0.0, 1.0] if kt == 1 else [0.0, 0.5, 1.0]
        for i, x in enumerate(nodes):
            psi, _ = orc.time_basis(kt, x)
            assert np.allclose(psi, np.eye(kt + 1)[i])
        # derivative by central differences
        psi_p, _ = orc.time_basis(kt, 0.3 + 1e-6)
        psi_m, _ = orc.time_basis(kt, 0.3 - 1e-6)
        _, dpsi = orc.time_basis(kt, 0.3)
        assert np.allclose((psi_p - psi_m) / 2e-6, dpsi, atol=1e-8)


def test_spacetime_moving_circle(orc):
    """Circle r=0.25 moving on (0.5+0.2cos 2pi t, 0.5+0.2 sin 2pi t), one slab
    dt=1/16 with P2-in-time level set: slab-averaged area and perimeter O(h^2)."""
    m = MakeStructured2DMesh(32, 32)
    sp = orc.Space(m, 1)

    def lsetf(t):
        cx, cy = 0.5 + 0.2 * math.cos(2 * math.pi * t), 0.5 + 0.2 * math.sin(2 * math.pi * t)
        return orc.interpolate_p1_perturb(np.sqrt((m.coords[:, 0] - cx) ** 2 + (m.coords[:, 1] - cy) ** 2) - 0.25)

    dt = 1 / 16
    lst = np.stack([lsetf(0), lsetf(dt / 2), lsetf(dt)])
    h = 1 / 32
    assert abs(sp.integrate_st(lst, 2, orc.NEG, 2, 4) - math.pi * 0.0625) < 2 * h * h
    assert abs(sp.integrate_st(lst, 2, orc.IF, 2, 4) - 2 * math.pi * 0.25) < 2 * h * h


def test_single_cut_triangle_all_orders(orc):
    """tests/pytests/test_localgeom.py: the triangle (0,0),(1,0),(0,1) cut by
    x + y - 1/4 has NEG measure 1/32 and POS measure 1/2 - 1/32 at every rule
    order 0..15, within 5e-16 (p+1)^2."""
    from ngsxfem_gb300.meshes import Mesh
    m = Mesh(np.array([[0.0, 0.0], [1.0, 0.0], [0.0, 1.0]]), np.array([[0, 1, 2]]))
    sp = orc.Space(m, 1)
    l = orc.interpolate_p1_perturb(m.coords[:, 0] + m.coords[:, 1] - 0.25)
    for order in range(16):
        neg, pos = sp.integrate(l, orc.NEG, order), sp.integrate(l, orc.POS, order)
        tol = 5e-16 * (order + 1) ** 2
        assert abs(neg - 1 / 32) < tol and abs(pos - (0.5 - 1 / 32)) < tol and abs(neg + pos - 0.5) < tol

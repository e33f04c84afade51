"""Skeleton terms of the oracle (cut-facet / DG skeleton integrals and the
derivative-jump ghost penalty; oracle/xg_oracle.cpp skel_add): closed-form
facet measures, polynomial reproduction, the H1 / L2 structure, transposes,
and the exact normal derivatives against the reference's central finite
differences (DiffOpDuDnk, xfem/ghostpenalty.cpp:221-365).  CPU only."""
import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

TRI_EDGES = [(0, 1), (0, 2), (1, 2)]
TET_EDGES = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


def poly_coefs(mesh, sp, p, l2):
    """Coefficients of the quadratic polynomial p(x) in the space's basis:
    vertex values, edge coefficients 4 p(mid) - 2 (p_a + p_b) of the
    lambda_s lambda_e functions, 0 for the cubic edge and face functions."""
    D, k = mesh.dim, sp.order
    edges = TRI_EDGES if D == 2 else TET_EDGES
    el_dofs = sp.el_dofs()
    out = np.zeros(sp.ndof)
    for e in range(mesh.ne):
        X = mesh.coords[mesh.elements[e]]
        loc = [p(X[i]) for i in range(D + 1)]
        if k >= 2:
            for a, b in edges:
                loc.append(4 * p(0.5 * (X[a] + X[b])) - 2 * (p(X[a]) + p(X[b])))
                if k == 3:
                    loc.append(0.0)
        loc += [0.0] * (sp.ndof_el - len(loc))
        out[el_dofs[e]] = loc
    return out


def dense(sp, csr):
    rowptr, cols, vals = csr
    A = np.zeros((sp.ndof, sp.ndof))
    for r in range(sp.ndof):
        for q in range(rowptr[r], rowptr[r + 1]):
            A[r, cols[q]] += vals[q]
    return A


def test_cut_facet_measure_2d(orc):
    """Sum of the vertex-vertex block of the jump matrix = |F in NEG| for every
    interior edge; the total over the 9x9 mesh against the closed form for the
    planar cut x = c."""
    n, c = 9, 0.37
    m = MakeStructured2DMesh(n, n)
    sp = orc.Space(m, 1, l2=True)
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - c)
    fe = sp.facet_els()
    total = 0.0
    T = [{"kind": orc.TERM_SKEL_JUMP, "domain": orc.NEG}]
    for f in range(sp.nfacets):
        if fe[f, 1] < 0:
            continue
        M = sp.facet_matrix(l, T, f)
        total += M[:3, :3].sum()
    expect = (n - 1) * c + sum(1 for i in range(1, n) if i / n < c) + np.sqrt(2) * n * c
    assert abs(total - expect) < 1e-12


@pytest.mark.parametrize("D,k", [(2, 1), (2, 2), (2, 3), (3, 1), (3, 2)])
def test_h1_jumps_vanish(orc, D, k):
    """For H1 every assembled jump term is 0: [v] = 0 for continuous v."""
    m = MakeStructured2DMesh(5, 4) if D == 2 else MakeStructured3DMesh(3)
    sp = orc.Space(m, k)
    l = orc.interpolate_p1_perturb(m.coords[:, 0] + 0.3 * m.coords[:, 1] - 0.55)
    for kind in (orc.TERM_SKEL_JUMP, orc.TERM_SKEL_FLUX, orc.TERM_SKEL_FLUX_T):
        for dom in (orc.NEG, orc.POS, orc.WHOLE):
            _, _, vals = sp.assemble(l, [{"kind": kind, "domain": dom, "coef": 1.7}])
            assert np.abs(vals).max() < 1e-13


@pytest.mark.parametrize("D,k", [(2, 1), (2, 2), (2, 3), (3, 1), (3, 2), (3, 3)])
def test_polynomials_have_no_jumps(orc, D, k):
    """A polynomial of the space's degree (quadratic at most) has no jump of
    itself or of its normal derivatives: the jump and DN matrices annihilate
    it, on L2 and H1, whole and cut facets."""
    m = MakeStructured2DMesh(4, 5) if D == 2 else MakeStructured3DMesh(3)
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - 0.2 * m.coords[:, 1] - 0.41)

    def p(x):
        if k == 1:
            return 0.3 + x[0] - 2 * x[1] + (0.5 * x[2] if D == 3 else 0)
        return 0.3 + x[0] - 2 * x[1] + x[0] * x[1] - 1.5 * x[1] ** 2 + (0.7 * x[2] * x[0] if D == 3 else 0)

    for l2 in (True, False):
        sp = orc.Space(m, k, l2=l2)
        u = poly_coefs(m, sp, p, l2)
        kinds = [orc.TERM_SKEL_JUMP] + [orc.TERM_SKEL_DN1 + j for j in range(k)]
        for kind in kinds:
            for dom in (orc.NEG, orc.WHOLE):
                A = dense(sp, sp.assemble(l, [{"kind": kind, "domain": dom, "hpow": -1}]))
                scale = np.abs(A).max() * np.abs(u).max()
                assert scale > 0 or (not l2 and kind == orc.TERM_SKEL_JUMP)
                assert np.abs(A @ u).max() <= 1e-11 * max(scale, 1.0), (l2, kind, dom)


@pytest.mark.parametrize("D,k", [(2, 2), (3, 2), (3, 3)])
def test_flux_transpose_and_symmetry(orc, D, k):
    m = MakeStructured2DMesh(4, 4) if D == 2 else MakeStructured3DMesh(2)
    sp = orc.Space(m, k, l2=True)
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - 0.45)
    fe = sp.facet_els()
    for f in [f for f in range(sp.nfacets) if fe[f, 1] >= 0][:12]:
        F = sp.facet_matrix(l, [{"kind": orc.TERM_SKEL_FLUX, "domain": orc.NEG}], f)
        Ft = sp.facet_matrix(l, [{"kind": orc.TERM_SKEL_FLUX_T, "domain": orc.NEG}], f)
        assert np.abs(F - Ft.T).max() <= 1e-14 * max(np.abs(F).max(), 1.0)
        for kind in [orc.TERM_SKEL_JUMP] + [orc.TERM_SKEL_DN1 + j for j in range(k)]:
            M = sp.facet_matrix(l, [{"kind": kind, "domain": orc.WHOLE}], f)
            assert np.abs(M - M.T).max() <= 1e-13 * max(np.abs(M).max(), 1.0)


def test_fd_stencils(orc):
    """The reference's stencils: the classical fourth-order central formulas."""
    c, e = orc.fd_stencil(1)
    assert np.allclose(c * 12, [1, -8, 0, 8, -1], atol=1e-12)
    c, e = orc.fd_stencil(2)
    assert np.allclose(c * 12, [-1, 16, -30, 16, -1], atol=1e-12)
    c, e = orc.fd_stencil(3)
    assert np.allclose(c * 8, [1, -8, 13, 0, -13, 8, -1], atol=1e-12)
    assert abs(orc.fd_stencil(1)[1] - (5 * np.finfo(float).eps) ** 0.2) < 1e-15


@pytest.mark.parametrize("D,k", [(2, 1), (2, 2), (2, 3), (3, 1), (3, 2), (3, 3)])
def test_exact_normal_derivatives_match_reference_fd(orc, D, k):
    """dn(u, k) of the reference is a central finite difference (accuracy 4;
    the reference documents about 1e-7 in general).  On element polynomials of
    degree <= 3 the fourth-order stencils are exact up to rounding, so the
    exact derivatives match the reference's operator to 1e-8 relative."""
    m = MakeStructured2DMesh(3, 4) if D == 2 else MakeStructured3DMesh(2)
    sp = orc.Space(m, k, l2=True)
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - 0.45)
    fe = sp.facet_els()
    for kd in range(1, k + 1):
        T = [{"kind": orc.TERM_SKEL_DN1 + kd - 1, "domain": orc.WHOLE, "hpow": 2 * kd - 1}]
        worst = 0.0
        for f in [f for f in range(sp.nfacets) if fe[f, 1] >= 0]:
            ex = sp.facet_matrix(l, T, f)
            fd = sp.facet_matrix(l, T, f, dn_fd=True)
            worst = max(worst, np.abs(ex - fd).max() / np.abs(ex).max())
        assert worst < 1e-8, (kd, worst)

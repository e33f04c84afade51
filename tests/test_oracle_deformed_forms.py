"""Bilinear forms on the deformed (isoparametric) mesh in the oracle
(orc_assemble_full with the per-element deformation of orc_iso_theta_mesh):
ngsxfem's P2 workflow `a += ... * dCut(lsetp1, NEG, deformation=deformation)`
(python/lsetcurv.py:281-356, xfem/symboliccutbfi.cpp:76-486 on the deformed
transformation).  Checks: the deformed mass matrix gives the deformed NEG
measure of orc_iso_integrate_mesh (1^T M 1), which converges to the circle's
area at third order (tests/pytests/test_intcurved.py's geometry); the
interface mass gives the circle's perimeter; a zero deformation gives the
undeformed terms.  CPU only."""
import math

import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh
from oracle import oracle as orc


def dense(sp, csr):
    rp, cols, vals = csr
    A = np.zeros((sp.ndof, sp.ndof))
    rows = np.repeat(np.arange(sp.ndof), np.diff(rp))
    np.add.at(A, (rows, cols), vals)
    return A


def circle(N, k):
    m = MakeStructured2DMesh(N, N, -1, 1, -1, 1)
    p2 = orc.p2_nodal_values(m, lambda p: np.sqrt(p[..., 0] ** 2 + p[..., 1] ** 2) - 0.5)
    l = np.zeros(m.nv)
    for i in range(3):
        l[m.elements[:, i]] = p2[:, i]
    l = np.where(np.abs(l) < 1e-14, 1e-14, l)
    theta, _ = orc.iso_theta_mesh(m, p2, threshold=0.2)
    sp = orc.Space(m, k)
    one = np.zeros(sp.ndof)
    one[: m.nv] = 1.0
    return m, p2, l, theta, sp, one


@pytest.mark.parametrize("k", [1, 2])
def test_deformed_mass_is_the_deformed_measure(k):
    errs = []
    for N in (8, 16, 32):
        m, p2, l, theta, sp, one = circle(N, k)
        A = dense(sp, sp.assemble(l, [], cterms=[dict(kind=orc.TERM_MASS, domain=orc.NEG, order=2, theta_el=theta)]))
        meas, _ = orc.iso_integrate_mesh(m, p2, orc.NEG, 2, threshold=0.2)
        assert abs(one @ A @ one - meas) < 1e-13
        errs.append(abs(one @ A @ one - 0.25 * math.pi))
        B = dense(sp, sp.assemble(l, [], cterms=[dict(kind=orc.TERM_MASS, domain=orc.IF, order=2, theta_el=theta)]))
        perim, _ = orc.iso_integrate_mesh(m, p2, orc.IF, 2, threshold=0.2)
        assert abs(one @ B @ one - perim) < 1e-13
    eoc = [math.log2(a / b) for a, b in zip(errs[:-1], errs[1:])]
    assert errs[-1] < 1e-5 and min(eoc) > 2.75, (errs, eoc)


@pytest.mark.parametrize("k", [1, 3])
def test_zero_deformation_gives_the_plain_terms(k):
    m, p2, l, theta, sp, one = circle(8, k)
    dom, _, bits = sp.cutinfo(l)
    zero = np.zeros_like(theta)
    for kind, domain, bi in [(orc.TERM_MASS, orc.NEG, 5), (orc.TERM_LAPLACE, orc.NEG, 5),
                             (orc.TERM_NGRADU_V, orc.IF, 4), (orc.TERM_MASS, orc.IF, 4)]:
        t = dict(kind=kind, domain=domain, coef=1.3, hpow=-1, defined_on=bits[bi])
        A = dense(sp, sp.assemble(l, [], cterms=[t]))
        B = dense(sp, sp.assemble(l, [], cterms=[dict(t, theta_el=zero)]))
        assert np.abs(A - B).max() < 1e-13 * np.abs(A).max(), kind


@pytest.mark.parametrize("k", [1, 2])
def test_deformed_patch(k):
    """dFacetPatch(deformation=...): MapPatchIntegrationPoint on the deformed
    maps.  A zero deformation gives the affine patch matrices; the deformed
    matrices are symmetric, annihilate the constants (u = 1 on both
    elements) and differ from the affine ones."""
    m, p2, l, theta, sp, one = circle(8, k)
    dom, _, bits = sp.cutinfo(l)
    fb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
    gp = [dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2, defined_on=fb)]
    A0 = dense(sp, sp.assemble(l, gp))
    Az = dense(sp, sp.assemble(l, gp, theta_patch=np.zeros_like(theta)))
    Ad = dense(sp, sp.assemble(l, gp, theta_patch=theta))
    scale = np.abs(A0).max()
    assert np.abs(Az - A0).max() < 1e-13 * scale
    assert np.abs(Ad - Ad.T).max() < 1e-14 * scale
    assert np.abs(Ad @ one).max() < 1e-12 * scale
    assert np.abs(Ad - A0).max() > 1e-6 * scale

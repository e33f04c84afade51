"""Integrate of polynomials in GridFunctions and their gradients on the GPU
(xg_integrate_fields, csrc/xg_cform.cu; `Integrate((gfu - gfex) ** 2 *
dCut(lset, NEG), mesh)` and `(grad(gfu) - grad(gfex)) ** 2`, the L2 and H1
errors of the reference's demos, cutint/cutintegral.cpp:126-212) against the
oracle (orc_integrate_fields).  Bar: within 1e-12 of the integral of the
integrand's squared parts; repeated calls bit-identical."""
import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


def gf_of(xg, m, vals):
    g = xg.GridFunction(xg.H1(m, order=1))
    g.vec.copy_(torch.from_numpy(np.ascontiguousarray(vals)))
    return g


def case(xg, orc, D, n):
    m = MakeStructured2DMesh(n, n) if D == 2 else MakeStructured3DMesh(n)
    c = m.coords
    l = orc.interpolate_p1_perturb(((c - 0.3) ** 2).sum(axis=1) - 0.36)
    return m, l, gf_of(xg, m, l)


@pytest.mark.parametrize("D,k,n", [(2, 1, 11), (2, 2, 9), (2, 3, 6), (3, 1, 4), (3, 2, 3)])
def test_error_norm_parity(xg, orc, D, k, n):
    m, l, g = case(xg, orc, D, n)
    V = xg.H1(m, order=k)
    rng = np.random.default_rng(11 + k)
    gfu = xg.GridFunction(V)
    gfu.vec.copy_(torch.from_numpy(rng.standard_normal(V.ndof)))
    if D == 2:
        gfex = xg.GridFunction(xg.H1(m, order=2)).Set(lambda x, y: x * x - 0.5 * y)
    else:
        gfex = xg.GridFunction(xg.H1(m, order=2)).Set(lambda x, y, z: x * z - 0.5 * y)
    sp, sp2 = orc.Space(m, k), orc.Space(m, 2)
    fu = (k, gfu.vec.cpu().numpy()[sp.el_dofs()])
    fe = (2, gfex.vec.cpu().numpy()[sp2.el_dofs()])
    ci = xg.CutInfo(m, g)
    hasneg = ci.GetElementsOfType(xg.HASNEG)
    z = (0, 0, 0)
    for dt in (xg.NEG, xg.POS, xg.IF):
        err = xg.Integrate((gfu - gfex) ** 2 * xg.dCut(g, dt, order=2 * k + 2), m)
        ref = sp.integrate_fields(l, dt, 2 * k + 2, [fu, fe],
                                  [(1.0, z, 0, 0), (-2.0, z, 0, 1), (1.0, z, 1, 1)])
        scale = sp.integrate_fields(l, dt, 2 * k + 2, [fu, fe], [(1.0, z, 0, 0), (1.0, z, 1, 1)])
        assert abs(err - ref) < 1e-12 * scale, (dt, err, ref)
        mom = xg.Integrate(xg.x * gfu * xg.dCut(g, dt, definedonelements=hasneg), m, order=k + 1)
        ref2 = sp.integrate_fields(l, dt, k + 1, [fu], [(1.0, (1, 0, 0), 0, -1)],
                                   defined_on=hasneg.words.cpu().numpy())
        assert abs(mom - ref2) < 1e-12 * max(1.0, abs(ref2)), (dt, mom, ref2)


def test_dict_form_and_determinism(xg, orc):
    """Integrate(levelset_domain={...}, cf=..., mesh=..., order=...) as in the
    demos; the sum is bit-identical over repeated calls."""
    m, l, g = case(xg, orc, 2, 16)
    V = xg.H1(m, order=2)
    gfu = xg.GridFunction(V).Set(lambda x, y: np.sin(3 * x) * y)
    dom = {"levelset": g, "domain_type": xg.NEG}
    a = xg.Integrate(levelset_domain=dom, cf=gfu * gfu, mesh=m, order=6)
    b = xg.Integrate(levelset_domain=dom, cf=gfu ** 2, mesh=m, order=6)
    c = xg.Integrate(gfu * gfu * xg.dCut(g, xg.NEG, order=6), m)
    assert a == b == c
    sp = orc.Space(m, 2)
    ref = sp.integrate_fields(l, xg.NEG, 6, [(2, gfu.vec.cpu().numpy()[sp.el_dofs()])], [(1.0, (0, 0, 0), 0, 0)])
    assert abs(a - ref) < 1e-13 * abs(ref)


@pytest.mark.parametrize("D", [2, 3])
def test_interpolated_polynomials_are_exact(xg, orc, D):
    """Fields that interpolate polynomials exactly (H1 and L2 of order 2):
    the integral equals the monomial Integrate of the same polynomial."""
    m, l, g = case(xg, orc, D, 8 if D == 2 else 4)
    f = (lambda x, y: x * x + 2 * y) if D == 2 else (lambda x, y, z: x * x + 2 * y)
    for space in (xg.H1, xg.L2):
        gf = xg.GridFunction(space(m, order=2)).Set(f)
        for dt in (xg.NEG, xg.IF):
            got = xg.Integrate(gf * xg.dCut(g, dt, order=4), m)
            ref = xg.Integrate(xg.x ** 2 * xg.dCut(g, dt, order=4), m) + 2 * xg.Integrate(xg.y * xg.dCut(g, dt, order=4), m)
            assert abs(got - ref) < 1e-13 * max(1.0, abs(ref)), (space, dt, got, ref)


@pytest.mark.parametrize("D,k,n", [(2, 2, 9), (2, 3, 6), (3, 1, 4), (3, 2, 3)])
def test_h1_error_parity(xg, orc, D, k, n):
    """The H1 error (grad(gfu) - grad(gfex)) ** 2 and grad(gfu) . (f_x, f_y[, f_z])
    against the oracle's derivative products."""
    m, l, g = case(xg, orc, D, n)
    V, V2 = xg.H1(m, order=k), xg.H1(m, order=2)
    rng = np.random.default_rng(3 + k)
    gfu = xg.GridFunction(V)
    gfu.vec.copy_(torch.from_numpy(rng.standard_normal(V.ndof)))
    gfex = xg.GridFunction(V2)
    gfex.vec.copy_(torch.from_numpy(rng.standard_normal(V2.ndof)))
    comps = [xg.GridFunction(xg.H1(m, order=1)) for _ in range(D)]
    for cmp in comps:
        cmp.vec.copy_(torch.from_numpy(rng.standard_normal(m.nv)))
    sp, sp2, sp1 = orc.Space(m, k), orc.Space(m, 2), orc.Space(m, 1)
    fu = (k, gfu.vec.cpu().numpy()[sp.el_dofs()])
    fe = (2, gfex.vec.cpu().numpy()[sp2.el_dofs()])
    fc = [(1, cmp.vec.cpu().numpy()[sp1.el_dofs()]) for cmp in comps]
    z = (0, 0, 0)
    for dt in (xg.NEG, xg.POS, xg.IF):
        q = 2 * k + 2
        err = xg.Integrate((xg.grad(gfu) - xg.grad(gfex)) ** 2 * xg.dCut(g, dt, order=q), m)
        prods = [(c, z, a, b, d, d) for d in range(D) for c, a, b in ((1.0, 0, 0), (-2.0, 0, 1), (1.0, 1, 1))]
        ref = sp.integrate_fields(l, dt, q, [fu, fe], prods)
        scale = sp.integrate_fields(l, dt, q, [fu, fe], [(1.0, z, a, a, d, d) for d in range(D) for a in (0, 1)])
        assert abs(err - ref) < 1e-12 * scale, (dt, err, ref)
        dot = xg.Integrate(xg.grad(gfu) * xg.CoefficientFunction(tuple(comps)) * xg.dCut(g, dt, order=q), m)
        ref2 = sp.integrate_fields(l, dt, q, [fu] + fc, [(1.0, z, 0, 1 + d, d, -1) for d in range(D)])
        scale2 = sp.integrate_fields(l, dt, q, [fu] + fc, [(1.0, z, 0, 0, d, d) for d in range(D)] +
                                     [(1.0, z, 1 + d, 1 + d) for d in range(D)])
        assert abs(dot - ref2) < 1e-12 * scale2, (dt, dot, ref2)


@pytest.mark.parametrize("dt_name", ["NEG", "IF"])
def test_deformed_field_integrals(xg, orc, dt_name):
    """Integrate((gfu) ** 2 * dCut(lsetp1, dt, deformation=...)) and its H1
    part against the oracle on its own deformation (separate Newton
    searches: 1e-10), and the constant field against the monomial Integrate
    on the same deformation (1e-12)."""
    dt = getattr(xg, dt_name)
    m = MakeStructured2DMesh(8, 8, -1, 1, -1, 1)
    phi = lambda x, y: np.sqrt(x * x + y * y) - 0.5  # noqa: E731
    adap = xg.LevelSetMeshAdaptation(m, order=2, threshold=0.2)
    deformation = adap.CalcDeformation(phi)
    lsetp1 = adap.lset_p1
    V = xg.H1(m, order=2)
    rng = np.random.default_rng(4)
    gfu = xg.GridFunction(V)
    gfu.vec.copy_(torch.from_numpy(rng.standard_normal(V.ndof)))
    one = xg.GridFunction(xg.H1(m, order=1)).Set(lambda x, y: np.ones_like(x))
    theta, _ = orc.iso_theta_mesh(m, xg.P2ElementValues(m, phi), threshold=0.2)
    sp = orc.Space(m, 2)
    fa = (2, gfu.vec.cpu().numpy()[sp.el_dofs()])
    l = lsetp1.vec.cpu().numpy()
    z = (0, 0, 0)
    ds = xg.dCut(lsetp1, dt, deformation=deformation, order=4)
    got = xg.Integrate(gfu * gfu * ds, m)
    ref = sp.integrate_fields(l, dt, 4, [fa], [(1.0, z, 0, 0)], theta=theta)
    assert abs(got - ref) < 1e-10 * abs(ref), (got, ref)
    got_h1 = xg.Integrate(xg.grad(gfu) ** 2 * ds, m)
    ref_h1 = sp.integrate_fields(l, dt, 4, [fa], [(1.0, z, 0, 0, d, d) for d in range(2)], theta=theta)
    assert abs(got_h1 - ref_h1) < 1e-10 * abs(ref_h1), (got_h1, ref_h1)
    meas = xg.Integrate(one * ds, m)
    assert abs(meas - xg.Integrate(ds, m)) < 1e-12 * abs(meas)

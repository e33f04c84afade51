"""Linear forms on cut domains (SymbolicCutLinearFormIntegrator,
xfem/symboliccutlfi.cpp:57-180) on the GPU through the C ABI and the Python
LinearForm, against the oracle (within 1e-12 of the largest entry), the
assembled mass matrix (b(u_h) = M u_h) and the cut measure (sum of the P1
vector with f = 1)."""
import ctypes

import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


def cases():
    m2 = MakeStructured2DMesh(18, 15, -1, 1, -1, 1)
    m3 = MakeStructured3DMesh(6, 5, 4)
    rng = np.random.default_rng(12)
    return {
        "circle2d": (m2, np.sqrt((m2.coords ** 2).sum(1)) - 0.6),
        "random3d": (m3, rng.standard_normal(m3.nv) + 0.25),
    }


def lterms(xg, terms, keep):
    arr = (xg._lib.LTerm * len(terms))()
    for k, t in enumerate(terms):
        arr[k].kind, arr[k].domain, arr[k].order, arr[k].coef = t["kind"], t["domain"], t.get("order", -1), t["coef"]
        for j in range(3):
            arr[k].e[j] = t.get("e", (0, 0, 0))[j]
        if t.get("gf") is not None:
            g = torch.from_numpy(t["gf"]).cuda()
            keep.append(g)
            arr[k].d_gf = g.data_ptr()
        else:
            arr[k].d_gf = None
        arr[k].d_defined_on = None
    return arr


@pytest.mark.parametrize("case", ["circle2d", "random3d"])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_linear_form_parity(xg, orc, case, order):
    m, vals = cases()[case]
    l = orc.interpolate_p1_perturb(vals)
    gf = xg.GridFunction(xg.H1(m, 1))
    xg.InterpolateToP1(vals, gf)
    V = xg.H1(m, order=order)
    rng = np.random.default_rng(order)
    uh = rng.standard_normal(V.ndof)
    terms = [dict(kind=0, domain=0, coef=1.5), dict(kind=0, domain=0, coef=-0.5, e=(2, 1, 0)),
             dict(kind=0, domain=2, coef=2.0, e=(0, 1, 1)), dict(kind=1, domain=1, coef=0.75, gf=uh),
             dict(kind=1, domain=2, coef=1.0, gf=uh, order=5)]
    keep = []
    arr = lterms(xg, terms, keep)
    h = ctypes.c_void_p()
    xg._lib.call("xg_lform_create", V.h, arr, len(terms), ctypes.byref(h))
    ci = xg.CutInfo(m, gf)
    out = torch.zeros(V.ndof, dtype=torch.float64, device="cuda")
    xg._lib.call("xg_lform_assemble", h, xg._vp(gf.vec), xg._vp(ci.dom), xg._vp(out), xg._stream())
    torch.cuda.synchronize()
    xg._lib.check(xg._lib.load().xg_lform_check(h), "lform")
    sp = orc.Space(m, order)
    ref = sp.linear_form(l, terms)
    got = out.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    xg._lib.call("xg_lform_destroy", h)


@pytest.mark.parametrize("case", ["circle2d", "random3d"])
def test_linear_form_python_api(xg, orc, case):
    """f += (1 + 2 x) * v * dx and f += u_h * v * dx against the mass matrix
    of a BilinearForm and the P1 measure of the NEG part."""
    m, vals = cases()[case]
    gf = xg.GridFunction(xg.H1(m, 1))
    xg.InterpolateToP1(vals, gf)
    V = xg.H1(m, order=2)
    v, u = V.TestFunction(), V.TrialFunction()
    dx = xg.dCut(gf, xg.NEG)
    uh = xg.GridFunction(V)
    uh.vec.copy_(torch.from_numpy(np.random.default_rng(1).standard_normal(V.ndof)))
    f = xg.LinearForm(V)
    f += uh * v * dx
    f.Assemble()
    a = xg.BilinearForm(V)
    a += u * v * dx
    a.Assemble()
    M = a.mat.to_scipy()
    ref = M @ uh.vec.cpu().numpy()
    got = f.vec.cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))
    # P1: sum of the vector with f = 1 is the measure of the NEG part
    V1 = xg.H1(m, order=1)
    f1 = xg.LinearForm(V1)
    f1 += 1.0 * V1.TestFunction() * dx
    f1.Assemble()
    meas = xg.Integrate(levelset_domain={"levelset": gf, "domain_type": xg.NEG, "order": 2}, mesh=m)
    assert abs(float(f1.vec.sum().item()) - meas) <= 1e-12 * max(1.0, abs(meas))
    f2 = xg.LinearForm(V1)
    f2 += (2.0 * xg.x) * V1.TestFunction() * dx
    f2.Assemble()
    mx = xg.Integrate(levelset_domain={"levelset": gf, "domain_type": xg.NEG, "order": 3}, mesh=m, cf=xg.x)
    assert abs(float(f2.vec.sum().item()) - 2 * mx) <= 1e-12 * max(1.0, abs(mx))


@pytest.mark.parametrize("D,k", [(2, 1), (2, 2), (3, 2)])
def test_source_from_another_space(xg, D, k):
    """A GridFunction source of another space (H1 of order 3, L2 of order 2)
    holding the same polynomial as the form's space gives the same vector
    (its own basis evaluated at the rule's points)."""
    m = MakeStructured2DMesh(9, 9) if D == 2 else MakeStructured3DMesh(4)
    g = xg.GridFunction(xg.H1(m, order=1))
    xg.InterpolateToP1(((m.coords - 0.4) ** 2).sum(axis=1) - 0.3 ** 2, g)
    poly = (lambda *p: 1.0 + p[0] - 0.5 * p[1]) if k == 1 else (lambda *p: 1.0 + p[0] * p[1] - p[D - 1] ** 2)
    V = xg.H1(m, order=k)
    u, v = V.TnT()
    sources = [xg.GridFunction(V).Set(poly), xg.GridFunction(xg.H1(m, order=3)).Set(poly),
               xg.GridFunction(xg.L2(m, order=2)).Set(poly)]
    for dt in (xg.NEG, xg.IF):
        vecs = []
        for s in sources:
            f = xg.LinearForm(V)
            f += 1.5 * s * v * xg.dCut(g, dt)
            f.Assemble()
            vecs.append(f.vec.cpu().numpy().copy())
        scale = np.abs(vecs[0]).max()
        assert scale > 0
        for w in vecs[1:]:
            assert np.abs(w - vecs[0]).max() < 1e-13 * scale, dt

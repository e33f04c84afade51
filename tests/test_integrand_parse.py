"""The integrand parser of the Python mirror (ngsxfem_gb300/xfem.py), which
maps `integrand * dCut(...)` onto the C ABI's terms, on the CPU: a vector
coefficient with GridFunction components, `CoefficientFunction((b_x, b_y))
* grad(u) * v` (the reference evaluates such a CoefficientFunction at every
point, xfem/symboliccutbfi.cpp:168-194), becomes one convection term per
field component (the unit vector, the component's field and its x^e and
constant factors) plus one plain convection term of the constant
components.  No device work: GridFunctions are placeholders here."""
import pytest

import ngsxfem_gb300.xfem as X


def fields(n):
    return [object.__new__(X.GridFunction) for _ in range(n)]


def parse(cf):
    u, v = X._Expr.atom(("u", False)), X._Expr.atom(("v", False))
    it = X.CoefficientFunction(cf) * X.grad(u) * v * X._Measure("cut", None, X.NEG)
    return it.terms(None)


def test_vector_of_fields_splits_into_components():
    gx, gy = fields(2)
    t = parse((gx, gy, 0.25))
    assert [x["kind"] for x in t] == [X.TERM_CONV] * 3
    assert t[0]["b"] == (0.0, 0.0, 0.25) and t[0]["gf"] is None
    assert t[1]["b"] == (1.0, 0.0, 0.0) and t[1]["gf"] is gx
    assert t[2]["b"] == (0.0, 1.0, 0.0) and t[2]["gf"] is gy


def test_component_factors_are_kept():
    gx, gy = fields(2)
    t = parse((2.0 * gx, X.x * gy))
    assert (t[0]["coef"], t[0]["gf"], t[0]["e"]) == (2.0, gx, (0, 0, 0))
    assert (t[1]["coef"], t[1]["gf"], t[1]["e"]) == (1.0, gy, (1, 0, 0))


def test_constant_vector_is_one_term():
    t = parse((1.0, -2.0))
    assert len(t) == 1 and t[0]["b"] == (1.0, -2.0, 0.0) and t[0]["gf"] is None


def test_vector_components_must_be_scalars():
    u = X._Expr.atom(("u", False))
    with pytest.raises(TypeError):
        X.CoefficientFunction((u, 1.0))


def test_integrate_of_fields_builds_the_products(monkeypatch):
    """Integrate((gfu - gfex) ** 2 * dCut(lset, NEG)) and the dict form with
    x * gfu + 3: the products handed to xg_integrate_fields (merged, fields
    numbered in order of appearance)."""
    import ctypes
    import types

    import torch

    class Space:
        def __init__(self, mesh, order):
            self.mesh, self.order, self.h = mesh, order, ctypes.c_void_p(1)

    mesh = types.SimpleNamespace(dim=2)

    def gf(order):
        g = object.__new__(X.GridFunction)
        g.space, g.vec = Space(mesh, order), torch.zeros(4, dtype=torch.float64)
        return g

    seen = {}
    monkeypatch.setattr(X, "_lset_vec", lambda l: torch.zeros(3, dtype=torch.float64))
    monkeypatch.setattr(X, "device_mesh", lambda m: types.SimpleNamespace(h=ctypes.c_void_p(1), check=lambda: None))
    monkeypatch.setattr(X, "_dev", lambda: "cpu")
    monkeypatch.setattr(X, "_stream", lambda: None)
    monkeypatch.setattr(X._lib, "call", lambda name, *a: seen.update(name=name, a=a))

    def products():
        a = seen["a"]
        return a[2], a[3], a[4], [(a[8][i].coef, tuple(a[8][i].e), a[8][i].f0, a[8][i].f1, a[8][i].d0, a[8][i].d1)
                                  for i in range(a[7])]

    lset, gu, ge = gf(1), gf(2), gf(2)
    X.Integrate((gu - ge) ** 2 * X.dCut(lset, X.NEG, order=4), mesh)
    assert seen["name"] == "xg_integrate_fields"
    z = (0, 0, 0)
    assert products() == (X.NEG, 4, 2, [(1.0, z, 0, 0, -1, -1), (-2.0, z, 0, 1, -1, -1), (1.0, z, 1, 1, -1, -1)])
    X.Integrate(levelset_domain={"levelset": lset, "domain_type": X.IF}, cf=X.x * gu + 3, mesh=mesh, order=3)
    assert products() == (X.IF, 3, 1, [(1.0, (1, 0, 0), 0, -1, -1, -1), (3.0, z, -1, -1, -1, -1)])
    with pytest.raises(NotImplementedError):
        X.Integrate(gu * gu * ge * X.dCut(lset, X.NEG), mesh)
    # the H1 error: (grad gu - grad ge)^2 = sum_d (d_d gu)^2 - 2 d_d gu d_d ge + (d_d ge)^2
    X.Integrate((X.grad(gu) - X.grad(ge)) ** 2 * X.dCut(lset, X.NEG), mesh)
    want = [(c, z, a, b, d, d) for d in (0, 1) for c, a, b in ((1.0, 0, 0), (-2.0, 0, 1), (1.0, 1, 1))]
    assert sorted(products()[3]) == sorted(want)
    # against a vector of fields: grad(gu) . (gx, gy) = gx d_0 gu + gy d_1 gu
    # (fields numbered as they appear: gx 0, gu 1, gy 2)
    gx, gy = gf(1), gf(1)
    X.Integrate(X.grad(gu) * X.CoefficientFunction((gx, gy)) * X.dCut(lset, X.NEG), mesh)
    assert sorted(products()[3]) == sorted([(1.0, z, 0, 1, -1, 0), (1.0, z, 1, 2, 1, -1)])


def test_tracefem_integrands():
    """P(grad u) . P(grad v) with P(w) = w - (w . n) n on the interface: the
    Laplacian, two normal-normal terms with -1 and one with +1 (n . n = 1);
    (grad u . n)(grad v . n) * dx(definedonelements=...) is a whole-element
    normal-normal term."""
    lset = object.__new__(X.GridFunction)
    n = X.Normalize(X.grad(lset))
    u, v = X._Expr.atom(("u", False)), X._Expr.atom(("v", False))

    def P(w):
        return w - (w * n) * n

    t = (P(X.grad(u)) * P(X.grad(v)) * X._Measure("cut", lset, X.IF)).terms(lset)
    got = sorted((x["kind"], x["coef"]) for x in t)
    assert got == sorted([(X.TERM_LAPLACE, 1.0), (X.TERM_NGRADU_NGRADV, -1.0), (X.TERM_NGRADU_NGRADV, -1.0),
                          (X.TERM_NGRADU_NGRADV, 1.0)])
    h = X.specialcf.mesh_size
    t = ((1.0 / h) * (X.grad(u) * n) * (X.grad(v) * n) * X.dx(definedonelements=None)).terms(lset)
    assert [(x["kind"], x["domain"], x["hpow"]) for x in t] == [(X.TERM_NGRADU_NGRADV, X.WHOLE, -1)]

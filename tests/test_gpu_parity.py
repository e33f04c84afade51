"""libxg (GPU, through the C ABI) against the oracle on seeded inputs.

Bars: domain types, counts and bitsets bit-exact; cut ratios bit-exact (the
marking translation unit is built with -fmad=false and the order-0 rules are
exact constants); rule points and weights within 1e-14 (the two sides build
their base rules with different algorithms, Golub-Welsch vs Newton, which may
differ in the last bit; the required bar is 1e-12); assembled FP64 matrices
within 1e-12 relative to the largest entry; mixed precision within 1e-5."""
import ctypes
import math

import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


def circle2d(n=40):
    m = MakeStructured2DMesh(n, n, -1, 1, -1, 1)
    return m, np.sqrt(m.coords[:, 0] ** 2 + m.coords[:, 1] ** 2) - 0.5


def sphere3d(n=10):
    m = MakeStructured3DMesh(n)
    c = m.coords - 0.5
    r = np.sqrt((c ** 2).sum(1))
    return m, r - 0.3 + 0.02 * np.sin(7 * m.coords[:, 0]) * np.sin(7 * m.coords[:, 1]) * np.sin(7 * m.coords[:, 2])


def random_lset(m, seed):
    rng = np.random.default_rng(seed)
    return rng.standard_normal(m.nv) + 0.3


CASES = {
    "circle2d": circle2d,
    "sphere3d": sphere3d,
    "random2d": lambda: (lambda m: (m, random_lset(m, 7)))(MakeStructured2DMesh(12, 9)),
    "random3d": lambda: (lambda m: (m, random_lset(m, 11)))(MakeStructured3DMesh(5, 4, 3)),
}


def setup_case(xg, orc, name):
    m, vals = CASES[name]()
    l = orc.interpolate_p1_perturb(vals)
    V1 = xg.H1(m, order=1)
    gf = xg.GridFunction(V1)
    xg.InterpolateToP1(vals, gf)
    assert np.array_equal(gf.vec.cpu().numpy(), l)
    return m, l, gf


@pytest.mark.parametrize("case", list(CASES))
def test_cutinfo_parity(xg, orc, case):
    m, l, gf = setup_case(xg, orc, case)
    sp = orc.Space(m, 1)
    dom, ratio, bits = sp.cutinfo(l)
    ci = xg.CutInfo(m, gf)
    ci.dm.check()
    assert np.array_equal(ci.dom.cpu().numpy(), dom)
    assert np.array_equal(ci.cut_ratio.cpu().numpy().view(np.uint64), ratio.view(np.uint64))
    assert np.array_equal(ci.bits.cpu().numpy().view(np.uint64), bits)


@pytest.mark.parametrize("case", list(CASES))
def test_facets_parity(xg, orc, case):
    m, l, gf = setup_case(xg, orc, case)
    sp = orc.Space(m, 1)
    dom, ratio, bits = sp.cutinfo(l)
    ci = xg.CutInfo(m, gf)
    assert np.array_equal(xg.device_mesh(m).facet_elements(), sp.facet_els())
    for bnd in (True, False):
        for use_and in (True, False):
            ref = sp.facets_with_neighbor_types(bits[5], bits[4], bnd, bnd, use_and)
            got = xg.GetFacetsWithNeighborTypes(m, a=ci.GetElementsOfType(xg.HASNEG), b=ci.GetElementsOfType(xg.IF),
                                                bnd_val_a=bnd, bnd_val_b=bnd, use_and=use_and)
            assert np.array_equal(got.words.cpu().numpy().view(np.uint64), ref)


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("dt", [0, 1, 2])
@pytest.mark.parametrize("order", [0, 2, 4])
def test_cut_rules_parity(xg, orc, case, dt, order):
    m, l, gf = setup_case(xg, orc, case)
    sp = orc.Space(m, 1)
    dom, _, _ = sp.cutinfo(l)
    els = np.concatenate([np.nonzero(dom == orc.IF)[0][:200], np.nonzero(dom != orc.IF)[0][:50]]).astype(np.int32)
    counts, pts, wts = xg.CutIntegrationRules(m, gf, els, dt, order)
    counts, pts, wts = counts.cpu().numpy(), pts.cpu().numpy(), wts.cpu().numpy()
    for i, e in enumerate(els):
        r = orc.straight_cut_rule(m.coords[m.elements[e]], l[m.elements[e]], dt, order)
        if r is None:
            assert counts[i] == -1
            continue
        p, w = r
        assert counts[i] == len(w)
        assert np.max(np.abs(pts[i, : len(w)] - p)) <= 1e-14, e
        assert np.max(np.abs(wts[i, : len(w)] - w)) <= 1e-14 * max(1e-300, np.max(np.abs(w))), e


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("dt", [0, 1, 2])
def test_integrate_parity(xg, orc, case, dt):
    m, l, gf = setup_case(xg, orc, case)
    sp = orc.Space(m, 1)
    for e in ((0, 0, 0), (1, 0, 0), (0, 2, 1)):
        ref = sp.integrate(l, dt, 4, *e)
        got = xg.Integrate(levelset_domain={"levelset": gf, "domain_type": dt, "order": 4},
                           cf=xg._Monomial(e), mesh=m)
        # summation orders differ (fixed tree on the GPU, sequential on the CPU)
        assert abs(got - ref) <= 1e-12 * max(1.0, abs(ref))


def test_planar_known_answers_gpu(xg):
    for N in (1, 10, 30):
        m = MakeStructured2DMesh(N, N)
        gf = xg.GridFunction(xg.H1(m, 1))
        xg.InterpolateToP1(lambda X, Y: 1 - 2 * X - 2 * Y, gf)
        for dt, ref in ((xg.NEG, 7 / 8), (xg.POS, 1 / 8), (xg.IF, 1 / math.sqrt(2))):
            for order in (2, 4, 8):
                val = xg.Integrate(levelset_domain={"levelset": gf, "domain_type": dt, "order": order}, mesh=m)
                assert abs(val - ref) < 5e-15 * (order + 1) ** 2
    m = MakeStructured3DMesh(1)
    gf = xg.GridFunction(xg.H1(m, 1))
    xg.InterpolateToP1(lambda X, Y, Z: 1 - 2 * X - 2 * Y - 2 * Z, gf)
    for dt, ref in ((xg.NEG, 47 / 48), (xg.POS, 1 / 48), (xg.IF, math.sqrt(3) / 8)):
        val = xg.Integrate(levelset_domain={"levelset": gf, "domain_type": dt, "order": 4}, mesh=m)
        assert abs(val - ref) < 5e-15 * 25


def oracle_pipeline_csr(orc, m, l, order, terms, ghost):
    """CutFEM pipeline on the oracle (CutInfo -> HASNEG/IF sets -> ghost facets -> assembly)."""
    sp = orc.Space(m, order)
    dom, ratio, bits = sp.cutinfo(l)
    fb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
    t2 = []
    for t in terms:
        t = dict(t)
        if t["kind"] == orc.TERM_GHOST_MASS:
            t["defined_on"] = fb
        else:
            t["defined_on"] = {orc.NEG: bits[5], orc.IF: bits[4], orc.POS: bits[6]}[t["domain"]]
        t2.append(t)
    return sp, sp.assemble(l, t2)


def to_dense_global(rp, cols, vals, n):
    A = np.zeros((n, n))
    for r in range(n):
        A[r, cols[rp[r]:rp[r + 1]]] += vals[rp[r]:rp[r + 1]]
    return A


def xg_terms_form(xg, space, terms, prec):
    arr = (xg._lib.Term * len(terms))()
    for k, t in enumerate(terms):
        arr[k].kind, arr[k].domain = t["kind"], t.get("domain", 0)
        arr[k].order, arr[k].hpow, arr[k].coef = t.get("order", -1), t.get("hpow", 0), t.get("coef", 1.0)
        for j in range(3):
            arr[k].b[j] = t.get("b", (0, 0, 0))[j]
        arr[k].d_defined_on = None
    h = ctypes.c_void_p()
    xg._lib.call("xg_form_create", space.h, arr, len(terms), prec, ctypes.byref(h))
    return h


def run_cutfem_step(xg, space, gf, terms, prec):
    form = xg_terms_form(xg, space, terms, prec)
    cap = np.zeros(2, dtype=np.int64)
    xg._lib.call("xg_form_capacity", form, cap.ctypes.data_as(ctypes.c_void_p))
    bf = xg.BilinearForm(space)
    bf._alloc(int(cap[0]), int(cap[1]))
    xg._lib.call("xg_cutfem_step", form, xg._vp(gf.vec), ctypes.byref(bf._csr), xg._stream())
    torch.cuda.synchronize()
    xg._lib.check(xg._lib.load().xg_form_check(form), "form")
    nrows, nnz = (int(v) for v in bf._counts.cpu().tolist())
    mat = xg.SparseMatrix(space.ndof, bf._row_dof, bf._rowptr, bf._cols, bf._vals, nrows, nnz)
    xg._lib.load().xg_form_destroy(form)
    return mat


FORMS = {
    # config-1 shape: mass + stiffness on NEG (orders 2 and 0), interface mass
    "c1": lambda orc: [dict(kind=orc.TERM_MASS, domain=orc.NEG, order=2),
                       dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, order=0),
                       dict(kind=orc.TERM_MASS, domain=orc.IF, order=2)],
    # config-2 shape: NEG stiffness, Nitsche on IF, ghost penalty 0.1/h^2
    "c2": lambda orc: [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG),
                       dict(kind=orc.TERM_NGRADU_V, domain=orc.IF, coef=-1.0),
                       dict(kind=orc.TERM_U_NGRADV, domain=orc.IF, coef=-1.0),
                       dict(kind=orc.TERM_MASS, domain=orc.IF, coef=40.0, hpow=-1),
                       dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2)],
    "conv_pos": lambda orc: [dict(kind=orc.TERM_CONV, domain=orc.POS, b=(1.0, -0.5, 0.25)),
                             dict(kind=orc.TERM_MASS, domain=orc.POS)],
    # a ghost-penalty rule below the integrand degree: the quadrature patch kernel
    "ghost_low": lambda orc: [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG),
                              dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2, order=1)],
}


@pytest.mark.parametrize("case", ["circle2d", "sphere3d", "random2d", "random3d"])
@pytest.mark.parametrize("order", [1, 2, 3])
@pytest.mark.parametrize("form", list(FORMS))
def test_cutfem_step_parity(xg, orc, case, order, form):
    if case == "sphere3d" and order == 3:
        pytest.skip("covered by the random 3D mesh at order 3")
    check_step_parity(xg, orc, case, order, form)


@pytest.mark.parametrize("case,order,form", [("sphere3d", 2, "c2"), ("random2d", 3, "conv_pos"),
                                             ("random3d", 1, "c1")])
def test_cut_workspace_overflow(xg, orc, monkeypatch, case, order, form):
    """Cut elements beyond the per-step moment workspace (capped to 7 elements
    here) take the quadrature-point kernel: the matrix is the same."""
    monkeypatch.setenv("XG_CUT_WORKSPACE", "7")
    check_step_parity(xg, orc, case, order, form)


@pytest.mark.parametrize("case,order,form", [("sphere3d", 2, "c2"), ("random3d", 3, "c2"), ("random2d", 2, "conv_pos"),
                                             ("circle2d", 1, "c1"), ("random3d", 1, "ghost_low")])
def test_direct_row_scatter(xg, orc, monkeypatch, case, order, form):
    """Forms whose full pattern exceeds the compaction scratch budget (here 0
    bytes) count their rows first and sum straight into the output: the same
    matrix, in FP64 and mixed precision."""
    monkeypatch.setenv("XG_ROWS_SCRATCH_BYTES", "0")
    check_step_parity(xg, orc, case, order, form)
    m, l, gf = setup_case(xg, orc, case)
    V = xg.H1(m, order=order)
    a = run_cutfem_step(xg, V, gf, FORMS[form](orc), xg.PREC_FP64)
    b = run_cutfem_step(xg, V, gf, FORMS[form](orc), xg.PREC_MIXED)
    assert a.nnz == b.nnz and torch.equal(a.cols[: a.nnz], b.cols[: b.nnz])
    rel = float((a.vals[: a.nnz] - b.vals[: b.nnz]).abs().max() / a.vals[: a.nnz].abs().max())
    assert rel < 1e-5, rel


def check_step_parity(xg, orc, case, order, form):
    m, l, gf = setup_case(xg, orc, case)
    terms = FORMS[form](orc)
    sp, (rp, cols, vals) = oracle_pipeline_csr(orc, m, l, order, terms, True)
    V = xg.H1(m, order=order)
    assert np.array_equal(V.element_dofs(), sp.el_dofs())
    mat = run_cutfem_step(xg, V, gf, terms, xg.PREC_FP64)
    r, c, v = mat.global_coo()
    ref_rows = np.repeat(np.arange(sp.ndof), np.diff(rp))
    # same pattern and values (within 1e-12 of the largest entry)
    ref = {(int(a), int(b)): float(x) for a, b, x in zip(ref_rows, cols, vals)}
    got = {(int(a), int(b)): float(x) for a, b, x in zip(r, c, v)}
    assert set(ref) == set(got)
    scale = max(1e-300, max(abs(x) for x in ref.values()))
    err = max(abs(got[k] - ref[k]) for k in ref) / scale
    assert err < 1e-12, err
    # rows are the active dofs in ascending order, columns ascending within rows
    rd = mat.row_dof[: mat.nrows].cpu().numpy()
    assert np.all(np.diff(rd) > 0)


@pytest.mark.parametrize("case", ["circle2d", "sphere3d"])
def test_determinism(xg, orc, case):
    m, l, gf = setup_case(xg, orc, case)
    V = xg.H1(m, order=2)
    terms = FORMS["c2"](orc)
    a = run_cutfem_step(xg, V, gf, terms, xg.PREC_FP64)
    v1 = a.vals[: a.nnz].clone()
    b = run_cutfem_step(xg, V, gf, terms, xg.PREC_FP64)
    assert torch.equal(v1, b.vals[: b.nnz])


@pytest.mark.parametrize("case", ["circle2d", "sphere3d", "random3d"])
@pytest.mark.parametrize("order", [1, 2, 3])
def test_mixed_precision(xg, orc, case, order):
    m, l, gf = setup_case(xg, orc, case)
    V = xg.H1(m, order=order)
    terms = FORMS["c2"](orc)
    a = run_cutfem_step(xg, V, gf, terms, xg.PREC_FP64)
    b = run_cutfem_step(xg, V, gf, terms, xg.PREC_MIXED)
    assert a.nnz == b.nnz and torch.equal(a.cols[: a.nnz], b.cols[: b.nnz])
    va, vb = a.vals[: a.nnz], b.vals[: b.nnz]
    rel = float((va - vb).abs().max() / va.abs().max())
    assert rel < 1e-5, rel


def test_python_api_matches_c_abi(xg, orc):
    """fictdom-shaped script through the Python mirror equals the C-ABI step."""
    m, l, gf = setup_case(xg, orc, "sphere3d")
    V = xg.H1(m, order=2)
    ci = xg.CutInfo(m, gf)
    hasneg, hasif = ci.GetElementsOfType(xg.HASNEG), ci.GetElementsOfType(xg.IF)
    ba = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=hasif)
    u, v = V.TnT()
    h = xg.specialcf.mesh_size
    n = xg.Normalize(xg.grad(gf))
    a = xg.BilinearForm(V)
    a += xg.grad(u) * xg.grad(v) * xg.dCut(gf, xg.NEG, definedonelements=hasneg)
    a += -xg.grad(u) * n * v * xg.dCut(gf, xg.IF, definedonelements=hasif)
    a += -xg.grad(v) * n * u * xg.dCut(gf, xg.IF, definedonelements=hasif)
    a += (40.0 / h) * u * v * xg.dCut(gf, xg.IF, definedonelements=hasif)
    a += 0.1 / h ** 2 * (u - u.Other()) * (v - v.Other()) * xg.dFacetPatch(definedonelements=ba)
    a.Assemble(cutinfo=ci)
    b = run_cutfem_step(xg, V, gf, FORMS["c2"](orc), xg.PREC_FP64)
    A1, A2 = a.mat.to_scipy(), b.to_scipy()
    assert abs(A1 - A2).max() <= 1e-14 * abs(A2).max()


def test_no_active_elements(xg, orc):
    m = MakeStructured2DMesh(6, 6)
    gf = xg.GridFunction(xg.H1(m, 1))
    xg.InterpolateToP1(np.ones(m.nv), gf)
    V = xg.H1(m, order=2)
    mat = run_cutfem_step(xg, V, gf, FORMS["c2"](orc), xg.PREC_FP64)
    assert mat.nrows == 0 and mat.nnz == 0


def test_exact_zero_vertex_is_an_error(xg):
    """A vertex value exactly 0 next to a negative vertex: the reference throws
    (straightcutrule.cpp:43-48); libxg reports XG_ERR_PLAIN_CUT."""
    m = MakeStructured2DMesh(1, 1)
    gf = xg.GridFunction(xg.H1(m, 1))
    # vertices p00, p10, p01, p11; triangle (p00, p10, p11) gets (0, -1, 1)
    vals = np.array([0.0, -1.0, 1.0, 1.0])
    gf.vec[: m.nv] = torch.from_numpy(vals)
    ci = xg.CutInfo(m, gf)
    with pytest.raises(xg._lib.XgError) as ei:
        ci.dm.check()
    assert ei.value.status == 4

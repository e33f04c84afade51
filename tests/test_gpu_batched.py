"""Batched steps in one CUDA graph (xg_step_graph_*), on the GPU through the C
ABI: the batched-mesh workload's shape (independent unit-cube meshes of
uneven sizes and orders 1..3 with rotated-ellipsoid level sets, the meshes of
one order joined into one disconnected mesh, the order groups as concurrent
graph branches) against the oracle within 1e-12, the space-time slab batch,
and graph replay against eager steps (bit-identical)."""
import ctypes

import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import (MakeStructured2DMesh, MakeStructured3DMesh, batched_ellipsoids, concatenate,
                                  ellipsoid_values)

pytestmark = pytest.mark.gpu

C2_TERMS = lambda orc, k: [dict(kind=orc.TERM_LAPLACE, domain=orc.NEG),  # noqa: E731
                           dict(kind=orc.TERM_NGRADU_V, domain=orc.IF, coef=-1.0),
                           dict(kind=orc.TERM_U_NGRADV, domain=orc.IF, coef=-1.0),
                           dict(kind=orc.TERM_MASS, domain=orc.IF, coef=10.0 * k * k, hpow=-1),
                           dict(kind=orc.TERM_GHOST_MASS, coef=0.1, hpow=-2)]


def batch_groups(count, max_tets, seed):
    spec = batched_ellipsoids(count, min_tets=1e3, max_tets=max_tets, seed=seed)
    groups = {}
    for n, order, centre, axes, rot in spec:
        m = MakeStructured3DMesh(n)
        g = groups.setdefault(order, ([], []))
        g[0].append(m)
        g[1].append(ellipsoid_values(m.coords, centre, axes, rot))
    return {k: (concatenate(ms), np.concatenate(vs)) for k, (ms, vs) in sorted(groups.items())}


def plain_form(xg, space, terms, prec):
    arr = (xg._lib.Term * len(terms))()
    for k, t in enumerate(terms):
        arr[k].kind, arr[k].domain = t["kind"], t.get("domain", 0)
        arr[k].order, arr[k].hpow, arr[k].coef = -1, t.get("hpow", 0), t.get("coef", 1.0)
        arr[k].d_defined_on = None
    h = ctypes.c_void_p()
    xg._lib.call("xg_form_create", space.h, arr, len(terms), prec, ctypes.byref(h))
    return h


def output(xg, form, ndof):
    cap = np.zeros(2, dtype=np.int64)
    xg._lib.call("xg_form_capacity", form, cap.ctypes.data_as(ctypes.c_void_p))

    class _S:
        pass
    _S.ndof = ndof
    bf = xg.BilinearForm.__new__(xg.BilinearForm)
    bf.space = _S()
    bf._form = None
    bf._alloc(int(cap[0]), int(cap[1]))
    return bf


def coo(xg, bf, ndof):
    nrows, nnz = (int(v) for v in bf._counts.cpu().tolist())
    return xg.SparseMatrix(ndof, bf._row_dof, bf._rowptr, bf._cols, bf._vals, nrows, nnz).global_coo()


def canon(r, c, v):
    o = np.lexsort((c, r))
    return r[o], c[o], v[o]


def graph(xg, forms, lsets, outs):
    n = len(forms)
    f = (ctypes.c_void_p * n)(*[x.value for x in forms])
    l = (ctypes.c_void_p * n)(*[x.data_ptr() for x in lsets])
    o = (xg._lib.Csr * n)(*[b._csr for b in outs])
    g = ctypes.c_void_p()
    xg._lib.call("xg_step_graph_create", f, l, o, n, ctypes.byref(g))
    return g


def oracle_csr(orc, m, l, order, terms):
    sp = orc.Space(m, order)
    dom, _, bits = sp.cutinfo(l)
    fb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
    t2 = []
    for t in terms:
        t = dict(t)
        t["defined_on"] = fb if t["kind"] == orc.TERM_GHOST_MASS else {orc.NEG: bits[5], orc.IF: bits[4]}[t["domain"]]
        t2.append(t)
    rp, cols, vals = sp.assemble(l, t2)
    return sp, np.repeat(np.arange(sp.ndof), np.diff(rp)), cols, vals


@pytest.mark.parametrize("prec", [0, 1])
def test_batched_meshes_one_graph(xg, orc, prec):
    groups = batch_groups(9, 6e3, seed=5)
    assert len(groups) >= 2
    objs, forms, lsets, outs = [], [], [], []
    for order, (m, vals) in groups.items():
        V = xg.H1(m, order=order)
        gf = xg.GridFunction(xg.H1(m, 1))
        xg.InterpolateToP1(vals, gf)
        forms.append(plain_form(xg, V, C2_TERMS(orc, order), prec))
        lsets.append(gf.vec)
        outs.append(output(xg, forms[-1], V.ndof))
        objs.append((m, V, gf, order))
    g = graph(xg, forms, lsets, outs)
    kc = np.zeros(1, dtype=np.int64)
    xg._lib.call("xg_step_graph_kernel_count", g, kc.ctypes.data_as(ctypes.c_void_p))
    assert kc[0] >= 10 * len(forms)
    first = None
    for rep in range(2):  # replays give identical results
        xg._lib.call("xg_step_graph_launch", g, xg._stream())
        torch.cuda.synchronize()
        for f in forms:
            xg._lib.check(xg._lib.load().xg_form_check(f), "graph form")
        res = [coo(xg, b, V.ndof) for b, (_, V, _, _) in zip(outs, objs)]
        if first is None:
            first = res
        else:
            for a, b in zip(first, res):
                assert all(np.array_equal(x, y) for x, y in zip(a, b))
    for (m, V, gf, order), (r, c, v) in zip(objs, first):
        l = gf.vec.cpu().numpy()
        sp, rr, rc, rv = oracle_csr(orc, m, l, order, C2_TERMS(orc, order))
        r, c, v = canon(r, c, v)
        rr, rc, rv = canon(rr, rc, rv)
        assert np.array_equal(V.element_dofs(), sp.el_dofs())
        assert np.array_equal(r, rr) and np.array_equal(c, rc)
        err = np.max(np.abs(v - rv)) / np.max(np.abs(rv))
        assert err < (1e-12 if prec == 0 else 1e-5), (order, err)
        # block diagonal: no entry couples two meshes of the batch
        comp_el = np.repeat(np.arange(len(m.component_element_counts)), m.component_element_counts)
        comp_dof = np.full(V.ndof, -1)
        eld = V.element_dofs()
        comp_dof[eld.ravel()] = np.repeat(comp_el, eld.shape[1])
        assert np.all(comp_dof >= 0)
        assert np.array_equal(comp_dof[r], comp_dof[c])
        assert len(np.unique(comp_dof[r])) > 1
    xg._lib.call("xg_step_graph_destroy", g)
    for f in forms:
        xg._lib.load().xg_form_destroy(f)


def test_graph_matches_eager_and_repeated_form(xg, orc):
    """Two forms on two meshes plus a second entry of the first form with
    another level set and output: the graph reproduces eager steps bit for bit."""
    m1 = MakeStructured2DMesh(20, 17, -1, 1, -1, 1)
    m2 = MakeStructured3DMesh(6, 5, 4)
    rng = np.random.default_rng(3)
    cases = [(m1, np.sqrt((m1.coords ** 2).sum(1)) - 0.5, 2), (m2, rng.standard_normal(m2.nv) + 0.3, 2),
             (m1, np.sqrt(((m1.coords - 0.1) ** 2).sum(1)) - 0.6, 2)]
    spaces, lsets = {}, []
    for m, vals, k in cases:
        gf = xg.GridFunction(xg.H1(m, 1))
        xg.InterpolateToP1(vals, gf)
        lsets.append(gf.vec)
        spaces.setdefault(id(m), xg.H1(m, order=k))
    f1 = plain_form(xg, spaces[id(m1)], C2_TERMS(orc, 2), 0)
    f2 = plain_form(xg, spaces[id(m2)], C2_TERMS(orc, 2), 0)
    forms = [f1, f2, f1]
    nd = [spaces[id(m1)].ndof, spaces[id(m2)].ndof, spaces[id(m1)].ndof]
    eager = []
    for f, l, n in zip(forms, lsets, nd):
        b = output(xg, f, n)
        xg._lib.call("xg_cutfem_step", f, xg._vp(l), ctypes.byref(b._csr), xg._stream())
        torch.cuda.synchronize()
        xg._lib.check(xg._lib.load().xg_form_check(f), "eager")
        eager.append(coo(xg, b, n))
    outs = [output(xg, f, n) for f, n in zip(forms, nd)]
    g = graph(xg, forms, lsets, outs)
    xg._lib.call("xg_step_graph_launch", g, xg._stream())
    torch.cuda.synchronize()
    for f in (f1, f2):
        xg._lib.check(xg._lib.load().xg_form_check(f), "graph")
    for b, n, ref in zip(outs, nd, eager):
        got = coo(xg, b, n)
        assert all(np.array_equal(x, y) for x, y in zip(got, ref))
    assert not np.array_equal(eager[0][2][:10], eager[2][2][:10]) or len(eager[0][2]) != len(eager[2][2])
    # two distinct forms writing one output are refused
    f = (ctypes.c_void_p * 2)(f1.value, f2.value)
    l = (ctypes.c_void_p * 2)(lsets[0].data_ptr(), lsets[1].data_ptr())
    o = (xg._lib.Csr * 2)(outs[0]._csr, outs[0]._csr)
    g2 = ctypes.c_void_p()
    assert xg._lib.load().xg_step_graph_create(f, l, o, 2, ctypes.byref(g2)) == 1
    xg._lib.call("xg_step_graph_destroy", g)
    for h in (f1, f2):
        xg._lib.load().xg_form_destroy(h)


def test_spacetime_slabs_one_graph(xg, orc):
    """Space-time slab forms of the moving-circle case as one graph, against
    eager steps (bit-identical) and the oracle (1e-12)."""
    import math
    m = MakeStructured2DMesh(14, 14)
    dm = xg.device_mesh(m)
    sh = ctypes.c_void_p()
    xg._lib.call("xg_space_create_st", dm.h, 1, 1, ctypes.byref(sh))
    info = np.zeros(6, dtype=np.int64)
    xg._lib.call("xg_space_info_st", sh, info.ctypes.data_as(ctypes.c_void_p))
    ndof = int(info[0])
    dt = 1.0 / 16
    forms, lsets, ls_host, terms_all = [], [], [], []
    for s in (2, 3, 9):
        vals = []
        for x in (0.0, 1.0):
            t = (s + x) * dt
            cx, cy = 0.5 + 0.2 * math.cos(2 * math.pi * t), 0.5 + 0.2 * math.sin(2 * math.pi * t)
            vals.append(orc.interpolate_p1_perturb(np.sqrt((m.coords[:, 0] - cx) ** 2 + (m.coords[:, 1] - cy) ** 2)
                                                   - 0.25))
        lst = np.stack(vals)
        w = 0.4 * math.pi
        terms = [dict(kind=orc.TERM_DT_U_V, domain=orc.NEG, coef=1.0),
                 dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, coef=dt),
                 dict(kind=orc.TERM_CONV, domain=orc.NEG, coef=dt, bc=(0.0, w, 0.0), bs=(-w, 0.0, 0.0),
                      omega=2 * math.pi, t0=s * dt, dt=dt),
                 dict(kind=orc.TERM_MASS, domain=orc.NEG, coef=1.0, tref=0.0),
                 dict(kind=orc.TERM_GHOST_MASS, coef=0.05 * dt, hpow=-2)]
        arr = (xg._lib.StTerm * len(terms))()
        for k, t in enumerate(terms):
            B = arr[k].base
            B.kind, B.domain, B.order, B.hpow, B.coef = t["kind"], t.get("domain", 0), -1, t.get("hpow", 0), t["coef"]
            for j in range(3):
                arr[k].bc[j] = t.get("bc", (0, 0, 0))[j]
                arr[k].bs[j] = t.get("bs", (0, 0, 0))[j]
            B.d_defined_on = None
            arr[k].tref = t.get("tref", -1.0)
            arr[k].omega, arr[k].t0, arr[k].dt = t.get("omega", 0.0), t.get("t0", 0.0), t.get("dt", 1.0)
        f = ctypes.c_void_p()
        xg._lib.call("xg_st_form_create", sh, 1, 2, arr, len(terms), 0, ctypes.byref(f))
        forms.append(f)
        lsets.append(torch.from_numpy(lst).cuda())
        ls_host.append(lst)
        terms_all.append(terms)
    outs = [output(xg, f, ndof) for f in forms]
    g = graph(xg, forms, lsets, outs)
    xg._lib.call("xg_step_graph_launch", g, xg._stream())
    torch.cuda.synchronize()
    for f in forms:
        xg._lib.check(xg._lib.load().xg_form_check(f), "graph st")
    sp = orc.Space(m, 1)
    for f, b, l, lst, terms in zip(forms, outs, lsets, ls_host, terms_all):
        r, c, v = coo(xg, b, ndof)
        e = output(xg, f, ndof)
        xg._lib.call("xg_st_cutfem_step", f, xg._vp(l), ctypes.byref(e._csr), xg._stream())
        torch.cuda.synchronize()
        assert all(np.array_equal(x, y) for x, y in zip((r, c, v), coo(xg, e, ndof)))
        dom, _, bits = sp.cutinfo_st(lst, 1)
        fb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
        t2 = [dict(t, defined_on=fb if t["kind"] == orc.TERM_GHOST_MASS else bits[5]) for t in terms]
        rp, rc, rv = sp.assemble_st(lst, 1, 1, 2, t2)
        rr, rc, rv = canon(np.repeat(np.arange(len(rp) - 1), np.diff(rp)), rc, rv)
        r, c, v = canon(r, c, v)
        assert np.array_equal(r, rr) and np.array_equal(c, rc)
        assert np.max(np.abs(v - rv)) / np.max(np.abs(rv)) < 1e-12
    xg._lib.call("xg_step_graph_destroy", g)
    for f in forms:
        xg._lib.load().xg_form_destroy(f)
    xg._lib.load().xg_space_destroy(sh)


@pytest.mark.parametrize("prec", [0, 1])
def test_batched_patch_launch_matches_eager(xg, orc, prec):
    """Distinct forms with basis-change patches (orders 1-3, 2D and 3D) share
    one persistent work-stealing patch launch per dimension in the graph: the
    graph's matrices equal the eager per-form steps bit for bit."""
    groups = batch_groups(7, 5e3, seed=9)
    m2 = MakeStructured2DMesh(14, 11, -1, 1, -1, 1)
    cases = [(m, vals, k) for k, (m, vals) in groups.items()]
    cases.append((m2, np.sqrt((m2.coords ** 2).sum(1)) - 0.55, 3))
    cases.append((m2, np.sqrt((m2.coords ** 2).sum(1)) - 0.45, 2))
    forms, lsets, spaces = [], [], []
    for m, vals, k in cases:
        gf = xg.GridFunction(xg.H1(m, 1))
        xg.InterpolateToP1(vals, gf)
        V = xg.H1(m, order=k)
        spaces.append(V)
        lsets.append(gf.vec)
        forms.append(plain_form(xg, V, C2_TERMS(orc, k), prec))
    eager = []
    for f, l, V in zip(forms, lsets, spaces):
        b = output(xg, f, V.ndof)
        xg._lib.call("xg_cutfem_step", f, xg._vp(l), ctypes.byref(b._csr), xg._stream())
        torch.cuda.synchronize()
        xg._lib.check(xg._lib.load().xg_form_check(f), "eager")
        eager.append(coo(xg, b, V.ndof))
    outs = [output(xg, f, V.ndof) for f, V in zip(forms, spaces)]
    g = graph(xg, forms, lsets, outs)
    for _ in range(2):
        xg._lib.call("xg_step_graph_launch", g, xg._stream())
        torch.cuda.synchronize()
        for f in forms:
            xg._lib.check(xg._lib.load().xg_form_check(f), "graph")
        for b, V, ref in zip(outs, spaces, eager):
            got = coo(xg, b, V.ndof)
            assert all(np.array_equal(x, y) for x, y in zip(got, ref))
    xg._lib.call("xg_step_graph_destroy", g)
    for f in forms:
        xg._lib.load().xg_form_destroy(f)


def test_autotune_keeps_parity_and_determinism(xg, orc):
    """The autotuner times launch choices on the form and keeps the fastest;
    the tuned step still matches the oracle within 1e-12, repeats bit for bit,
    and the table names every tuned key."""
    import json
    m = MakeStructured3DMesh(9)
    c = m.coords - 0.5
    vals = np.sqrt((c ** 2).sum(1)) - 0.31
    gf = xg.GridFunction(xg.H1(m, 1))
    xg.InterpolateToP1(vals, gf)
    for k in (1, 2):
        V = xg.H1(m, order=k)
        f = plain_form(xg, V, C2_TERMS(orc, k), 0)
        b = output(xg, f, V.ndof)
        xg._lib.call("xg_form_autotune", f, xg._vp(gf.vec), ctypes.byref(b._csr), xg._stream())
        res = []
        for _ in range(2):
            xg._lib.call("xg_cutfem_step", f, xg._vp(gf.vec), ctypes.byref(b._csr), xg._stream())
            torch.cuda.synchronize()
            xg._lib.check(xg._lib.load().xg_form_check(f), "tuned")
            res.append(coo(xg, b, V.ndof))
        assert all(np.array_equal(x, y) for x, y in zip(res[0], res[1]))
        sp, rr, rc, rv = oracle_csr(orc, m, gf.vec.cpu().numpy(), k, C2_TERMS(orc, k))
        r, cc, v = canon(*res[0])
        rr, rc, rv = canon(rr, rc, rv)
        assert np.array_equal(r, rr) and np.array_equal(cc, rc)
        assert np.max(np.abs(v - rv)) / np.max(np.abs(rv)) < 1e-12
        xg._lib.load().xg_form_destroy(f)
    need = xg._lib.load().xg_autotune_table(None, 0)
    buf = ctypes.create_string_buffer(int(need))
    xg._lib.load().xg_autotune_table(buf, need)
    table = json.loads(buf.value.decode())
    assert any(key.endswith("/d3/k1/fp64") for key in table) and any(key.endswith("/d3/k2/fp64") for key in table)
    for rec in table.values():
        assert rec["row_pass_rows_per_block"] in (4, 8) and 1 <= rec["row_pass_accumulator_copies"] <= 4
        assert rec["uncut_elements_per_block"] in (16, 32)

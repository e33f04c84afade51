"""Space-time path on the GPU (through the C ABI) against the oracle:
SpaceTimeCutIntegrationRule (cutint/spacetimecutrule.cpp:106-244), space-time
CutInfo (time_order=0) and the space-time CutFEM step shaped like
demos/spacetime/spacetimeDG_unfitted.py:143-168 on a moving circle."""
import ctypes
import math

import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu

DT = 1.0 / 16


def circle_lset(m, t):
    cx, cy = 0.5 + 0.2 * math.cos(2 * math.pi * t), 0.5 + 0.2 * math.sin(2 * math.pi * t)
    return np.sqrt((m.coords[:, 0] - cx) ** 2 + (m.coords[:, 1] - cy) ** 2) - 0.25


def st_lset(orc, m, kt, slab=3):
    t0 = slab * DT
    nodes = [0.0, 1.0] if kt == 1 else [0.0, 0.5, 1.0]
    return np.stack([orc.interpolate_p1_perturb(circle_lset(m, t0 + DT * x)) for x in nodes])


def random_st(orc, m, kt, seed):
    rng = np.random.default_rng(seed)
    base = rng.standard_normal(m.nv) + 0.2
    return np.stack([orc.interpolate_p1_perturb(base + 0.8 * rng.standard_normal(m.nv)) for _ in range(kt + 1)])


CASES = {
    "circle_kt1": lambda orc: (lambda m: (m, st_lset(orc, m, 1), 1))(MakeStructured2DMesh(16, 16)),
    "circle_kt2": lambda orc: (lambda m: (m, st_lset(orc, m, 2), 2))(MakeStructured2DMesh(16, 16)),
    "random2d_kt2": lambda orc: (lambda m: (m, random_st(orc, m, 2, 3), 2))(MakeStructured2DMesh(8, 7)),
    "random3d_kt1": lambda orc: (lambda m: (m, random_st(orc, m, 1, 5), 1))(MakeStructured3DMesh(3, 3, 2)),
}


def dev(x, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(x)).to("cuda", dtype)


@pytest.mark.parametrize("case", list(CASES))
def test_cutinfo_st_parity(xg, orc, case):
    m, lst, kt = CASES[case](orc)
    sp = orc.Space(m, 1)
    dom, ratio, bits = sp.cutinfo_st(lst, kt)
    dm = xg.device_mesh(m)
    d_dom = torch.zeros(m.ne, dtype=torch.uint8, device="cuda")
    d_ratio = torch.zeros(m.ne, dtype=torch.float64, device="cuda")
    d_bits = torch.zeros((8, (m.ne + 63) // 64), dtype=torch.int64, device="cuda")
    d_lst = dev(lst)  # keep the device buffers alive until the kernels have run
    xg._lib.call("xg_cutinfo_update_st", dm.h, xg._vp(d_lst), kt, xg._vp(d_dom), xg._vp(d_ratio), xg._vp(d_bits),
                 xg._stream())
    dm.check()
    assert np.array_equal(d_dom.cpu().numpy(), dom)
    assert np.array_equal(d_ratio.cpu().numpy().view(np.uint64), ratio.view(np.uint64))
    assert np.array_equal(d_bits.cpu().numpy().view(np.uint64), bits)
    assert (dom == 2).sum() > 0


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("dt", [0, 1, 2])
@pytest.mark.parametrize("orders", [(0, 0), (2, 2), (2, 4)])
def test_st_cut_rules_parity(xg, orc, case, dt, orders):
    m, lst, kt = CASES[case](orc)
    sp = orc.Space(m, 1)
    dom, _, _ = sp.cutinfo_st(lst, kt)
    els = np.concatenate([np.nonzero(dom == 2)[0][:150], np.nonzero(dom != 2)[0][:30]]).astype(np.int32)
    dm = xg.device_mesh(m)
    n, maxp = len(els), 1024
    counts = torch.zeros(n, dtype=torch.int32, device="cuda")
    pts = torch.zeros((n, maxp, 4), dtype=torch.float64, device="cuda")
    wts = torch.zeros((n, maxp), dtype=torch.float64, device="cuda")
    d_lst, d_els = dev(lst), dev(els, torch.int32)  # alive until the kernel has run
    xg._lib.call("xg_st_cut_rules", dm.h, xg._vp(d_lst), kt, xg._vp(d_els), n, dt, orders[0], orders[1], maxp,
                 xg._vp(counts), xg._vp(pts), xg._vp(wts), xg._stream())
    dm.check()
    counts, pts, wts = counts.cpu().numpy(), pts.cpu().numpy(), wts.cpu().numpy()
    D = m.dim
    for i, e in enumerate(els):
        vs = m.elements[e]
        r = orc.spacetime_cut_rule(m.coords[vs], lst[:, vs], kt, dt, orders[0], orders[1])
        if r is None:
            assert counts[i] == -1
            continue
        p, w = r
        assert counts[i] == len(w), (int(e), counts[i], len(w), pts[i, : max(counts[i], 0)].tolist(), p.tolist(),
                                     wts[i, : max(counts[i], 0)].tolist(), w.tolist(), lst[:, vs].tolist())
        assert np.max(np.abs(pts[i, : len(w)] - p)) <= 1e-14
        assert np.max(np.abs(wts[i, : len(w)] - w)) <= 1e-14 * np.max(np.abs(w))
    assert D in (2, 3)


def c5_terms(orc, t0, order_k):
    """demos/spacetime/spacetimeDG_unfitted.py:158-168 without deformation:
    v dt(u) dQ + grad u.grad v dQ + v (w.grad u) dQ + u v dOmold + ghost penalty."""
    w_amp = 0.4 * math.pi
    gamma = 0.05
    return [
        dict(kind=orc.TERM_DT_U_V, domain=orc.NEG, coef=1.0),
        dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, coef=DT),
        dict(kind=orc.TERM_CONV, domain=orc.NEG, coef=DT, b=(0.0, 0.0, 0.0), bc=(0.0, w_amp, 0.0),
             bs=(-w_amp, 0.0, 0.0), omega=2 * math.pi, t0=t0, dt=DT),
        dict(kind=orc.TERM_MASS, domain=orc.NEG, coef=1.0, tref=0.0),
        dict(kind=orc.TERM_GHOST_MASS, coef=gamma * DT, hpow=-2),
        dict(kind=orc.TERM_GHOST_MASS, coef=gamma * DT * DT, hpow=-3),
    ]


def oracle_st_csr(orc, m, lst, kt_l, kt, order_time, terms, order):
    sp = orc.Space(m, order)
    dom, ratio, bits = sp.cutinfo_st(lst, kt_l)
    fb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
    t2 = []
    for t in terms:
        t = dict(t)
        t["defined_on"] = fb if t["kind"] == orc.TERM_GHOST_MASS else {orc.NEG: bits[5], orc.IF: bits[4],
                                                                       orc.POS: bits[6]}[t["domain"]]
        t2.append(t)
    return sp, sp.assemble_st(lst, kt_l, kt, order_time, t2)


def xg_st_step(xg, m, lst, kt_l, kt, order_time, terms, order, prec):
    dm = xg.device_mesh(m)
    h = ctypes.c_void_p()
    xg._lib.call("xg_space_create_st", dm.h, order, kt, ctypes.byref(h))
    info = np.zeros(6, dtype=np.int64)
    xg._lib.call("xg_space_info_st", h, info.ctypes.data_as(ctypes.c_void_p))
    arr = (xg._lib.StTerm * len(terms))()
    for k, t in enumerate(terms):
        B = arr[k].base
        B.kind, B.domain, B.order, B.hpow, B.coef = t["kind"], t.get("domain", 0), -1, t.get("hpow", 0), t["coef"]
        for j in range(3):
            B.b[j] = t.get("b", (0, 0, 0))[j]
            arr[k].bc[j] = t.get("bc", (0, 0, 0))[j]
            arr[k].bs[j] = t.get("bs", (0, 0, 0))[j]
        B.d_defined_on = None
        arr[k].tref = t.get("tref", -1.0)
        arr[k].omega, arr[k].t0, arr[k].dt = t.get("omega", 0.0), t.get("t0", 0.0), t.get("dt", 1.0)
    form = ctypes.c_void_p()
    xg._lib.call("xg_st_form_create", h, kt_l, order_time, arr, len(terms), prec, ctypes.byref(form))
    cap = np.zeros(2, dtype=np.int64)
    xg._lib.call("xg_form_capacity", form, cap.ctypes.data_as(ctypes.c_void_p))

    class _S:  # space stand-in for BilinearForm._alloc
        ndof = int(info[0])
    bf = xg.BilinearForm.__new__(xg.BilinearForm)
    bf.space = _S()
    bf._alloc(int(cap[0]), int(cap[1]))
    d_lst = dev(lst)
    xg._lib.call("xg_st_cutfem_step", form, xg._vp(d_lst), ctypes.byref(bf._csr), xg._stream())
    torch.cuda.synchronize()
    xg._lib.check(xg._lib.load().xg_form_check(form), "st form")
    nrows, nnz = (int(v) for v in bf._counts.cpu().tolist())
    mat = xg.SparseMatrix(int(info[0]), bf._row_dof, bf._rowptr, bf._cols, bf._vals, nrows, nnz)
    r, c, v = mat.global_coo()
    xg._lib.load().xg_form_destroy(form)
    xg._lib.load().xg_space_destroy(h)
    return r, c, v


@pytest.mark.parametrize("case", ["circle_kt1", "circle_kt2", "random2d_kt2", "random3d_kt1"])
@pytest.mark.parametrize("order", [1, 2])
def test_st_step_parity(xg, orc, case, order):
    m, lst, kt = CASES[case](orc)
    terms = c5_terms(orc, 3 * DT, order)
    order_time = 2 * kt
    sp, (rp, cols, vals) = oracle_st_csr(orc, m, lst, kt, kt, order_time, terms, order)
    r, c, v = xg_st_step(xg, m, lst, kt, kt, order_time, terms, order, 0)
    ref_rows = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    ref = {(int(a), int(b)): float(x) for a, b, x in zip(ref_rows, cols, vals)}
    got = {(int(a), int(b)): float(x) for a, b, x in zip(r, c, v)}
    assert set(ref) == set(got)
    scale = max(abs(x) for x in ref.values())
    err = max(abs(got[k] - ref[k]) for k in ref) / scale
    assert err < 1e-12, err


@pytest.mark.parametrize("case", ["circle_kt2", "random3d_kt1"])
def test_st_mixed_precision(xg, orc, case):
    m, lst, kt = CASES[case](orc)
    terms = c5_terms(orc, 3 * DT, 1)
    a = xg_st_step(xg, m, lst, kt, kt, 2 * kt, terms, 1, 0)
    b = xg_st_step(xg, m, lst, kt, kt, 2 * kt, terms, 1, 1)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    rel = np.max(np.abs(a[2] - b[2])) / np.max(np.abs(a[2]))
    assert rel < 1e-5, rel

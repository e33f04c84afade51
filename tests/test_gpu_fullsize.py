"""Parity on the benchmarked configurations at their full sizes (GPU through
the C ABI against the oracle on all host threads):

* the 3D CutFEM Poisson step of the default bench line: 64^3 x 6 Kuhn tets,
  P2, NEG stiffness + Nitsche interface terms + ghost penalty 0.1/h^2
  (xfem/symboliccutbfi.cpp:76-486, :1982-2377; demos/fictdom.py:95-133);
* the order-3 group of the batched uneven meshes (the P3 meshes of the 512,
  joined into one disconnected mesh: 5.7M tets);
* one slab of the space-time moving circle (256^2 x 2 triangles, P1 x P1).

Bars: the compressed pattern (active rows and their columns) identical, FP64
values within 1e-12 of the largest entry; the mixed form (FP32 contractions,
FP64 sums) within 1e-5 of the largest entry of the FP64 matrix, with the same
pattern.  Both CSRs are row-major with ascending columns, so the comparison
is element by element."""
import ctypes
import os

import numpy as np
import pytest
import torch

import bench

pytestmark = pytest.mark.gpu

NTH = os.cpu_count() or 1


def plain_form(xg, space_h, terms, prec):
    arr = (xg._lib.Term * len(terms))()
    for k, t in enumerate(terms):
        arr[k].kind, arr[k].domain, arr[k].order = t["kind"], t["domain"], -1
        arr[k].hpow, arr[k].coef = t["hpow"], t["coef"]
        arr[k].d_defined_on = None
    f = ctypes.c_void_p()
    xg._lib.call("xg_form_create", space_h, arr, len(terms), prec, ctypes.byref(f))
    return f


def gpu_step(xg, V, d_lset, terms, prec):
    """One xg_cutfem_step; returns (global rows, global cols, vals) numpy."""
    form = plain_form(xg, V.h, terms, prec)
    cap = np.zeros(2, dtype=np.int64)
    xg._lib.call("xg_form_capacity", form, cap.ctypes.data_as(ctypes.c_void_p))
    bf = xg.BilinearForm(V)
    first = int(cap[1]) if cap[1] * 12 <= (1 << 31) else 1 << 20
    bf._alloc(int(cap[0]), first)
    xg._lib.call("xg_cutfem_step", form, xg._vp(d_lset), ctypes.byref(bf._csr), xg._stream())
    torch.cuda.synchronize()
    st = xg._lib.load().xg_form_check(form)
    nnz = int(bf._counts[1].item())
    if st == xg._lib.XG_ERR_CAPACITY or nnz > first:
        bf._alloc(int(cap[0]), nnz + 1024)
        xg._lib.call("xg_cutfem_step", form, xg._vp(d_lset), ctypes.byref(bf._csr), xg._stream())
        torch.cuda.synchronize()
        st = xg._lib.load().xg_form_check(form)
    xg._lib.check(st, "full-size step")
    nrows, nnz = (int(v) for v in bf._counts.cpu().tolist())
    out = xg.SparseMatrix(V.ndof, bf._row_dof, bf._rowptr, bf._cols, bf._vals, nrows, nnz).global_coo()
    xg._lib.load().xg_form_destroy(form)
    del bf
    torch.cuda.empty_cache()
    return out


def oracle_step(orc, m, l, order, terms):
    sp = orc.Space(m, order)
    dom, _, bits = sp.cutinfo(l, nthreads=NTH)
    fb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
    t2 = [dict(t, defined_on=fb if t["kind"] == orc.TERM_GHOST_MASS else {orc.NEG: bits[5], orc.IF: bits[4]}[
        t["domain"]]) for t in terms]
    rp, cols, vals = sp.assemble(l, t2, nthreads=NTH)
    rows = np.repeat(np.arange(sp.ndof, dtype=np.int64), np.diff(rp))
    return rows, cols, vals, int((dom == orc.IF).sum())


def compare(got, ref, tol):
    r, c, v = got
    rr, rc, rv = ref[:3]
    assert len(v) == len(rv), (len(v), len(rv))
    assert np.array_equal(r, rr)
    assert np.array_equal(c, rc)
    err = float(np.max(np.abs(v - rv)) / np.max(np.abs(rv)))
    assert err < tol, err
    return err


def run_plain_case(xg, orc, m, vals, order, terms, mixed=True):
    l = orc.interpolate_p1_perturb(vals)
    V = xg.H1(m, order=order)
    d_lset = torch.from_numpy(l).cuda()
    ref = oracle_step(orc, m, l, order, terms)
    assert ref[3] > 0
    got = gpu_step(xg, V, d_lset, terms, xg.PREC_FP64)
    err = compare(got, ref, 1e-12)
    print("fp64 vs oracle: %d nnz, %d cut, max rel err %.3e" % (len(ref[2]), ref[3], err))
    if mixed:
        gm = gpu_step(xg, V, d_lset, terms, xg.PREC_MIXED)
        errm = compare(gm, got, 1e-5)
        print("mixed vs fp64: max rel err %.3e" % errm)


def test_c2_full_size(xg, orc):
    """The default bench workload at 64^3 x 6 (1,572,864 tets, P2)."""
    m, vals = bench.c2_mesh(64)
    run_plain_case(xg, orc, m, vals, 2, bench.terms_c2(2))


def test_c3_order3_group_full_size(xg, orc):
    """The P3 meshes of the 512 batched meshes as one disconnected mesh."""
    groups = bench.c3_groups(512)
    m, vals = groups[3]
    assert m.ne > 5_000_000
    run_plain_case(xg, orc, m, vals, 3, bench.terms_c2(3), mixed=False)


def test_c5_slab_full_size(xg, orc):
    """One space-time slab of the moving circle at 256^2 x 2 triangles."""
    m = bench.c5_mesh(256)
    slab = 5
    lst = np.stack([orc.interpolate_p1_perturb(x) for x in bench.c5_slab_values(m, slab, 1)])
    terms = bench.terms_c5(slab * bench.C5_DT)
    dm = xg.device_mesh(m)
    sh = ctypes.c_void_p()
    xg._lib.call("xg_space_create_st", dm.h, 1, 1, ctypes.byref(sh))
    info = np.zeros(6, dtype=np.int64)
    xg._lib.call("xg_space_info_st", sh, info.ctypes.data_as(ctypes.c_void_p))
    ndof = int(info[0])
    arr = (xg._lib.StTerm * len(terms))()
    for k, t in enumerate(terms):
        B = arr[k].base
        B.kind, B.domain, B.order, B.hpow, B.coef = t["kind"], t.get("domain", 0), -1, t.get("hpow", 0), t["coef"]
        for j in range(3):
            B.b[j] = 0.0
            arr[k].bc[j] = t.get("bc", (0, 0, 0))[j]
            arr[k].bs[j] = t.get("bs", (0, 0, 0))[j]
        B.d_defined_on = None
        arr[k].tref = t.get("tref", -1.0)
        arr[k].omega, arr[k].t0, arr[k].dt = t.get("omega", 0.0), t.get("t0", 0.0), t.get("dt", 1.0)
    f = ctypes.c_void_p()
    xg._lib.call("xg_st_form_create", sh, 1, 2, arr, len(terms), xg.PREC_FP64, ctypes.byref(f))
    cap = np.zeros(2, dtype=np.int64)
    xg._lib.call("xg_form_capacity", f, cap.ctypes.data_as(ctypes.c_void_p))
    bf = xg.BilinearForm.__new__(xg.BilinearForm)

    class _S:
        pass
    _S.ndof = ndof
    bf.space, bf._form = _S(), None
    bf._alloc(int(cap[0]), int(cap[1]))
    d_l = torch.from_numpy(lst).cuda()
    xg._lib.call("xg_st_cutfem_step", f, xg._vp(d_l), ctypes.byref(bf._csr), xg._stream())
    torch.cuda.synchronize()
    xg._lib.check(xg._lib.load().xg_form_check(f), "full-size space-time step")
    nrows, nnz = (int(v) for v in bf._counts.cpu().tolist())
    got = xg.SparseMatrix(ndof, bf._row_dof, bf._rowptr, bf._cols, bf._vals, nrows, nnz).global_coo()
    sp = orc.Space(m, 1)
    dom, _, bits = sp.cutinfo_st(lst, 1, nthreads=NTH)
    fb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
    t2 = [dict(t, defined_on=fb if t["kind"] == orc.TERM_GHOST_MASS else bits[5]) for t in terms]
    rp, rc, rv = sp.assemble_st(lst, 1, 1, 2, t2, nthreads=NTH)
    ref = (np.repeat(np.arange(len(rp) - 1, dtype=np.int64), np.diff(rp)), rc, rv)
    err = compare(got, ref, 1e-12)
    print("space-time slab fp64 vs oracle: %d nnz, %d cut, max rel err %.3e" % (nnz, int((dom == 2).sum()), err))
    xg._lib.load().xg_form_destroy(f)
    xg._lib.load().xg_space_destroy(sh)

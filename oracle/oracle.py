"""ctypes front end of the oracle library (test infrastructure only).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline and
reference legs.  Never imported by the product package.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

NEG, POS, IF, WHOLE = 0, 1, 2, 3
TERM_MASS, TERM_LAPLACE, TERM_NGRADU_V, TERM_U_NGRADV, TERM_CONV, TERM_GHOST_MASS, TERM_DT_U_V = range(7)
TERM_SKEL_JUMP, TERM_SKEL_FLUX, TERM_SKEL_FLUX_T, TERM_SKEL_DN1, TERM_SKEL_DN2, TERM_SKEL_DN3 = range(7, 13)
TERM_NGRADU_NGRADV = 13


class Term(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("domain", ctypes.c_int),
        ("order", ctypes.c_int),
        ("hpow", ctypes.c_int),
        ("coef", ctypes.c_double),
        ("b", ctypes.c_double * 3),
        ("defined_on", ctypes.c_void_p),
    ]


class BTerm(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("domain", ctypes.c_int),
        ("order", ctypes.c_int),
        ("hpow", ctypes.c_int),
        ("coef", ctypes.c_double),
        ("defined_on", ctypes.c_void_p),
    ]


class CTerm(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("domain", ctypes.c_int),
        ("order", ctypes.c_int),
        ("hpow", ctypes.c_int),
        ("coef", ctypes.c_double),
        ("b", ctypes.c_double * 3),
        ("e", ctypes.c_int * 3),
        ("gf_order", ctypes.c_int),
        ("gf_el", ctypes.c_void_p),
        ("defined_on", ctypes.c_void_p),
        ("theta_el", ctypes.c_void_p),
    ]


class MlTerm(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("order", ctypes.c_int),
        ("hpow", ctypes.c_int),
        ("normal_lset", ctypes.c_int),
        ("coef", ctypes.c_double),
        ("b", ctypes.c_double * 3),
        ("ntup", ctypes.c_int),
        ("dts", ctypes.c_void_p),
        ("defined_on", ctypes.c_void_p),
    ]


class StTerm(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int),
        ("domain", ctypes.c_int),
        ("order", ctypes.c_int),
        ("hpow", ctypes.c_int),
        ("coef", ctypes.c_double),
        ("b", ctypes.c_double * 3),
        ("defined_on", ctypes.c_void_p),
        ("tref", ctypes.c_double),
        ("bc", ctypes.c_double * 3),
        ("bs", ctypes.c_double * 3),
        ("omega", ctypes.c_double),
        ("t0", ctypes.c_double),
        ("dt", ctypes.c_double),
    ]


def build():
    subprocess.check_call(["make", "-s", "-C", HERE])


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()  # make: a no-op when the library is current
        L = ctypes.CDLL(LIB)
        P = ctypes.c_void_p
        L.orc_check_if_straight_cut.argtypes = [P, ctypes.c_int, ctypes.c_double]
        L.orc_interpolate_p1_perturb.argtypes = [P, ctypes.c_int, ctypes.c_double]
        L.orc_base_rule.argtypes = [ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int]
        L.orc_straight_cut_rule.argtypes = [ctypes.c_int, P, P, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int]
        L.orc_space_create.restype = P
        L.orc_space_create.argtypes = [ctypes.c_int, ctypes.c_int, P, ctypes.c_int, P, ctypes.c_int]
        L.orc_space_create_l2.restype = P
        L.orc_space_create_l2.argtypes = [ctypes.c_int, ctypes.c_int, P, ctypes.c_int, P, ctypes.c_int]
        L.orc_facet_matrix.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
        L.orc_fd_stencil.argtypes = [ctypes.c_int, ctypes.c_int, P, P]
        L.orc_assemble_ex.restype = P
        L.orc_assemble_ex.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_subdiv_rule.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P,
                                      ctypes.c_int]
        L.orc_integrate_subdiv.restype = ctypes.c_double
        L.orc_integrate_subdiv.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.c_int, P, P]
        L.orc_subdiv_moments_p2.argtypes = [ctypes.c_int64, P, ctypes.c_int, P, ctypes.c_int]
        L.orc_assemble_full.restype = P
        L.orc_assemble_full.argtypes = [P, P, P, ctypes.c_int, P, ctypes.c_int, P, ctypes.c_int, P, ctypes.c_int,
                                        ctypes.c_int]
        L.orc_assemble_bnd.restype = P
        L.orc_assemble_bnd.argtypes = [P, P, P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_mlset_assemble.restype = P
        L.orc_mlset_assemble.argtypes = [P, ctypes.c_int, P, P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int]
        L.orc_space_destroy.argtypes = [P]
        L.orc_space_info.argtypes = [P, P]
        L.orc_space_el_dofs.argtypes = [P, P]
        L.orc_space_facet_els.argtypes = [P, P]
        L.orc_cutinfo.argtypes = [P, P, P, P, P, ctypes.c_int]
        L.orc_facets_with_neighbor_types.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
        L.orc_integrate.restype = ctypes.c_double
        L.orc_integrate.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
        L.orc_integrate_fields.restype = ctypes.c_double
        L.orc_integrate_fields.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int, P, P,
                                           P, P, P, P, P, P]
        L.orc_element_matrix.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int, P]
        L.orc_patch_matrix.argtypes = [P, P, ctypes.c_int, ctypes.c_int, P]
        L.orc_assemble.restype = P
        L.orc_assemble.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int]
        L.orc_csr_nnz.restype = ctypes.c_int64
        L.orc_csr_nnz.argtypes = [P]
        L.orc_csr_get.argtypes = [P, P, P, P]
        L.orc_csr_destroy.argtypes = [P]
        L.orc_time_basis.argtypes = [ctypes.c_int, ctypes.c_double, P, P]
        L.orc_spacetime_cut_rule.argtypes = [ctypes.c_int, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             P, P, ctypes.c_int]
        L.orc_cutinfo_st.argtypes = [P, P, ctypes.c_int, P, P, P, ctypes.c_int]
        L.orc_st_element_matrix.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, ctypes.c_int,
                                            ctypes.c_int, P]
        L.orc_assemble_st.restype = P
        L.orc_assemble_st.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, ctypes.c_int, ctypes.c_int]
        L.orc_integrate_st.restype = ctypes.c_double
        L.orc_integrate_st.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_iso_deformation.argtypes = [ctypes.c_int, P, P, ctypes.c_double, P, P]
        L.orc_iso_cut_rule.argtypes = [ctypes.c_int, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                       P, P, ctypes.c_int, P]
        L.orc_iso_moments_tet.argtypes = [ctypes.c_int64, P, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int]
        L.orc_subdiv_moments_tet.argtypes = [P, ctypes.c_int, P]
        L.orc_iso_integrate_mesh.restype = ctypes.c_double
        L.orc_iso_integrate_mesh.argtypes = [ctypes.c_int, ctypes.c_int, P, ctypes.c_int, P, P, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_double, ctypes.c_int, P]
        L.orc_quad_assemble.restype = P
        L.orc_quad_assemble.argtypes = [ctypes.c_int, ctypes.c_int, P, ctypes.c_int, P, P, P, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, P]
        L.orc_iso_theta_mesh.argtypes = [ctypes.c_int, ctypes.c_int, P, ctypes.c_int, P, P, ctypes.c_double, P, P]
        L.orc_boundary_elements.argtypes = [P, P, P]
        L.orc_cutinfo_bnd.argtypes = [P, P, P, P, P]
        L.orc_cutinfo_nodes.argtypes = [P, P, P, P, P, P, P, P, P, P, P]
        L.orc_linear_form.argtypes = [P, P, P, ctypes.c_int, P]
        L.orc_pipeline.restype = ctypes.c_int64
        L.orc_pipeline.argtypes = [P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        I = ctypes.c_int
        L.orc_quad_cut_rule.argtypes = [I, P, I, I, I, P, P, I]
        L.orc_quad_straight_cut_rule.argtypes = [I, P, P, I, I, I, P, P, I]
        L.orc_quad_integrate.restype = ctypes.c_double
        L.orc_quad_integrate.argtypes = [I, I, P, I, P, P, I, I, I, I, I, I, P]
        L.orc_quad_cutinfo.argtypes = [I, I, P, I, P, P, I, P, P, P]
        L.orc_quad_integrate_mt.restype = ctypes.c_double
        L.orc_quad_integrate_mt.argtypes = [I, I, P, I, P, P, I, I, I, I, I, I, I, P]
        L.orc_mlset_cut_rule.argtypes = [I, P, I, P, I, P, I, P, P, I]
        L.orc_mlset_integrate.restype = ctypes.c_double
        L.orc_mlset_integrate.argtypes = [I, I, P, I, P, I, P, I, P, I, I, I, I, P]
        L.orc_mlset_mark.argtypes = [I, I, P, I, P, I, P, I, P, I, P]
        L.orc_integrate_bnd.restype = ctypes.c_double
        L.orc_integrate_bnd.argtypes = [I, I, P, I, P, P, I, I, I, I, I, P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def check_if_straight_cut(vals, eps=0.0):
    v = np.ascontiguousarray(vals, dtype=np.float64)
    return lib().orc_check_if_straight_cut(_p(v), len(v), eps)


def interpolate_p1_perturb(vals, eps=1e-14):
    v = np.array(vals, dtype=np.float64, copy=True)
    lib().orc_interpolate_p1_perturb(_p(v), len(v), eps)
    return v


def base_rule(d, p):
    pts = np.zeros((4096, 3))
    w = np.zeros(4096)
    n = lib().orc_base_rule(d, p, _p(pts), _p(w), 4096)
    return pts[:n].copy(), w[:n].copy()


def straight_cut_rule(elcoords, lset, dt, order):
    """Returns (points (n,3) in reference coordinates, weights) or None (no rule)."""
    elc = np.ascontiguousarray(elcoords, dtype=np.float64)
    D = elc.shape[1]
    l = np.ascontiguousarray(lset, dtype=np.float64)
    pts = np.zeros((2048, 3))
    w = np.zeros(2048)
    n = lib().orc_straight_cut_rule(D, _p(elc), _p(l), dt, order, _p(pts), _p(w), 2048)
    if n == -1:
        return None
    if n < -1:
        raise RuntimeError("oracle cut rule error %d" % n)
    return pts[:n].copy(), w[:n].copy()


# ---- quadrilaterals and hexahedra (cutint/straightcutrule.cpp:206-501) --------------
QUAD_FIRST, QUAD_OPTIMAL, QUAD_FALLBACK = 0, 1, 2


def quad_cut_rule(lset_vals, dt, order, policy=QUAD_OPTIMAL, elcoords=None, maxpts=8192):
    """Cut rule on the unit square / cube for the multilinear level set with
    the given vertex values (vertex order (0,0),(1,0),(1,1),(0,1) [, z = 1]).
    With elcoords (nv x 3) the interface weights include the element map.
    Returns (points, weights), None for "no rule"; raises on an error."""
    l = np.ascontiguousarray(lset_vals, dtype=np.float64)
    D = 2 if len(l) == 4 else 3
    pts = np.zeros((maxpts, 3))
    w = np.zeros(maxpts)
    if elcoords is None:
        n = lib().orc_quad_cut_rule(D, _p(l), dt, order, policy, _p(pts), _p(w), maxpts)
    else:
        xv = np.zeros((len(l), 3))
        xv[:, :D] = np.asarray(elcoords, dtype=np.float64)[:, :D]
        n = lib().orc_quad_straight_cut_rule(D, _p(xv), _p(l), dt, order, policy, _p(pts), _p(w), maxpts)
    if n == -1:
        return None
    if n < -1:
        raise RuntimeError("oracle quad rule status %d" % (-n - 1))
    return pts[:n].copy(), w[:n].copy()


def quad_cutinfo(mesh, lset, policy=QUAD_OPTIMAL):
    """CutInfo on a quad / hex mesh: (dom, ratio, bits[8][nwords] as uint64)."""
    c = np.ascontiguousarray(mesh.coords, dtype=np.float64)
    el = np.ascontiguousarray(mesh.elements, dtype=np.int32)
    l = np.ascontiguousarray(lset, dtype=np.float64)
    ne = el.shape[0]
    dom = np.zeros(ne, dtype=np.uint8)
    ratio = np.zeros(ne)
    bits = np.zeros((8, (ne + 63) // 64), dtype=np.uint64)
    st = lib().orc_quad_cutinfo(c.shape[1], c.shape[0], _p(c), ne, _p(el), _p(l), policy, _p(dom), _p(ratio),
                                _p(bits))
    if st:
        raise RuntimeError("oracle quad cutinfo status %d" % st)
    return dom, ratio, bits


def quad_integrate(mesh, lset, dt, order, policy=QUAD_OPTIMAL, exps=(0, 0, 0), nthreads=1):
    """Integrate(x^a y^b z^c * dCut) on a quad / hex mesh; returns (value, status)."""
    c = np.ascontiguousarray(mesh.coords, dtype=np.float64)
    el = np.ascontiguousarray(mesh.elements, dtype=np.int32)
    l = np.ascontiguousarray(lset, dtype=np.float64)
    st = np.zeros(1, dtype=np.int32)
    if nthreads > 1:
        v = lib().orc_quad_integrate_mt(c.shape[1], c.shape[0], _p(c), el.shape[0], _p(el), _p(l), dt, order,
                                        policy, exps[0], exps[1], exps[2], nthreads, _p(st))
    else:
        v = lib().orc_quad_integrate(c.shape[1], c.shape[0], _p(c), el.shape[0], _p(el), _p(l), dt, order, policy,
                                     exps[0], exps[1], exps[2], _p(st))
    return v, int(st[0])


# ---- several level sets (cutint/straightcutrule.cpp:679-812, mlsetintegration.cpp) --
def _tuples(dts, M):
    t = np.ascontiguousarray(np.array(dts, dtype=np.int32).reshape(-1, M))
    return t, t.shape[0]


def mlset_cut_rule(elcoords, lsets, dts, order, maxpts=20000):
    """Rule of one simplex for the domain tuples dts (list of M-tuples), the M
    level sets given by their vertex values lsets (M x (D+1)).  Returns
    (points, weights) in reference coordinates, None for no rule."""
    elc = np.ascontiguousarray(elcoords, dtype=np.float64)
    D = elc.shape[1]
    l = np.ascontiguousarray(lsets, dtype=np.float64)
    M = l.shape[0]
    t, nt = _tuples(dts, M)
    pts = np.zeros((maxpts, 3))
    w = np.zeros(maxpts)
    n = lib().orc_mlset_cut_rule(D, _p(elc), M, _p(l), nt, _p(t), order, _p(pts), _p(w), maxpts)
    if n == -1:
        return None
    if n < -1:
        raise RuntimeError("oracle mlset rule status %d" % (-n - 1))
    return pts[:n].copy(), w[:n].copy()


def mlset_integrate(mesh, lsets, dts, order, exps=(0, 0, 0)):
    """Integrate(x^a y^b z^c) over the union of the domain tuples dts of the
    level sets lsets (M x nv); returns (value, status)."""
    c = np.ascontiguousarray(mesh.coords, dtype=np.float64)
    el = np.ascontiguousarray(mesh.elements, dtype=np.int32)
    l = np.ascontiguousarray(lsets, dtype=np.float64)
    M = l.shape[0]
    t, nt = _tuples(dts, M)
    st = np.zeros(1, dtype=np.int32)
    v = lib().orc_mlset_integrate(c.shape[1], c.shape[0], _p(c), el.shape[0], _p(el), M, _p(l), nt, _p(t), order,
                                  exps[0], exps[1], exps[2], _p(st))
    return v, int(st[0])


def mlset_mark(mesh, lsets, dts, mode):
    """MultiLevelsetCutInfo markers (mode 0: elements of the tuples' types,
    1: elements with a contribution); returns a bool array over the elements."""
    c = np.ascontiguousarray(mesh.coords, dtype=np.float64)
    el = np.ascontiguousarray(mesh.elements, dtype=np.int32)
    l = np.ascontiguousarray(lsets, dtype=np.float64)
    M = l.shape[0]
    t, nt = _tuples(dts, M)
    bits = np.zeros((el.shape[0] + 63) // 64, dtype=np.uint64)
    st = lib().orc_mlset_mark(c.shape[1], c.shape[0], _p(c), el.shape[0], _p(el), M, _p(l), nt, _p(t), mode,
                              _p(bits))
    if st:
        raise RuntimeError("oracle mlset marking status %d" % st)
    return np.unpackbits(bits.view(np.uint8), bitorder="little")[: el.shape[0]].astype(bool)


def integrate_bnd(mesh, lset, dt, order, exps=(0, 0, 0), defined_on=None):
    """Integrate(x^a y^b z^c * dCut(lset, dt, vb=BND)); defined_on: optional
    boolean mask over the BND elements (boundary facets in lexicographic order
    of their sorted vertices).  Returns (value, status)."""
    c = np.ascontiguousarray(mesh.coords, dtype=np.float64)
    el = np.ascontiguousarray(mesh.elements, dtype=np.int32)
    l = np.ascontiguousarray(lset, dtype=np.float64)
    st = np.zeros(1, dtype=np.int32)
    mask = None if defined_on is None else np.ascontiguousarray(defined_on, dtype=np.uint8)
    v = lib().orc_integrate_bnd(c.shape[1], c.shape[0], _p(c), el.shape[0], _p(el), _p(l), dt, order, exps[0],
                                exps[1], exps[2], None if mask is None else _p(mask), _p(st))
    return v, int(st[0])


def time_basis(kt, tau):
    psi = np.zeros(3)
    dpsi = np.zeros(3)
    lib().orc_time_basis(kt, tau, _p(psi), _p(dpsi))
    return psi[: kt + 1].copy(), dpsi[: kt + 1].copy()


def spacetime_cut_rule(elcoords, lset_st, kt, dt, order_space, order_time):
    """lset_st: (kt+1, D+1) time-major values.  Returns (points (n,4): xi,eta,zeta,tau, weights) or None."""
    elc = np.ascontiguousarray(elcoords, dtype=np.float64)
    D = elc.shape[1]
    l = np.ascontiguousarray(lset_st, dtype=np.float64).ravel()
    pts = np.zeros((8192, 4))
    w = np.zeros(8192)
    n = lib().orc_spacetime_cut_rule(D, _p(elc), _p(l), kt, dt, order_space, order_time, _p(pts), _p(w), 8192)
    if n == -1:
        return None
    if n < -1:
        raise RuntimeError("oracle space-time rule error %d" % n)
    return pts[:n].copy(), w[:n].copy()


def _st_terms(terms):
    arr = (StTerm * len(terms))()
    keep = []
    for i, t in enumerate(terms):
        arr[i].kind = t["kind"]
        arr[i].domain = t.get("domain", NEG)
        arr[i].order = t.get("order", -1)
        arr[i].hpow = t.get("hpow", 0)
        arr[i].coef = t.get("coef", 1.0)
        for k, name in ((0, "b"), (1, "bc"), (2, "bs")):
            v = t.get(name, (0.0, 0.0, 0.0))
            for j in range(3):
                getattr(arr[i], name)[j] = v[j]
        arr[i].tref = t.get("tref", -1.0)
        arr[i].omega = t.get("omega", 0.0)
        arr[i].t0 = t.get("t0", 0.0)
        arr[i].dt = t.get("dt", 1.0)
        d = t.get("defined_on")
        if d is not None:
            d = np.ascontiguousarray(d, dtype=np.uint64)
            keep.append(d)
            arr[i].defined_on = d.ctypes.data
        else:
            arr[i].defined_on = None
    return arr, keep


def iso_deformation(elcoords, p2vals, threshold=-1.0):
    """Per-element LevelSetMeshAdaptation deformation: (theta[nedges, D], deformed, nonconv)."""
    elc = np.ascontiguousarray(elcoords, dtype=np.float64)
    D = elc.shape[1]
    v = np.ascontiguousarray(p2vals, dtype=np.float64)
    th = np.zeros((3 if D == 2 else 6, D))
    nc = ctypes.c_int(0)
    r = lib().orc_iso_deformation(D, _p(elc), _p(v), threshold, _p(th), ctypes.byref(nc))
    if r < 0:
        raise RuntimeError("orc_iso_deformation failed: %d" % r)
    return th, bool(r), nc.value


def iso_cut_rule(elcoords, p2vals, dt, order, threshold=-1.0, deform=True):
    """Cut rule of the (per-element) isoparametrically deformed simplex: (points, weights, nonconv)."""
    elc = np.ascontiguousarray(elcoords, dtype=np.float64)
    D = elc.shape[1]
    v = np.ascontiguousarray(p2vals, dtype=np.float64)
    pts = np.zeros((8192, 3))
    wts = np.zeros(8192)
    nc = ctypes.c_int(0)
    n = lib().orc_iso_cut_rule(D, _p(elc), _p(v), dt, order, threshold, int(deform), _p(pts), _p(wts), 8192,
                               ctypes.byref(nc))
    if n == -1:
        return None
    if n < 0:
        raise RuntimeError("orc_iso_cut_rule failed: %d" % n)
    return pts[:n, :D].copy(), wts[:n].copy(), nc.value


def iso_integrate_mesh(mesh, p2vals, dt, order, threshold=-1.0, deform=True):
    """Integral of 1 over the dt part of the deformed mesh (mesh-level deformation)."""
    v = np.ascontiguousarray(p2vals, dtype=np.float64)
    nc = ctypes.c_int(0)
    r = lib().orc_iso_integrate_mesh(mesh.dim, mesh.nv, _p(mesh.coords), mesh.ne, _p(mesh.elements), _p(v), dt, order,
                                     threshold, int(deform), ctypes.byref(nc))
    return r, nc.value


def quad_assemble(mesh, lset, terms, policy=1, nthreads=1):
    """Bilinear form of the Q1 space on a quad / hex mesh (orc_quad_assemble):
    CSR triple over the mesh's vertices and the first rule error (0: none)."""
    arr, keep = Space._terms(terms)
    l = np.ascontiguousarray(lset, dtype=np.float64)
    st = ctypes.c_int(0)
    c = lib().orc_quad_assemble(mesh.dim, mesh.nv, _p(mesh.coords), mesh.ne, _p(mesh.elements), _p(l),
                                ctypes.cast(arr, ctypes.c_void_p), len(terms), policy, nthreads, ctypes.byref(st))
    nnz = lib().orc_csr_nnz(c)
    rowptr = np.zeros(mesh.nv + 1, dtype=np.int64)
    cols = np.zeros(nnz, dtype=np.int32)
    vals = np.zeros(nnz)
    lib().orc_csr_get(c, _p(rowptr), _p(cols), _p(vals))
    lib().orc_csr_destroy(c)
    return (rowptr, cols, vals), st.value


def iso_theta_mesh(mesh, p2vals, threshold=-1.0):
    """The mesh-level deformation per element: (ne, 6, 3) edge coefficients in
    each element's reference frame, and the count of non-converged searches."""
    v = np.ascontiguousarray(p2vals, dtype=np.float64)
    out = np.zeros((mesh.ne, 6, 3))
    nc = ctypes.c_int(0)
    r = lib().orc_iso_theta_mesh(mesh.dim, mesh.nv, _p(mesh.coords), mesh.ne, _p(mesh.elements), _p(v), threshold,
                                 _p(out), ctypes.byref(nc))
    if r:
        raise RuntimeError("oracle deformation error %d" % r)
    return out, nc.value


def p2_nodal_values(mesh, f):
    """Element-local P2 nodal values (vertices, then edge midpoints) of f(points)."""
    D = mesh.dim
    E = [(0, 1), (0, 2), (1, 2)] if D == 2 else [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    P = mesh.coords[mesh.elements]  # ne x (D+1) x D
    nodes = [P[:, i] for i in range(D + 1)] + [0.5 * (P[:, a] + P[:, b]) for a, b in E]
    return np.stack([f(x) for x in nodes], axis=1)


def iso_moments_tet(vals10, order=11, deform=True, nthreads=1):
    """NEG-part moments (n, 35) of the reference tet for P2 values (n, 10), and the
    per-element count of non-converged point searches."""
    v = np.ascontiguousarray(vals10, dtype=np.float64).reshape(-1, 10)
    out = np.zeros((v.shape[0], 35))
    nc = np.zeros(v.shape[0], dtype=np.int32)
    lib().orc_iso_moments_tet(v.shape[0], _p(v), order, int(deform), _p(out), _p(nc), nthreads)
    return out, nc


def subdiv_moments_tet(vals10, levels):
    v = np.ascontiguousarray(vals10, dtype=np.float64)
    out = np.zeros(35)
    lib().orc_subdiv_moments_tet(_p(v), levels, _p(out))
    return out


def moment_exponents():
    """(a, b, c) of the 35 moments in their graded order."""
    return [(a, b, t - a - b) for t in range(5) for a in range(t, -1, -1) for b in range(t - a, -1, -1)]


class LTerm(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("domain", ctypes.c_int), ("order", ctypes.c_int), ("e", ctypes.c_int * 3),
                ("coef", ctypes.c_double), ("gf", ctypes.c_void_p), ("defined_on", ctypes.c_void_p)]


def subdiv_moments_p2(vals10, levels, nthreads=1):
    """NEG moments of P2 level sets on the reference tetrahedron by the
    subdivision rule (n x 10 values -> n x 35)."""
    v = np.ascontiguousarray(vals10, dtype=np.float64)
    out = np.zeros((v.shape[0], 35))
    r = lib().orc_subdiv_moments_p2(v.shape[0], _p(v), levels, _p(out), nthreads)
    if r:
        raise RuntimeError("oracle subdivision rule error %d" % r)
    return out


def fd_stencil(k, acc=4):
    """Central finite-difference stencil of DiffOpDuDnk (offsets -w..w) and its
    step factor (times the element size)."""
    c = np.zeros(16)
    eps = np.zeros(1)
    w = lib().orc_fd_stencil(k, acc, _p(c), _p(eps))
    return c[: 2 * w + 1].copy(), float(eps[0])


class Space:
    """H1 space of order k over a simplex mesh, with the oracle's topology
    (l2=True: the discontinuous space, element-local dofs)."""

    def __init__(self, mesh, order, l2=False):
        self.mesh = mesh
        self.order = order
        create = lib().orc_space_create_l2 if l2 else lib().orc_space_create
        self.h = create(mesh.dim, mesh.nv, _p(mesh.coords), mesh.ne, _p(mesh.elements), order)
        if not self.h:
            raise ValueError("bad space")
        info = np.zeros(5, dtype=np.int64)
        lib().orc_space_info(self.h, _p(info))
        self.ndof, self.nedges, self.nfaces, self.nfacets, self.ndof_el = (int(x) for x in info)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_space_destroy(self.h)
            self.h = None

    def el_dofs(self):
        out = np.zeros((self.mesh.ne, self.ndof_el), dtype=np.int32)
        lib().orc_space_el_dofs(self.h, _p(out))
        return out

    def facet_els(self):
        out = np.zeros((self.nfacets, 2), dtype=np.int32)
        lib().orc_space_facet_els(self.h, _p(out))
        return out

    def cutinfo(self, lset, nthreads=1):
        ne = self.mesh.ne
        nw = (ne + 63) // 64
        dom = np.zeros(ne, dtype=np.uint8)
        ratio = np.zeros(ne)
        bits = np.zeros((8, nw), dtype=np.uint64)
        l = np.ascontiguousarray(lset, dtype=np.float64)
        r = lib().orc_cutinfo(self.h, _p(l), _p(dom), _p(ratio), _p(bits), nthreads)
        if r:
            raise RuntimeError("oracle cutinfo error %d" % r)
        return dom, ratio, bits

    def boundary_elements(self):
        n = lib().orc_boundary_elements(self.h, None, None)
        D = self.mesh.dim
        facets = np.zeros(n, dtype=np.int32)
        verts = np.zeros((n, D), dtype=np.int32)
        lib().orc_boundary_elements(self.h, _p(facets), _p(verts))
        return facets, verts

    def cutinfo_bnd(self, lset):
        n = lib().orc_boundary_elements(self.h, None, None)
        dom = np.zeros(n, dtype=np.uint8)
        ratio = np.zeros(n)
        bits = np.zeros((8, (n + 63) // 64), dtype=np.uint64)
        l = np.ascontiguousarray(lset, dtype=np.float64)
        r = lib().orc_cutinfo_bnd(self.h, _p(l), _p(dom), _p(ratio), _p(bits))
        if r:
            raise RuntimeError("oracle cutinfo_bnd error %d" % r)
        return dom, ratio, bits

    def cutinfo_nodes(self, dom, ratio):
        info = np.zeros(5, dtype=np.int64)
        lib().orc_space_info(self.h, _p(info))
        nv, ne, D = self.mesh.nv, self.mesh.ne, self.mesh.dim
        nedges, nfaces = int(info[1]), int(info[2])
        w = lambda n: np.zeros((n + 63) // 64, dtype=np.uint64)  # noqa: E731
        nb_v, nb_e, nb_f, nb_el = w(nv), w(nedges), w(max(nfaces, 1)), w(ne)
        dv, de = np.zeros(nv, np.uint8), np.zeros(nedges, np.uint8)
        df, dc = np.zeros(max(nfaces, 1), np.uint8), np.zeros(ne, np.uint8)
        d8 = np.ascontiguousarray(dom, dtype=np.uint8)
        rr = np.ascontiguousarray(ratio, dtype=np.float64)
        lib().orc_cutinfo_nodes(self.h, _p(d8), _p(rr), _p(nb_v), _p(nb_e), _p(nb_f), _p(nb_el), _p(dv), _p(de),
                                _p(df), _p(dc))
        return (nb_v, nb_e, nb_f[: (nfaces + 63) // 64], nb_el), (dv, de, df[:nfaces], dc)

    def linear_form(self, lset, terms):
        """terms: dicts kind (0 monomial source, 1 same-space function), domain, coef,
        e (exponents), gf (dof vector), order, defined_on (bits)."""
        arr = (LTerm * len(terms))()
        keep = []
        for k, t in enumerate(terms):
            arr[k].kind, arr[k].domain, arr[k].order = t["kind"], t.get("domain", 0), t.get("order", -1)
            for j in range(3):
                arr[k].e[j] = t.get("e", (0, 0, 0))[j]
            arr[k].coef = t.get("coef", 1.0)
            gf = t.get("gf")
            if gf is not None:
                gf = np.ascontiguousarray(gf, dtype=np.float64)
                keep.append(gf)
            arr[k].gf = gf.ctypes.data if gf is not None else None
            d = t.get("defined_on")
            if d is not None:
                d = np.ascontiguousarray(d, dtype=np.uint64)
                keep.append(d)
            arr[k].defined_on = d.ctypes.data if d is not None else None
        info = np.zeros(5, dtype=np.int64)
        lib().orc_space_info(self.h, _p(info))
        out = np.zeros(int(info[0]))
        l = np.ascontiguousarray(lset, dtype=np.float64)
        r = lib().orc_linear_form(self.h, _p(l), ctypes.cast(arr, ctypes.c_void_p), len(terms), _p(out))
        if r:
            raise RuntimeError("oracle linear form error %d" % r)
        return out

    def facets_with_neighbor_types(self, a, b, bnd_a=False, bnd_b=False, use_and=True):
        out = np.zeros((self.nfacets + 63) // 64, dtype=np.uint64)
        a = np.ascontiguousarray(a, dtype=np.uint64)
        b = np.ascontiguousarray(b, dtype=np.uint64)
        lib().orc_facets_with_neighbor_types(self.h, _p(a), _p(b), int(bnd_a), int(bnd_b), int(use_and), _p(out))
        return out

    def integrate(self, lset, dt, order, ex=0, ey=0, ez=0, defined_on=None):
        l = np.ascontiguousarray(lset, dtype=np.float64)
        d = None if defined_on is None else np.ascontiguousarray(defined_on, dtype=np.uint64)
        return lib().orc_integrate(self.h, _p(l), dt, order, ex, ey, ez, _p(d))

    def integrate_fields(self, lset, dt, order, fields, monos, defined_on=None, theta=None):
        """Integrate of sum_m c_m x^e_m F_a F_b over the straight cut rule.
        fields: list of (order, element coefficients [ne][nd]); monos: list of
        (c, (ex, ey, ez), a, b[, da, db]), a / b field indices or -1, da / db
        -1 for the value or the direction of a derivative."""
        if len(fields) > 8:
            raise ValueError("at most 8 fields")
        l = np.ascontiguousarray(lset, dtype=np.float64)
        d = None if defined_on is None else np.ascontiguousarray(defined_on, dtype=np.uint64)
        fo = np.array([k for k, _ in fields] or [0], dtype=np.int32)
        fe = [np.ascontiguousarray(v, dtype=np.float64) for _, v in fields]
        fp = (ctypes.c_void_p * max(len(fe), 1))(*[v.ctypes.data for v in fe])
        c = np.array([m[0] for m in monos], dtype=np.float64)
        e3 = np.array([m[1] for m in monos], dtype=np.int32).reshape(-1)
        f0 = np.array([m[2] for m in monos], dtype=np.int32)
        f1 = np.array([m[3] for m in monos], dtype=np.int32)
        d0 = np.array([m[4] if len(m) > 4 else -1 for m in monos], dtype=np.int32)
        d1 = np.array([m[5] if len(m) > 5 else -1 for m in monos], dtype=np.int32)
        th = None if theta is None else np.ascontiguousarray(theta, dtype=np.float64)
        return lib().orc_integrate_fields(self.h, _p(l), dt, order, len(fe), _p(fo), ctypes.cast(fp, ctypes.c_void_p),
                                          len(monos), _p(c), _p(e3), _p(f0), _p(f1), _p(d0), _p(d1), _p(d), _p(th))

    @staticmethod
    def _terms(terms):
        arr = (Term * len(terms))()
        keep = []
        for i, t in enumerate(terms):
            arr[i].kind = t["kind"]
            arr[i].domain = t.get("domain", NEG)
            arr[i].order = t.get("order", -1)
            arr[i].hpow = t.get("hpow", 0)
            arr[i].coef = t.get("coef", 1.0)
            b = t.get("b", (0.0, 0.0, 0.0))
            for k in range(3):
                arr[i].b[k] = b[k]
            d = t.get("defined_on")
            if d is not None:
                d = np.ascontiguousarray(d, dtype=np.uint64)
                keep.append(d)
                arr[i].defined_on = d.ctypes.data
            else:
                arr[i].defined_on = None
        return arr, keep

    def element_matrix(self, lset, terms, e):
        arr, keep = self._terms(terms)
        n = self.ndof_el
        out = np.zeros((n, n))
        l = np.ascontiguousarray(lset, dtype=np.float64)
        r = lib().orc_element_matrix(self.h, _p(l), ctypes.cast(arr, ctypes.c_void_p), len(terms), e, _p(out))
        if r:
            raise RuntimeError("oracle element matrix error %d" % r)
        return out

    def patch_matrix(self, terms, f):
        arr, keep = self._terms(terms)
        n = 2 * self.ndof_el
        out = np.zeros((n, n))
        r = lib().orc_patch_matrix(self.h, ctypes.cast(arr, ctypes.c_void_p), len(terms), f, _p(out))
        if r:
            raise RuntimeError("oracle patch matrix error %d" % r)
        return out

    def subdiv_rule(self, lset_coefs, e, dt, order, subdivlvl, maxpts=200000):
        """Subdivision rule of element e (physical points, physical weights) for
        the level set given by its coefficients in this space."""
        c = np.ascontiguousarray(lset_coefs, dtype=np.float64)
        pts = np.zeros((maxpts, 3))
        wts = np.zeros(maxpts)
        n = lib().orc_subdiv_rule(self.h, _p(c), e, dt, order, subdivlvl, _p(pts), _p(wts), maxpts)
        if n < 0:
            raise RuntimeError("oracle subdivision rule error %d" % n)
        return pts[:n].copy(), wts[:n].copy()

    def integrate_subdiv(self, lset_coefs, dt, order, subdivlvl, ex=0, ey=0, ez=0, defined_on=None):
        c = np.ascontiguousarray(lset_coefs, dtype=np.float64)
        d = None if defined_on is None else np.ascontiguousarray(defined_on, dtype=np.uint64)
        st = ctypes.c_int(0)
        v = lib().orc_integrate_subdiv(self.h, _p(c), dt, order, subdivlvl, ex, ey, ez, _p(d), ctypes.byref(st))
        if st.value:
            raise RuntimeError("oracle subdivision rule error %d" % st.value)
        return v

    def mlset_assemble(self, lsets, terms, patch_terms=(), nthreads=1):
        """Terms on regions of several level sets (lsets: M x nv vertex values;
        terms: dicts kind, tuples (ntup x M), coef, hpow, order, normal_lset, b,
        defined_on) and patch terms; CSR triple over all dofs."""
        L = np.ascontiguousarray(lsets, dtype=np.float64)
        M = L.shape[0]
        arr = (MlTerm * len(terms))()
        keep = []
        for i, t in enumerate(terms):
            arr[i].kind, arr[i].order = t["kind"], t.get("order", -1)
            arr[i].hpow, arr[i].normal_lset = t.get("hpow", 0), t.get("normal_lset", 0)
            arr[i].coef = t.get("coef", 1.0)
            for k in range(3):
                arr[i].b[k] = t.get("b", (0.0, 0.0, 0.0))[k]
            tup = np.ascontiguousarray(np.array(t["tuples"], dtype=np.int32).reshape(-1, M))
            keep.append(tup)
            arr[i].ntup, arr[i].dts = tup.shape[0], tup.ctypes.data
            d = t.get("defined_on")
            if d is not None:
                d = np.ascontiguousarray(d, dtype=np.uint64)
                keep.append(d)
            arr[i].defined_on = d.ctypes.data if d is not None else None
        parr, pkeep = self._terms(list(patch_terms))
        c = lib().orc_mlset_assemble(self.h, M, _p(L), ctypes.cast(arr, ctypes.c_void_p), len(terms),
                                     ctypes.cast(parr, ctypes.c_void_p), len(patch_terms), nthreads)
        if not c:
            raise RuntimeError("oracle mlset assembly error")
        nnz = lib().orc_csr_nnz(c)
        rowptr = np.zeros(self.ndof + 1, dtype=np.int64)
        cols = np.zeros(nnz, dtype=np.int32)
        vals = np.zeros(nnz)
        lib().orc_csr_get(c, _p(rowptr), _p(cols), _p(vals))
        lib().orc_csr_destroy(c)
        return rowptr, cols, vals

    def facet_matrix(self, lset, terms, f, dn_fd=False):
        """Patch and skeleton terms of facet f ((2n)^2, row = test)."""
        arr, keep = self._terms(terms)
        n = 2 * self.ndof_el
        out = np.zeros((n, n))
        l = None if lset is None else np.ascontiguousarray(lset, dtype=np.float64)
        r = lib().orc_facet_matrix(self.h, _p(l), ctypes.cast(arr, ctypes.c_void_p), len(terms), f, int(dn_fd),
                                   _p(out))
        if r:
            raise RuntimeError("oracle facet matrix error %d" % r)
        return out

    def assemble(self, lset, terms, nthreads=1, dn_fd=False, bterms=(), cterms=(), theta_patch=None):
        """Returns scipy-free CSR triple (rowptr int64, cols int32, vals float64) over all dofs.
        bterms: boundary terms (dicts: domain, coef, order, hpow, defined_on
        over the BND elements), mass terms of orc_assemble_bnd.  cterms:
        volume terms with a coefficient field (dicts: kind, domain, coef,
        order, hpow, b, e, gf_order, gf_el [ne][nd_gf], defined_on)."""
        arr, keep = self._terms(terms)
        l = np.ascontiguousarray(lset, dtype=np.float64)
        barr = (BTerm * max(len(bterms), 1))()
        for i, t in enumerate(bterms):
            barr[i].kind = TERM_MASS
            barr[i].domain = t["domain"]
            barr[i].order = t.get("order", -1)
            barr[i].hpow = t.get("hpow", 0)
            barr[i].coef = t.get("coef", 1.0)
            d = t.get("defined_on")
            if d is not None:
                d = np.ascontiguousarray(d, dtype=np.uint64)
                keep.append(d)
            barr[i].defined_on = d.ctypes.data if d is not None else None
        carr = (CTerm * max(len(cterms), 1))()
        for i, t in enumerate(cterms):
            carr[i].kind = t["kind"]
            carr[i].domain = t.get("domain", NEG)
            carr[i].order = t.get("order", -1)
            carr[i].hpow = t.get("hpow", 0)
            carr[i].coef = t.get("coef", 1.0)
            for k in range(3):
                carr[i].b[k] = t.get("b", (0.0, 0.0, 0.0))[k]
                carr[i].e[k] = t.get("e", (0, 0, 0))[k]
            g = t.get("gf_el")
            if g is not None:
                g = np.ascontiguousarray(g, dtype=np.float64)
                keep.append(g)
                carr[i].gf_order = t["gf_order"]
            carr[i].gf_el = g.ctypes.data if g is not None else None
            d = t.get("defined_on")
            if d is not None:
                d = np.ascontiguousarray(d, dtype=np.uint64)
                keep.append(d)
            carr[i].defined_on = d.ctypes.data if d is not None else None
            th = t.get("theta_el")
            if th is not None:
                th = np.ascontiguousarray(th, dtype=np.float64)
                keep.append(th)
            carr[i].theta_el = th.ctypes.data if th is not None else None
        tp = None if theta_patch is None else np.ascontiguousarray(theta_patch, dtype=np.float64)
        c = lib().orc_assemble_full(self.h, _p(l), ctypes.cast(arr, ctypes.c_void_p), len(terms),
                                    ctypes.cast(barr, ctypes.c_void_p), len(bterms),
                                    ctypes.cast(carr, ctypes.c_void_p), len(cterms), _p(tp), nthreads, int(dn_fd))
        if not c:
            raise RuntimeError("oracle assembly error")
        nnz = lib().orc_csr_nnz(c)
        rowptr = np.zeros(self.ndof + 1, dtype=np.int64)
        cols = np.zeros(nnz, dtype=np.int32)
        vals = np.zeros(nnz)
        lib().orc_csr_get(c, _p(rowptr), _p(cols), _p(vals))
        lib().orc_csr_destroy(c)
        return rowptr, cols, vals

    # ---- space-time: lset_st is (kt+1, nv) time-major
    def cutinfo_st(self, lset_st, kt, nthreads=1):
        ne = self.mesh.ne
        nw = (ne + 63) // 64
        dom = np.zeros(ne, dtype=np.uint8)
        ratio = np.zeros(ne)
        bits = np.zeros((8, nw), dtype=np.uint64)
        l = np.ascontiguousarray(lset_st, dtype=np.float64)
        r = lib().orc_cutinfo_st(self.h, _p(l), kt, _p(dom), _p(ratio), _p(bits), nthreads)
        if r:
            raise RuntimeError("oracle space-time cutinfo error %d" % r)
        return dom, ratio, bits

    def integrate_st(self, lset_st, kt, dt, order_space, order_time):
        l = np.ascontiguousarray(lset_st, dtype=np.float64)
        return lib().orc_integrate_st(self.h, _p(l), kt, dt, order_space, order_time)

    def st_element_matrix(self, lset_st, kt_l, kt, order_time, terms, e):
        arr, keep = _st_terms(terms)
        n = self.ndof_el * (kt + 1)
        out = np.zeros((n, n))
        l = np.ascontiguousarray(lset_st, dtype=np.float64)
        r = lib().orc_st_element_matrix(self.h, _p(l), kt_l, kt, order_time, ctypes.cast(arr, ctypes.c_void_p),
                                        len(terms), e, _p(out))
        if r:
            raise RuntimeError("oracle space-time element matrix error %d" % r)
        return out

    def assemble_st(self, lset_st, kt_l, kt, order_time, terms, nthreads=1):
        arr, keep = _st_terms(terms)
        l = np.ascontiguousarray(lset_st, dtype=np.float64)
        c = lib().orc_assemble_st(self.h, _p(l), kt_l, kt, order_time, ctypes.cast(arr, ctypes.c_void_p), len(terms),
                                  nthreads)
        if not c:
            raise RuntimeError("oracle space-time assembly error")
        nnz = lib().orc_csr_nnz(c)
        rowptr = np.zeros(self.ndof * (kt + 1) + 1, dtype=np.int64)
        cols = np.zeros(nnz, dtype=np.int32)
        vals = np.zeros(nnz)
        lib().orc_csr_get(c, _p(rowptr), _p(cols), _p(vals))
        lib().orc_csr_destroy(c)
        return rowptr, cols, vals

    def pipeline(self, lset, terms, ghost_facets=True, nthreads=1):
        arr, keep = self._terms(terms)
        l = np.ascontiguousarray(lset, dtype=np.float64)
        return lib().orc_pipeline(self.h, _p(l), ctypes.cast(arr, ctypes.c_void_p), len(terms), int(ghost_facets),
                                  nthreads)

"""Several level sets: the oracle's restatement of StraightCutsIntegrationRule
/ CreateMultiLevelsetCutIntegrationRule (oracle/xg_oracle_mlset.cpp) against
the closed-form answers of ngsxfem's tests/pytests/test_mlset_integration.py
(tests/golden/known_answers.json), the product's rule code
(csrc/xg_mlset.cuh, host build) against the oracle bit for bit, and the
region algebra of ngsxfem_gb300.mlset.  CPU only."""
import itertools
import json
import os
import shutil
import subprocess

import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh
from ngsxfem_gb300.mlset import DomainTypeArray, TensorIntersection, TensorUnion
from ngsxfem_gb300.xfem import ANY, IF, NEG, POS

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
KA = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))


def lsets_2d(orc, n=7):
    b = KA["mlset2d"]["box"]
    m = MakeStructured2DMesh(n, n, b[0][0], b[0][1], b[1][0], b[1][1])
    X, Y = m.coords[:, 0], m.coords[:, 1]
    return m, np.array([orc.interpolate_p1_perturb(f) for f in (Y - 1, 2 * X - Y, -2 * X - Y)])


def lsets_3d(orc, n=5):
    b = KA["mlset3d"]["box"]
    m = MakeStructured3DMesh(n, box=(tuple(b),) * 3)
    X, Y, Z = m.coords.T
    return m, np.array([orc.interpolate_p1_perturb(f) for f in (X - .5, X + .5, Y - .5, Y + .5, Z - .5, Z + .5)])


def integ(orc, m, L, region, order=0, exps=(0, 0, 0)):
    tuples = region.as_list if isinstance(region, DomainTypeArray) else region
    v, st = orc.mlset_integrate(m, L, tuples, order, exps)
    assert st == 0
    return v


def x_plus_y(orc, m, L, region, dim=2):
    return sum(integ(orc, m, L, region, 0, e) for e in ((1, 0, 0), (0, 1, 0), (0, 0, 1))[:dim])


def test_2d_triangle_of_three_lines(orc):
    ref, tol = KA["mlset2d"], KA["mlset2d"]["tol"]
    m, L = lsets_2d(orc)
    tri = DomainTypeArray((NEG, NEG, NEG))
    assert abs(integ(orc, m, L[:1], [(NEG,)]) - ref["area_neg0"]) < tol
    assert abs(integ(orc, m, L, tri) - ref["triangle"]) < tol
    assert abs(integ(orc, m, L, ~tri) - ref["complement"]) < tol
    assert abs(integ(orc, m, L, [(IF, NEG, NEG)]) - ref["side_t"]) < tol
    assert abs(integ(orc, m, L, [(NEG, IF, NEG)]) - ref["side_r"]) < tol
    assert abs(integ(orc, m, L, [(NEG, NEG, IF)]) - ref["side_l"]) < tol
    assert abs(integ(orc, m, L, tri.Boundary()) - ref["perimeter"]) < tol
    pts = ref["x_plus_y"]
    assert abs(x_plus_y(orc, m, L, [(IF, IF, NEG)]) - pts["tl"]) < tol
    assert abs(x_plus_y(orc, m, L, [(IF, NEG, IF)]) - pts["tr"]) < tol
    assert abs(x_plus_y(orc, m, L, [(NEG, IF, IF)]) - pts["b"]) < tol
    assert abs(x_plus_y(orc, m, L, tri.Boundary().Boundary()) - pts["corners"]) < tol


def test_2d_higher_order_square(orc):
    ref = KA["mlset2d_ho"]
    b = ref["box"]
    m = MakeStructured2DMesh(5, 5, b[0][0], b[0][1], b[1][0], b[1][1])
    X, Y = m.coords[:, 0], m.coords[:, 1]
    L = np.array([orc.interpolate_p1_perturb(f) for f in (-Y, X - 1, Y - 1, -X)])
    sq = [(NEG,) * 4]
    # x (1 - x) y (1 - y) = x y - x^2 y - x y^2 + x^2 y^2
    v = sum(s * integ(orc, m, L, sq, 4, e) for e, s in (((1, 1, 0), 1), ((2, 1, 0), -1), ((1, 2, 0), -1),
                                                           ((2, 2, 0), 1)))
    assert abs(v - ref["value"]) < ref["tol"]


def test_2d_overlapping_unions(orc):
    """Three descriptions of one region (union with overlaps, ANY, algebra)
    integrate to the same area."""
    m = MakeStructured2DMesh(24, 24, -1.1, 1.1, -1.1, 1.1)
    X, Y = m.coords[:, 0], m.coords[:, 1]
    L = np.array([orc.interpolate_p1_perturb(f) for f in (X * X + Y * Y - 1, -X - 1 / 3, X - 1 / 3, Y - 0.5)])
    z1 = DomainTypeArray([(NEG, NEG, NEG, POS), (NEG, POS, NEG, POS), (NEG, POS, NEG, NEG), (NEG, NEG, POS, NEG),
                          (NEG, NEG, POS, POS)])
    z2 = DomainTypeArray([(NEG, ANY, ANY, POS), (NEG, POS, ANY, ANY), (NEG, ANY, POS, ANY)])
    z3 = DomainTypeArray((NEG, ANY, ANY, ANY)) & ~DomainTypeArray((NEG, NEG, NEG, NEG))
    a1, a2, a3 = (integ(orc, m, L, z) for z in (z1, z2, z3))
    assert abs(a1 - a2) < 1e-12 and abs(a1 - a3) < 1e-12


def test_3d_cube_of_six_planes(orc):
    ref, tol = KA["mlset3d"], KA["mlset3d"]["tol"]
    m, L = lsets_3d(orc)
    cube = DomainTypeArray([(NEG, POS, NEG, POS, NEG, POS)])
    assert abs(integ(orc, m, L, cube) - ref["cube"]) < tol
    assert abs(integ(orc, m, L, ~cube) - ref["complement"]) < tol
    sides = []
    for i in range(6):
        d = [NEG, POS, NEG, POS, NEG, POS]
        d[i] = IF
        sides.append(tuple(d))
        assert abs(integ(orc, m, L, [tuple(d)]) - ref["side"]) < tol
    assert sorted(cube.Boundary().as_list) == sorted(sides)
    assert abs(integ(orc, m, L, cube.Boundary()) - ref["surface"]) < tol
    assert abs(integ(orc, m, L, cube.Boundary().Boundary()) - ref["edges"]) < tol
    edge = (IF, POS, IF, POS, NEG, POS)
    assert abs(integ(orc, m, L, [edge]) - ref["edge"]) < tol
    for key, val in ref["corners_x_plus_y_plus_z"].items():
        d = []
        for s, (a, b) in zip(key, ((0, 1), (2, 3), (4, 5))):
            d += [IF, POS] if s == "p" else [NEG, IF]
        assert abs(x_plus_y(orc, m, L, [tuple(d)], 3) - val) < tol, key


def test_region_algebra():
    tri = DomainTypeArray((NEG, NEG, NEG))
    assert len(~tri) == 7 and tri not in [] and (NEG, NEG, NEG) in tri
    assert sorted(tri.Boundary().as_list) == [(NEG, NEG, IF), (NEG, IF, NEG), (IF, NEG, NEG)]
    assert (tri | DomainTypeArray((POS, NEG, NEG))) == DomainTypeArray((ANY, NEG, NEG))
    # intersection of a volume and a side: the side
    assert (tri & DomainTypeArray((IF, NEG, NEG))) == DomainTypeArray((IF, NEG, NEG))
    # two volumes that differ in one entry meet on its interface
    assert (DomainTypeArray((NEG, NEG)) & DomainTypeArray((NEG, IF))) == DomainTypeArray((NEG, IF))
    tu = TensorUnion(DomainTypeArray((NEG,)), DomainTypeArray((POS,)))
    assert tu == DomainTypeArray([(NEG, ANY), (ANY, POS)])
    ti = TensorIntersection(DomainTypeArray((NEG,)), DomainTypeArray([(POS,), (NEG,)]))
    assert ti == DomainTypeArray((NEG, ANY))
    with pytest.raises(ValueError):
        DomainTypeArray([(NEG, IF), (NEG, NEG)])
    with pytest.raises(ValueError):
        DomainTypeArray((NEG, IF)) | DomainTypeArray((NEG, NEG))
    cube = DomainTypeArray((NEG, POS, NEG, POS, NEG, POS))
    with pytest.raises(ValueError):
        cube.Boundary().Boundary().Boundary().Boundary()


def test_device_rule_code_matches_oracle_bitwise(orc, tmp_path):
    """csrc/xg_mlset.cuh compiled as host code against the oracle
    (tests/native/mlset_rule_check.cu)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    libdir = os.path.dirname(orc.LIB)
    exe = str(tmp_path / "mlset_rule_check")
    subprocess.check_call([nvcc, "-x", "cu", "-std=c++17", "-O1", "-Xcompiler", "-ffp-contract=off",
                           "-diag-suppress", "20011,20014", "-I", os.path.join(ROOT, "ngsxfem_gb300", "csrc"),
                           "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "native", "mlset_rule_check.cu"),
                           "-L", libdir, "-loracle", "-Xlinker", "-rpath", "-Xlinker", libdir, "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout


def test_c_abi_rejects_bad_domains():
    """Argument checks of xg_integrate_mlset / xg_cut_rules_mlset run before
    any device work."""
    import ctypes
    from ngsxfem_gb300 import _lib
    L = _lib.load()
    P = ctypes.c_void_p
    tup = np.array([[NEG, NEG]], dtype=np.int8)
    assert L.xg_integrate_mlset(None, P(8), 2, tup.ctypes.data_as(P), 1, 0, 0, 0, 0, None, P(8), None) == 1
    assert L.xg_mlset_rule_capacity(2, 2, 1, 0) == 9
    assert L.xg_mlset_rule_capacity(2, 9, 1, 0) == -1
    assert L.xg_mlset_rule_capacity(4, 2, 1, 0) == -1


def test_marker_relations(orc):
    """MultiLevelsetCutInfo relations asserted by test_mlset_integration.py,
    on the oracle's markers."""
    m, L = lsets_2d(orc)
    tri = DomainTypeArray((NEG, NEG, NEG))
    neg = orc.mlset_mark(m, L, tri.as_list, 0)
    hasneg = orc.mlset_mark(m, L, tri.as_list, 1)
    not_neg = orc.mlset_mark(m, L, (~tri).as_list, 1)
    if_ = orc.mlset_mark(m, L, tri.Boundary().as_list, 1)
    assert neg.any() and if_.any()
    assert (~neg == not_neg).all()
    assert (if_ == (hasneg & ~neg)).all()
    m3, L3 = lsets_3d(orc)
    cube = DomainTypeArray((NEG, POS, NEG, POS, NEG, POS))
    neg3 = orc.mlset_mark(m3, L3, cube.as_list, 0)
    has3 = orc.mlset_mark(m3, L3, cube.as_list, 1)
    if3 = orc.mlset_mark(m3, L3, cube.Boundary().as_list, 1)
    assert (~neg3 == orc.mlset_mark(m3, L3, (~cube).as_list, 1)).all()
    assert (if3 == (has3 & ~neg3)).all()
    sides = np.zeros_like(if3)
    for t in cube.Boundary().as_list:
        sides |= orc.mlset_mark(m3, L3, [t], 1)
    assert (sides == if3).all()


def lines_cases():
    """The three line regions of test_mlset_integration.py::test_3d_codim2_cross
    as (level-set functions, region tuples, key); on meshes with different x
    and y grids (an equal grid puts mesh faces on the plane x = y)."""
    return [
        (lambda X, Y, Z: (X - .5, X + .5, X - Y, Z), [(NEG, POS, IF, IF)], "line"),
        (lambda X, Y, Z: (X - .5, -X - .5, Z - Y, X - Z, X + Z), [(NEG, NEG, IF, IF, ANY), (NEG, NEG, IF, ANY, IF)],
         "cross"),
        (lambda X, Y, Z: (X - .5, -X - .5, -Z - .5, Z + Y, X + Y, Z + Y + .1),
         [(NEG, NEG, NEG, IF, IF, ANY), (NEG, NEG, NEG, ANY, IF, IF)], "lines"),
    ]


def test_3d_line_lengths(orc):
    ref = KA["mlset3d_lines"]
    for dims in ((5, 6, 7), (7, 9, 11)):
        m = MakeStructured3DMesh(*dims, box=((-0.8, 0.8),) * 3)
        for fs, tuples, key in lines_cases():
            L = np.array([orc.interpolate_p1_perturb(f) for f in fs(*m.coords.T)])
            assert abs(integ(orc, m, L, DomainTypeArray(tuples)) - ref[key]) < ref["tol"], (dims, key)


@pytest.mark.parametrize("k", [1, 2, 3])
def test_mlset_forms_known_answers(orc, k):
    """orc_mlset_assemble on the unit square as the region of four lines:
    1^T M 1 = 1 (area), the boundary pieces' mass sums to the perimeter 4,
    the stiffness matrix annihilates constants and x^T K x = |region|."""
    m = MakeStructured2DMesh(7, 7, -0.2, 1.2, -0.2, 1.2)
    X, Y = m.coords.T
    L = np.stack([orc.interpolate_p1_perturb(v) for v in (-Y, X - 1, Y - 1, -X)])
    sp = orc.Space(m, k)
    NEG, IF = orc.NEG, orc.IF
    sq = [(NEG,) * 4]
    bnd = [(IF, NEG, NEG, NEG), (NEG, IF, NEG, NEG), (NEG, NEG, IF, NEG), (NEG, NEG, NEG, IF)]
    one = np.zeros(sp.ndof)
    xs = np.zeros(sp.ndof)
    el = sp.el_dofs()
    for e in range(m.ne):
        one[el[e][:3]] = 1.0
        xs[el[e][:3]] = m.coords[m.elements[e], 0]

    def dense(csr):
        rp, cols, vals = csr
        A = np.zeros((sp.ndof, sp.ndof))
        for r in range(sp.ndof):
            A[r, cols[rp[r]:rp[r + 1]]] += vals[rp[r]:rp[r + 1]]
        return A
    Mm = dense(sp.mlset_assemble(L, [dict(kind=orc.TERM_MASS, tuples=sq)]))
    assert abs(one @ Mm @ one - 1.0) < 1e-13
    Mb = dense(sp.mlset_assemble(L, [dict(kind=orc.TERM_MASS, tuples=bnd)]))
    assert abs(one @ Mb @ one - 4.0) < 1e-13
    K = dense(sp.mlset_assemble(L, [dict(kind=orc.TERM_LAPLACE, tuples=sq)]))
    assert np.abs(K @ one).max() < 1e-12
    assert abs(xs @ K @ xs - 1.0) < 1e-13

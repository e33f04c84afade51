"""Several level sets on the GPU (xg_integrate_mlset, xg_cut_rules_mlset)
against the oracle's restatement of CreateMultiLevelsetCutIntegrationRule /
StraightCutsIntegrationRule and against the closed forms of ngsxfem's
tests/pytests/test_mlset_integration.py.

Bars: integrals within 1e-12 of the closed forms and within 1e-12 relative of
the oracle; rule counts equal, points within 1e-14, weights within 1e-13
relative (the rule code equals the oracle's to the bit on the same table,
tests/test_oracle_mlset.py; the two base-rule tables agree to ~4e-16)."""
import itertools
import json
import os

import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))


def gfs(xg, mesh, vals):
    sp = xg.H1(mesh, order=1)
    out = []
    for v in vals:
        g = xg.GridFunction(sp)
        g.vec.copy_(torch.from_numpy(np.ascontiguousarray(v, dtype=np.float64)))
        out.append(g)
    return tuple(out)


def integ(xg, mesh, G, region, order=0, exps=(0, 0, 0)):
    cf = xg.x ** exps[0] * xg.y ** exps[1] * xg.z ** exps[2] if any(exps) else None
    return xg.Integrate(levelset_domain={"levelset": G, "domain_type": region}, cf=cf, mesh=mesh, order=order)


def test_2d_triangle(xg, orc):
    from ngsxfem_gb300.mlset import DomainTypeArray
    ref, tol = KA["mlset2d"], KA["mlset2d"]["tol"]
    b = ref["box"]
    m = MakeStructured2DMesh(7, 7, b[0][0], b[0][1], b[1][0], b[1][1])
    X, Y = m.coords[:, 0], m.coords[:, 1]
    G = gfs(xg, m, [orc.interpolate_p1_perturb(f) for f in (Y - 1, 2 * X - Y, -2 * X - Y)])
    tri = DomainTypeArray((xg.NEG, xg.NEG, xg.NEG))
    assert abs(integ(xg, m, G, tri) - ref["triangle"]) < tol
    assert abs(integ(xg, m, G, ~tri) - ref["complement"]) < tol
    assert abs(integ(xg, m, G, tri.Boundary()) - ref["perimeter"]) < tol
    corners = tri.Boundary().Boundary()
    assert abs(integ(xg, m, G, corners, 0, (1, 0, 0)) + integ(xg, m, G, corners, 0, (0, 1, 0)) -
               ref["x_plus_y"]["corners"]) < tol


def test_3d_cube(xg, orc):
    from ngsxfem_gb300.mlset import DomainTypeArray
    ref, tol = KA["mlset3d"], KA["mlset3d"]["tol"]
    b = ref["box"]
    m = MakeStructured3DMesh(5, box=(tuple(b),) * 3)
    X, Y, Z = m.coords.T
    G = gfs(xg, m, [orc.interpolate_p1_perturb(f) for f in (X - .5, X + .5, Y - .5, Y + .5, Z - .5, Z + .5)])
    N, P = xg.NEG, xg.POS
    cube = DomainTypeArray((N, P, N, P, N, P))
    assert abs(integ(xg, m, G, cube) - ref["cube"]) < tol
    assert abs(integ(xg, m, G, ~cube) - ref["complement"]) < tol
    assert abs(integ(xg, m, G, cube.Boundary()) - ref["surface"]) < tol
    assert abs(integ(xg, m, G, cube.Boundary().Boundary()) - ref["edges"]) < tol
    ppp = (xg.IF, P, xg.IF, P, xg.IF, P)
    v = sum(integ(xg, m, G, ppp, 0, e) for e in ((1, 0, 0), (0, 1, 0), (0, 0, 1)))
    assert abs(v - ref["corners_x_plus_y_plus_z"]["ppp"]) < tol


def random_case(D, seed):
    rng = np.random.default_rng(seed)
    m = MakeStructured2DMesh(9, 8) if D == 2 else MakeStructured3DMesh(4, 4, 3)
    M = 3
    # planes and a sphere-like quadric through the mesh
    vals = [m.coords @ rng.standard_normal(D) + rng.uniform(-0.3, 0.3) for _ in range(M - 1)]
    vals.append(((m.coords - 0.5) ** 2).sum(1) - 0.1)
    tuples = [t for t in itertools.product((0, 1, 2), repeat=M) if rng.uniform() < 0.4] or [(0, 0, 0)]
    return m, np.array(vals), tuples


@pytest.mark.parametrize("D,seed", [(2, 1), (2, 2), (3, 3), (3, 4)])
def test_integrate_matches_oracle(xg, orc, D, seed):
    m, L, tuples = random_case(D, seed)
    L = np.array([orc.interpolate_p1_perturb(v) for v in L])
    G = gfs(xg, m, L)
    for codim in range(D + 1):
        region = [t for t in tuples if t.count(2) == codim]
        if not region:
            continue
        for order in (0, 2, 4):
            ref, st = orc.mlset_integrate(m, L, region, order, (1, 0, 0))
            assert st == 0
            v = integ(xg, m, G, region, order, (1, 0, 0))
            assert abs(v - ref) <= 1e-12 * max(1.0, abs(ref)), (codim, order, v, ref)


@pytest.mark.parametrize("D,seed", [(2, 5), (3, 6)])
def test_rules_match_oracle(xg, orc, D, seed):
    m, L, tuples = random_case(D, seed)
    L = np.array([orc.interpolate_p1_perturb(v) for v in L])
    G = gfs(xg, m, L)
    els = np.arange(m.ne, dtype=np.int32)
    for codim in range(D + 1):
        region = [t for t in tuples if t.count(2) == codim]
        if not region:
            continue
        counts, pts, wts = xg.MultiLevelsetCutIntegrationRules(m, G, region, els, 2)
        counts, pts, wts = counts.cpu().numpy(), pts.cpu().numpy(), wts.cpu().numpy()
        for e in range(m.ne):
            vtx = m.elements[e]
            r = orc.mlset_cut_rule(m.coords[vtx], L[:, vtx], region, 2)
            if r is None:
                assert counts[e] == -1, (e, counts[e])
                continue
            n = len(r[1])
            assert counts[e] == n, (e, counts[e], n)
            assert np.max(np.abs(pts[e, :n] - r[0]), initial=0) <= 1e-14
            assert np.max(np.abs(wts[e, :n] - r[1]) / np.maximum(1e-300, np.abs(r[1])), initial=0) <= 1e-13


def test_multilevelset_cutinfo(xg, orc):
    """MultiLevelsetCutInfo markers against the oracle's, and the Update
    semantics of test_mlset_integration.py::test_multilevelsetcutinfo."""
    from ngsxfem_gb300.mlset import DomainTypeArray, MultiLevelsetCutInfo
    ref = KA["mlset2d"]
    b = ref["box"]
    m = MakeStructured2DMesh(7, 7, b[0][0], b[0][1], b[1][0], b[1][1])
    X, Y = m.coords[:, 0], m.coords[:, 1]
    L = np.array([orc.interpolate_p1_perturb(f) for f in (Y - 1, 2 * X - Y, -2 * X - Y)])
    G = gfs(xg, m, L)
    mlci = MultiLevelsetCutInfo(m, G)
    tri = DomainTypeArray((xg.NEG, xg.NEG, xg.NEG))
    for region in (tri, ~tri, tri.Boundary(), tri.Boundary().Boundary()):
        for mode, get in ((0, mlci.GetElementsOfType), (1, mlci.GetElementsWithContribution)):
            assert (get(region).numpy() == orc.mlset_mark(m, L, region.as_list, mode)).all()
    neg = mlci.GetElementsOfType(tri).numpy()
    assert (mlci.GetElementsWithContribution(tri.Boundary()).numpy() ==
            (mlci.GetElementsWithContribution(tri).numpy() & ~neg)).all()
    # markers follow Update, not the level sets they were built from
    m2 = MakeStructured2DMesh(10, 10, -1, 1, -1, 1)
    X2, Y2 = m2.coords[:, 0], m2.coords[:, 1]
    H = gfs(xg, m2, [X2 + 0.5, X2 - 0.5])
    ci = MultiLevelsetCutInfo(m2, H)
    a0 = ci.GetElementsOfType((xg.POS, xg.NEG)).numpy().copy()
    for g, v in zip(H, (Y2 + 0.5, Y2 - 0.5)):
        g.vec.copy_(torch.from_numpy(v))
    assert (ci.GetElementsOfType((xg.POS, xg.NEG)).numpy() == a0).all()
    ci.Update(H)
    assert not (ci.GetElementsOfType((xg.POS, xg.NEG)).numpy() == a0).all()
    with pytest.raises(ValueError):
        ci.GetElementsOfType((xg.NEG, xg.NEG, xg.NEG))
    with pytest.raises(TypeError):
        MultiLevelsetCutInfo(m2, (1.0, 2.0))


def test_3d_line_lengths(xg, orc):
    """Lines (codimension 2) of test_mlset_integration.py::test_3d_codim2_cross."""
    from ngsxfem_gb300.mlset import DomainTypeArray
    ref = KA["mlset3d_lines"]
    m = MakeStructured3DMesh(5, 6, 7, box=((-0.8, 0.8),) * 3)
    N, P, I, A = xg.NEG, xg.POS, xg.IF, xg.ANY
    X, Y, Z = m.coords.T
    G = gfs(xg, m, [orc.interpolate_p1_perturb(f) for f in (X - .5, -X - .5, Z - Y, X - Z, X + Z)])
    cross = DomainTypeArray([(N, N, I, I, A), (N, N, I, A, I)])
    assert abs(integ(xg, m, G, cross) - ref["cross"]) < ref["tol"]

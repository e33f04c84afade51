"""libxg's quadrilateral / hexahedral cut rules and Integrate (GPU, through the
C ABI: xg_mesh_create_tensor, xg_integrate_ex, xg_cut_rules_ex) against the
oracle's restatement of LevelsetCutQuadrilateral and against the closed-form
answers of ngsxfem's quad / hex tests.

Bars: rule counts equal; points within 1e-14 and weights within 1e-13
relative (the product's and the oracle's base rules agree to ~4e-16, and the
rule code is bit-identical to the oracle's on the same table, which
tests/test_oracle_quad.py checks on the CPU); integrals within 1e-12 relative
to the oracle and within 5e-15 (p+1)^2 of the closed forms."""
import json
import math
import os

import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import Mesh, MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))
DTS = (("NEG", 0), ("POS", 1), ("IF", 2))


def vlset(orc, mesh, f):
    return orc.interpolate_p1_perturb(np.array([f(*p) for p in mesh.coords]))


def planar(coef):
    return lambda *x: coef[0] + sum(c * xi for c, xi in zip(coef[1:], x))


def gpu_integrate(xg, mesh, l, dt, order, policy=1, exps=(0, 0, 0)):
    sp = xg.H1(mesh, order=1)
    gf = xg.GridFunction(sp)
    gf.vec.copy_(torch.from_numpy(np.ascontiguousarray(l, dtype=np.float64)))
    lsd = {"levelset": gf, "domain_type": dt, "quad_dir_policy": policy}
    return xg.Integrate(levelset_domain=lsd, cf=xg.x ** exps[0] * xg.y ** exps[1] * xg.z ** exps[2]
                        if any(exps) else None, mesh=mesh, order=order)


def deformed_quads(n, seed):
    """n x n quads of [0,1]^2 with the interior vertices moved (bilinear maps
    with a varying Jacobian)."""
    m = MakeStructured2DMesh(quads=True, nx=n, ny=n)
    c = m.coords.copy()
    rng = np.random.default_rng(seed)
    inner = (c[:, 0] > 0) & (c[:, 0] < 1) & (c[:, 1] > 0) & (c[:, 1] < 1)
    c[inner] += rng.uniform(-0.2, 0.2, (inner.sum(), 2)) / n
    return Mesh(c, m.elements)


def deformed_hexes(n, seed):
    m = MakeStructured3DMesh(n, hexes=True)
    c = m.coords.copy()
    rng = np.random.default_rng(seed)
    inner = np.all((c > 0) & (c < 1), axis=1)
    c[inner] += rng.uniform(-0.15, 0.15, (inner.sum(), 3)) / n
    return Mesh(c, m.elements)


@pytest.mark.parametrize("N", KA["planar2d"]["N"])
def test_planar_quads(xg, orc, N):
    m = MakeStructured2DMesh(quads=True, nx=N, ny=N)
    l = vlset(orc, m, planar(KA["planar2d"]["lset"]))
    for order in KA["planar2d"]["orders"]:
        for name, dt in DTS:
            v = gpu_integrate(xg, m, l, dt, order)
            assert abs(v - KA["planar2d"]["values"][name]) < 5e-15 * (order + 1) ** 2, (order, name, v)


@pytest.mark.parametrize("N", [1, 2])
def test_planar_hexes(xg, orc, N):
    m = MakeStructured3DMesh(N, hexes=True)
    l = vlset(orc, m, planar(KA["planar3d"]["lset"]))
    for order in KA["planar3d"]["orders"]:
        for name, dt in DTS:
            v = gpu_integrate(xg, m, l, dt, order)
            assert abs(v - KA["planar3d"]["values"][name]) < 5e-15 * (order + 1) ** 2, (order, name, v)


def test_hex_monomials_and_zero_value(xg, orc):
    m = MakeStructured3DMesh(KA["quad3d_mono"]["N"], hexes=True)
    l = vlset(orc, m, planar(KA["planar3d"]["lset"]))
    for ref in KA["mono3d"]:
        for d in range(3):
            e = [0, 0, 0]
            e[d] = ref["alpha"]
            for name, dt in DTS[:2]:
                assert abs(gpu_integrate(xg, m, l, dt, 4, exps=e) - ref[name]) < 5e-15 * 25
    z = KA["zero_val"]
    m2 = MakeStructured3DMesh(z["N"], hexes=True)
    l2 = vlset(orc, m2, planar(KA["planar3d"]["lset"]))
    assert abs(gpu_integrate(xg, m2, l2, 1, z["order"], exps=(z["alpha"], 0, 0)) - z["POS"]) < 5e-15 * 25


CASES = {
    "circle_quads": lambda orc: (lambda m: (m, vlset(orc, m, lambda x, y: math.hypot(x, y) - 0.6)))(
        MakeStructured2DMesh(quads=True, nx=24, ny=24)),
    "random_quads": lambda orc: (lambda m: (m, np.random.default_rng(3).standard_normal(m.nv) + 0.2))(
        deformed_quads(9, 5)),
    "sphere_hexes": lambda orc: (lambda m: (m, vlset(orc, m, lambda x, y, z: math.sqrt(x * x + y * y + z * z) - 0.72)))(
        MakeStructured3DMesh(8, hexes=True)),
    "random_hexes": lambda orc: (lambda m: (m, np.random.default_rng(7).standard_normal(m.nv) + 0.1))(
        deformed_hexes(5, 11)),
    "tpmc_10": lambda orc: (lambda m: (m, np.array([x * ((7 * y - 13) * z + 6) + y * (3 - 8 * z) + 8 * z - 4
                                                    for x, y, z in m.coords])))(MakeStructured3DMesh(10, hexes=True)),
}


@pytest.mark.parametrize("case", list(CASES))
@pytest.mark.parametrize("policy", [0, 1, 2])
def test_integrate_matches_oracle(xg, orc, case, policy):
    m, l = CASES[case](orc)
    for order in (0, 2, 5):
        for name, dt in DTS:
            ref, st = orc.quad_integrate(m, l, dt, order, policy=policy)
            if st:
                continue  # an element the reference rejects (interface scaling bound)
            v = gpu_integrate(xg, m, l, dt, order, policy=policy)
            assert abs(v - ref) <= 1e-12 * max(1.0, abs(ref)), (case, order, name, v, ref)


@pytest.mark.parametrize("case", ["random_quads", "random_hexes", "tpmc_10"])
def test_rules_match_oracle(xg, orc, case):
    m, l = CASES[case](orc)
    gf_vals = torch.from_numpy(np.ascontiguousarray(l, dtype=np.float64)).cuda()
    nve = m.elements.shape[1]
    els = np.arange(m.ne, dtype=np.int32)
    for order in (1, 4):
        for policy in (0, 1, 2):
            for name, dt in DTS:
                refs = []
                for e in range(m.ne):
                    xv = np.zeros((nve, 3))
                    xv[:, : m.dim] = m.coords[m.elements[e]]
                    try:
                        refs.append(orc.quad_cut_rule(l[m.elements[e]], dt, order, policy, elcoords=xv))
                    except RuntimeError:
                        refs.append("error")
                try:
                    counts, pts, wts = xg.CutIntegrationRules(m, gf_vals, els, dt, order, quad_dir_policy=policy)
                except RuntimeError as ex:
                    # an element the reference rejects (the interface scaling bound,
                    # straightcutrule.cpp:273-286): the whole call fails, as the oracle does
                    assert "error" in refs, (order, policy, name, ex)
                    continue
                assert "error" not in refs
                counts, pts, wts = counts.cpu().numpy(), pts.cpu().numpy(), wts.cpu().numpy()
                for e, r in enumerate(refs):
                    if r is None:
                        assert counts[e] == -1, (e, counts[e])
                        continue
                    n = len(r[1])
                    assert counts[e] == n, (e, counts[e], n)
                    assert np.max(np.abs(pts[e, :n] - r[0]), initial=0) <= 1e-14
                    assert np.max(np.abs(wts[e, :n] - r[1]) / np.maximum(1e-300, np.abs(r[1])), initial=0) <= 1e-13


def test_tensor_mesh_rejects_simplex_only_calls(xg, orc):
    m = MakeStructured2DMesh(quads=True, nx=3, ny=3)
    with pytest.raises(Exception):
        xg.H1(m, order=2)
    a = xg.BitArray(m.ne)
    with pytest.raises(Exception):
        xg.GetFacetsWithNeighborTypes(m, a, b=a)


def test_rule_capacity_and_bad_element(xg, orc):
    m = MakeStructured2DMesh(quads=True, nx=4, ny=4)
    l = torch.from_numpy(vlset(orc, m, lambda x, y: math.hypot(x - 0.5, y - 0.4) - 0.3)).cuda()
    cut = [e for e in range(m.ne) if len(set(np.sign(l.cpu().numpy()[m.elements[e]]))) > 1]
    # too small a capacity: XG_ERR_CAPACITY from the device, nothing written past max_pts
    with pytest.raises(RuntimeError, match="capacity"):
        xg.CutIntegrationRules(m, l, cut, 0, 4, max_pts=2)
    # an element number outside the mesh: XG_ERR_ARG from the device, no read of it
    with pytest.raises(RuntimeError, match="invalid argument"):
        xg.CutIntegrationRules(m, l, [0, m.ne + 5], 0, 4)
    counts, _, _ = xg.CutIntegrationRules(m, l, cut, 0, 4)
    assert (counts.cpu().numpy() > 0).all()

"""Subdivision cut rules on the GPU (xg_integrate_subdiv, xg_subdiv_moments_tet;
csrc/xg_subdiv.cu[h]) against the oracle's restatement of the reference's
CutIntegrationRule with subdivlvl (orc_integrate_subdiv, orc_subdiv_rule):
integrals within 1e-12 relative on 2D / 3D meshes, level sets of order 1..3,
NEG / POS / IF, levels 0..3; the Python surface (GridFunction.Set, Integrate
with a higher-order level set and subdivlvl); per-element NEG moments of P2
level sets on the reference tetrahedron."""
import ctypes

import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


def quad_lset(D):
    if D == 2:
        return lambda x, y: (x - .5) ** 2 + (y - .47) ** 2 - 0.31 ** 2
    return lambda x, y, z: (x - .5) ** 2 + (y - .47) ** 2 + (z - .52) ** 2 - 0.29 ** 2


def cubic_lset(D):
    if D == 2:
        return lambda x, y: (x - .5) ** 2 + 0.8 * (y - .45) ** 2 + 0.6 * (x - .5) ** 3 - 0.3 ** 2
    return lambda x, y, z: (x - .5) ** 2 + (y - .45) ** 2 + 0.7 * (z - .5) ** 2 + 0.5 * (x - .5) * (y - .5) * (
        z - .5) - 0.28 ** 2


@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("k", [1, 2, 3])
def test_integrate_subdiv_parity(xg, orc, D, k):
    m = MakeStructured2DMesh(9, 8) if D == 2 else MakeStructured3DMesh(4)
    V = xg.H1(m, order=k)
    gf = xg.GridFunction(V)
    gf.Set(cubic_lset(D) if k == 3 else quad_lset(D))
    sp = orc.Space(m, k)
    assert np.array_equal(V.element_dofs(), sp.el_dofs())
    coefs = gf.vec.cpu().numpy()
    res = torch.zeros(1, dtype=torch.float64, device="cuda")
    for dt in (orc.NEG, orc.POS, orc.IF):
        for L in range(4):
            for mono, order in (((0, 0, 0), 0), ((1, 0, 0), 2), ((0, 2, 1), 4)):
                xg._lib.call("xg_integrate_subdiv", V.h, xg._vp(gf.vec), dt, order, L, *mono, None, xg._vp(res),
                             xg._stream())
                torch.cuda.synchronize()
                got = float(res.item())
                ref = orc.Space.integrate_subdiv(sp, coefs, dt, order, L, *mono)
                assert abs(got - ref) <= 1e-12 * max(1.0, abs(ref)), (dt, L, mono, got, ref)
    xg.device_mesh(m).check()


def test_python_integrate_with_subdivision(xg, orc):
    """Integrate(x * dCut(lset_h, NEG, subdivlvl=L)) with a P2 GridFunction set
    from a quadratic level set converges to the exact region's moment."""
    m = MakeStructured2DMesh(10, 10)
    V = xg.H1(m, order=2)
    gf = xg.GridFunction(V).Set(lambda x, y: (x - .5) ** 2 + (y - .5) ** 2 - 0.33 ** 2)
    exact = 0.5 * np.pi * 0.33 ** 2
    errs = []
    for L in range(4):
        v = xg.Integrate(xg.x * xg.dCut(gf, xg.NEG, order=2, subdivlvl=L), m)
        sp = orc.Space(m, 2)
        ref = sp.integrate_subdiv(gf.vec.cpu().numpy(), orc.NEG, 2, L, 1, 0, 0)
        assert abs(v - ref) < 1e-13
        errs.append(abs(v - exact))
    assert all(errs[i] / errs[i + 1] > 3.0 for i in range(3)), errs


def test_subdiv_moments_tet(xg, orc):
    """Per-element NEG moments of P2 level sets on the reference tetrahedron
    against the oracle's rule on a one-element mesh."""
    rng = np.random.default_rng(5)
    n = 60
    vals = rng.standard_normal((n, 10))
    vals[:, :4] += np.where(rng.random((n, 1)) < 0.5, 0.4, -0.4)
    d_v = torch.from_numpy(vals).cuda()
    out = torch.zeros((n, 35), dtype=torch.float64, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    for L in (0, 2, 3):
        xg._lib.call("xg_subdiv_moments_tet", xg._vp(d_v), n, L, xg._vp(out), xg._vp(err), xg._stream())
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        got = out.cpu().numpy()

        class One:
            dim, nv, ne = 3, 4, 1
            coords = np.array([[1.0, 0, 0], [0, 1.0, 0], [0, 0, 1.0], [0, 0, 0]])
            elements = np.array([[0, 1, 2, 3]], dtype=np.int32)
        sp = orc.Space(One, 2)
        edges = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
        for e in range(n):
            c = np.zeros(sp.ndof)
            el = sp.el_dofs()[0]
            loc = list(vals[e, :4]) + [4 * vals[e, 4 + j] - 2 * (vals[e, a] + vals[e, b]) for j, (a, b) in enumerate(edges)]
            c[el] = loc
            P, W = sp.subdiv_rule(c, 0, orc.NEG, 4, L)
            ref = np.zeros(35)
            k = 0
            for t in range(5):
                for a in range(t, -1, -1):
                    for b in range(t - a, -1, -1):
                        ref[k] = np.sum(W * P[:, 0] ** a * P[:, 1] ** b * P[:, 2] ** (t - a - b))
                        k += 1
            assert np.abs(got[e] - ref).max() < 1e-13, (L, e, np.abs(got[e] - ref).max())

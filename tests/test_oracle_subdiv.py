"""Subdivision cut rules of the oracle (orc_integrate_subdiv: the reference's
CutIntegrationRule with subdivlvl, cutint/xintegration.cpp:620-1063,
1626-1754) on higher-order level sets given as H1 coefficients: closed-form
limits (circle area and perimeter, sphere volume) with the second-order
convergence of the refined linear interpolant, exactness for linear level
sets at every level, NEG + POS = the mesh measure, and the straight cut at
level 0.  CPU only."""
import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

TRI_EDGES = [(0, 1), (0, 2), (1, 2)]
TET_EDGES = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


def h1_coefs(mesh, sp, p):
    """Coefficients of the polynomial p (degree <= 2) in the H1 basis of sp."""
    D, k = mesh.dim, sp.order
    edges = TRI_EDGES if D == 2 else TET_EDGES
    el = sp.el_dofs()
    out = np.zeros(sp.ndof)
    for e in range(mesh.ne):
        X = mesh.coords[mesh.elements[e]]
        loc = [p(X[i]) for i in range(D + 1)]
        if k >= 2:
            for a, b in edges:
                loc.append(4 * p(0.5 * (X[a] + X[b])) - 2 * (p(X[a]) + p(X[b])))
                if k == 3:
                    loc.append(0.0)
        loc += [0.0] * (sp.ndof_el - len(loc))
        out[el[e]] = loc
    return out


def test_circle_converges(orc):
    r = 0.33
    m = MakeStructured2DMesh(10, 10)
    sp = orc.Space(m, 2)
    c = h1_coefs(m, sp, lambda X: (X[0] - .5) ** 2 + (X[1] - .5) ** 2 - r * r)
    ea, ep = [], []
    for L in range(5):
        ea.append(abs(sp.integrate_subdiv(c, orc.NEG, 2, L) - np.pi * r * r))
        ep.append(abs(sp.integrate_subdiv(c, orc.IF, 2, L) - 2 * np.pi * r))
        total = sp.integrate_subdiv(c, orc.NEG, 2, L) + sp.integrate_subdiv(c, orc.POS, 2, L)
        assert abs(total - 1.0) < 1e-13
    # second order in the sub-simplex size: the error drops by about 4 per level
    for L in range(1, 5):
        assert 3.2 < ea[L - 1] / ea[L] < 4.8, ea
        assert 3.2 < ep[L - 1] / ep[L] < 4.8, ep
    assert ea[4] < 5e-5 and ep[4] < 1e-4


def test_sphere_converges(orc):
    r = 0.3
    m = MakeStructured3DMesh(5)
    sp = orc.Space(m, 2)
    c = h1_coefs(m, sp, lambda X: (X[0] - .5) ** 2 + (X[1] - .5) ** 2 + (X[2] - .5) ** 2 - r * r)
    ev = [abs(sp.integrate_subdiv(c, orc.NEG, 2, L) - 4 / 3 * np.pi * r ** 3) for L in range(4)]
    es = [abs(sp.integrate_subdiv(c, orc.IF, 2, L) - 4 * np.pi * r ** 2) for L in range(4)]
    for L in range(1, 4):
        assert 3.0 < ev[L - 1] / ev[L] < 5.0, ev
        assert es[L - 1] / es[L] > 3.0, es  # the surface of the interpolant: second order, not yet asymptotic
    assert ev[3] < 1.5e-3 and es[3] < 1e-3
    total = sp.integrate_subdiv(c, orc.NEG, 2, 2) + sp.integrate_subdiv(c, orc.POS, 2, 2)
    assert abs(total - 1.0) < 1e-13


@pytest.mark.parametrize("D", [2, 3])
@pytest.mark.parametrize("k", [1, 2, 3])
def test_linear_level_set_is_exact_at_every_level(orc, D, k):
    """A linear level set is its own interpolant on every sub-simplex: every
    level gives the straight cut (orc_integrate) of the vertex values."""
    m = MakeStructured2DMesh(5, 4) if D == 2 else MakeStructured3DMesh(3)
    sp = orc.Space(m, k)
    f = lambda X: 0.7 * X[0] - 0.4 * X[1] + (0.2 * X[2] if D == 3 else 0) - 0.23  # noqa: E731
    c = h1_coefs(m, sp, f)
    sp1 = orc.Space(m, 1)
    lv = orc.interpolate_p1_perturb(h1_coefs(m, sp1, f))
    for dt in (orc.NEG, orc.POS, orc.IF):
        for mono in ((0, 0, 0), (1, 0, 0), (0, 2, 1)):
            ref = sp1.integrate(lv, dt, 4, *mono)
            for L in range(3):
                got = sp.integrate_subdiv(c, dt, 4, L, *mono)
                assert abs(got - ref) < 1e-13 * max(1.0, abs(ref)), (dt, mono, L, got, ref)


def test_level_zero_is_the_straight_cut_of_the_vertex_values(orc):
    r = 0.3
    m = MakeStructured3DMesh(4)
    sp = orc.Space(m, 2)
    f = lambda X: (X[0] - .5) ** 2 + (X[1] - .45) ** 2 + (X[2] - .52) ** 2 - r * r  # noqa: E731
    c = h1_coefs(m, sp, f)
    sp1 = orc.Space(m, 1)
    lv = h1_coefs(m, sp1, f)
    for dt in (orc.NEG, orc.POS, orc.IF):
        assert abs(sp.integrate_subdiv(c, dt, 2, 0) - sp1.integrate(lv, dt, 2)) < 1e-14


def test_rule_points_lie_in_the_element(orc):
    r = 0.33
    m = MakeStructured2DMesh(6, 6)
    sp = orc.Space(m, 2)
    c = h1_coefs(m, sp, lambda X: (X[0] - .5) ** 2 + (X[1] - .5) ** 2 - r * r)
    for e in range(m.ne):
        pts, w = sp.subdiv_rule(c, e, orc.NEG, 2, 2)
        if len(w) == 0:
            continue
        X = m.coords[m.elements[e]]
        A = np.stack([X[0] - X[2], X[1] - X[2]], 1)
        lam = np.linalg.solve(A, (pts[:, :2] - X[2]).T).T
        assert lam.min() > -1e-12 and lam.sum(1).max() < 1 + 1e-12
        assert w.min() > 0


def test_device_rule_code_matches_oracle(orc, tmp_path):
    """csrc/xg_subdiv.cuh compiled as host code against orc_subdiv_rule
    (tests/native/subdiv_check.cu): points and weights within 1e-12."""
    import os
    import shutil
    import subprocess
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    libdir = os.path.dirname(orc.LIB)
    exe = str(tmp_path / "subdiv_check")
    subprocess.check_call([nvcc, "-x", "cu", "-std=c++17", "-O1", "-Xcompiler", "-ffp-contract=off",
                           "-diag-suppress", "20011,20014", "-I", os.path.join(root, "ngsxfem_gb300", "csrc"),
                           "-I", os.path.join(root, "include"), os.path.join(here, "native", "subdiv_check.cu"),
                           "-L", libdir, "-loracle", "-Xlinker", "-rpath", "-Xlinker", libdir, "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout

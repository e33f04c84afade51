"""The P2 (isoparametric) oracle and the learned-quadrature oracle, on the CPU.

* Mesh-level isoparametric integration pinned against the reference's
  curved-circle test (tests/pytests/test_intcurved.py:17-91, order 2): the
  circle sqrt(x^2+y^2) - 0.5 on [-1,1]^2, N = 4 * 2^l, errors of the NEG, POS
  and IF measures below 1e-5 at the finest level and mean EOC above 2.75.
* Single-element rule: a linear level set needs no deformation (isoparametric
  moments == straight-cut moments == exact subdivision moments).
* The network objective's gradient against central differences."""
import math

import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh
from oracle import learned_ref as L
from oracle import oracle as orc


def test_intcurved_order2_known_answers():
    phi = lambda p: np.sqrt(p[..., 0] ** 2 + p[..., 1] ** 2) - 0.5  # noqa: E731
    exact = {orc.NEG: 0.25 * math.pi, orc.POS: 4 - 0.25 * math.pi, orc.IF: math.pi}
    errs = {k: [] for k in exact}
    for l in range(5):
        N = 4 * 2 ** l
        m = MakeStructured2DMesh(N, N, -1, 1, -1, 1)
        v = orc.p2_nodal_values(m, phi)
        for dt in exact:
            val, _ = orc.iso_integrate_mesh(m, v, dt, 2, threshold=0.2)
            errs[dt].append(abs(val - exact[dt]))
    for dt, e in errs.items():
        eoc = [math.log(a / b) / math.log(2) for a, b in zip(e[:-1], e[1:])]
        assert e[-1] < 1e-5, (dt, e)
        assert sum(eoc) / len(eoc) > 2.75, (dt, eoc)
    # without the deformation the P1 geometry error is second order only
    m = MakeStructured2DMesh(64, 64, -1, 1, -1, 1)
    v = orc.p2_nodal_values(m, phi)
    plain, _ = orc.iso_integrate_mesh(m, v, orc.NEG, 2, deform=False)
    assert abs(plain - exact[orc.NEG]) > 10 * errs[orc.NEG][-1]


def test_linear_level_set_needs_no_deformation():
    E = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]
    rng = np.random.default_rng(4)
    for _ in range(5):
        v = rng.standard_normal(4)
        v -= rng.uniform(v.min(), v.max())
        p2 = np.concatenate([v, [0.5 * (v[a] + v[b]) for a, b in E]])
        iso, nc = orc.iso_moments_tet(p2[None], 8, True)
        p1, _ = orc.iso_moments_tet(p2[None], 4, False)
        th, band, _ = orc.iso_deformation(np.array([[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 0, 0.]]), p2)
        assert band and np.max(np.abs(th)) < 1e-15
        ex = orc.subdiv_moments_tet(p2, 1)
        assert np.max(np.abs(iso - p1)) < 1e-15 and np.max(np.abs(ex - p1[0])) < 1e-15


def test_isoparametric_beats_straight_cut_on_resolved_elements():
    """Mildly curved elements: the isoparametric moments are closer to the exact
    NEG moments (subdivision, Richardson-extrapolated) than the straight cut."""
    rng = np.random.default_rng(8)
    v = L.resolved_values(6, rng, curvature=0.05)
    iso, _ = orc.iso_moments_tet(v, 8, True)
    p1, _ = orc.iso_moments_tet(v, 4, False)
    better = 0
    for i in range(len(v)):
        e4, e5 = orc.subdiv_moments_tet(v[i], 4), orc.subdiv_moments_tet(v[i], 5)
        ex = (4 * e5 - e4) / 3
        sc = np.abs(ex).max()
        better += np.abs(iso[i] - ex).max() / sc < np.abs(p1[i] - ex).max() / sc
    assert better >= 5


def test_network_objective_gradient_central_differences():
    rng = np.random.default_rng(0)
    n = sum(int(np.prod(s)) for _, s in L.SHAPES)
    p = rng.standard_normal(n) * 0.05
    x = rng.uniform(-1, 1, (8, 10))
    t = rng.standard_normal((8, 35)) * 0.01
    s = rng.uniform(0.5, 1, 8)
    _, g = L.loss_grad(p, x, t, s)
    # biases enter unrounded: central differences apply directly
    for idx in [n - 1, n - 5, 2560 + 3, 2560 + 256 + 65536 + 7]:
        e = np.zeros(n)
        e[idx] = 1e-6
        fd = (L.loss_grad(p + e, x, t, s)[0] - L.loss_grad(p - e, x, t, s)[0]) / 2e-6
        assert abs(fd - g[idx]) <= 1e-6 * max(1.0, abs(g[idx])), (idx, fd, g[idx])
    assert np.linalg.matrix_rank(L.vandermonde()) == 24


def test_mesh_level_device_code_matches_oracle(tmp_path):
    """csrc/xg_isomesh.cuh (per-element contributions, per-edge averages in
    element order, mapped rules) compiled as host code against
    orc_iso_integrate_mesh (tests/native/isomesh_check.cu): 2D circle and 3D
    sphere, NEG / POS / IF, orders 2 and 4, with and without clipping and
    deformation, within 1e-12 relative."""
    import os
    import shutil
    import subprocess
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    orc.build()
    libdir = os.path.dirname(orc.LIB)
    exe = str(tmp_path / "isomesh_check")
    subprocess.check_call([nvcc, "-x", "cu", "-std=c++17", "-O1", "-Xcompiler", "-ffp-contract=off",
                           "-diag-suppress", "20011,20013,20014", "-I", os.path.join(root, "ngsxfem_gb300", "csrc"),
                           "-I", os.path.join(root, "include"), os.path.join(here, "native", "isomesh_check.cu"),
                           "-L", libdir, "-loracle", "-Xlinker", "-rpath", "-Xlinker", libdir, "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout


def test_p2_element_values_match_the_oracle_layout():
    from ngsxfem_gb300.meshes import MakeStructured3DMesh
    from ngsxfem_gb300.xfem import P2ElementValues
    for m in (MakeStructured2DMesh(3, 4), MakeStructured3DMesh(2)):
        f = lambda *x: sum((k + 1) * xi ** 2 for k, xi in enumerate(x))  # noqa: E731
        g = lambda p: sum((k + 1) * p[..., k] ** 2 for k in range(m.dim))  # noqa: E731
        assert np.array_equal(P2ElementValues(m, f), orc.p2_nodal_values(m, g))

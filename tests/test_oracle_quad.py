"""The oracle's quadrilateral / hexahedral cut rules
(oracle/xg_oracle_quad.cpp, LevelsetCutQuadrilateral of
cutint/straightcutrule.cpp:206-501) against the closed-form answers that
ngsxfem's tests assert on quad and hex meshes (tests/golden/known_answers.json,
from tests/pytests/test_straightcutrule.py and test_quadchallenges.py), and
the host build of the product's rule code (csrc/xg_quadcut.cuh) against the
oracle bit for bit.  CPU only."""
import json
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
KA = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))
DTS = (("NEG", 0), ("POS", 1), ("IF", 2))


def vertex_lset(orc, mesh, f):
    return orc.interpolate_p1_perturb(np.array([f(*p) for p in mesh.coords]))


def planar(coef):
    return lambda *x: coef[0] + sum(c * xi for c, xi in zip(coef[1:], x))


def tol(order):
    return 5e-15 * (order + 1) ** 2


@pytest.mark.parametrize("N", KA["planar2d"]["N"])
@pytest.mark.parametrize("order", KA["planar2d"]["orders"])
def test_planar_quads(orc, N, order):
    m = MakeStructured2DMesh(quads=True, nx=N, ny=N)
    l = vertex_lset(orc, m, planar(KA["planar2d"]["lset"]))
    for name, dt in DTS:
        v, st = orc.quad_integrate(m, l, dt, order)
        assert st == 0 and abs(v - KA["planar2d"]["values"][name]) < tol(order), (name, v)


@pytest.mark.parametrize("order", [2, 4, 8])
@pytest.mark.parametrize("dim", [0, 1])
def test_monomials_quad(orc, order, dim):
    m = MakeStructured2DMesh(quads=True, nx=1, ny=1)
    l = vertex_lset(orc, m, planar(KA["planar2d"]["lset"]))
    for ref in KA["mono2d"]:
        e = [0, 0, 0]
        e[dim] = ref["alpha"]
        for name, dt in DTS[:2]:
            v, st = orc.quad_integrate(m, l, dt, order, exps=e)
            assert st == 0 and abs(v - ref[name]) < tol(order)


@pytest.mark.parametrize("axis", [0, 1])
def test_orthogonal_cuts_quad(orc, axis):
    m = MakeStructured2DMesh(quads=True, nx=1, ny=1)
    for eps in KA["orth2d"]["eps"]:
        f = (lambda x, y: 1 - 2 * x + eps * (y - 0.5)) if axis == 0 else (lambda x, y: 1 - 2 * y + eps * (x - 0.5))
        l = vertex_lset(orc, m, f)
        refs = {"NEG": 0.5, "POS": 0.5, "IF": math.sqrt(1 + eps * eps / 4)}
        for name, dt in DTS:
            v, st = orc.quad_integrate(m, l, dt, 2)
            assert st == 0 and abs(v - refs[name]) < tol(2), (eps, name, v)
    s = KA["orth_axis2d"]["slope"]
    l = vertex_lset(orc, m, (lambda x, y: 1 - s * x) if axis == 0 else (lambda x, y: 1 - s * y))
    for name, dt in DTS:
        v, st = orc.quad_integrate(m, l, dt, 2)
        assert st == 0 and abs(v - KA["orth_axis2d"][name]) < tol(2)


@pytest.mark.parametrize("dt_name,dt", DTS)
def test_circle_eoc_quads(orc, dt_name, dt):
    ref = KA["circle_eoc"]
    r = ref["r"]
    for order in (2, 4, 8):
        errs = []
        for i in range(8):
            m = MakeStructured2DMesh(quads=True, nx=2 ** i, ny=2 ** i)
            l = vertex_lset(orc, m, lambda x, y: math.sqrt(x * x + y * y) - r)
            v, st = orc.quad_integrate(m, l, dt, order)
            assert st == 0
            errs.append(abs(v - ref[dt_name]))
        eoc = [math.log(errs[i + 1] / errs[i]) / math.log(0.5) for i in range(7)]
        assert sum(eoc[1:]) / 6 > ref["min_mean_eoc"]


@pytest.mark.parametrize("N,orders", [(1, KA["planar3d"]["orders"]), (KA["quad3d_planar"]["N"], KA["quad3d_planar"]["orders"])])
def test_planar_hexes(orc, N, orders):
    m = MakeStructured3DMesh(N, hexes=True)
    l = vertex_lset(orc, m, planar(KA["planar3d"]["lset"]))
    for order in orders:
        for name, dt in DTS:
            v, st = orc.quad_integrate(m, l, dt, order)
            assert st == 0 and abs(v - KA["planar3d"]["values"][name]) < tol(order), (order, name, v)


@pytest.mark.parametrize("N", [1, KA["quad3d_mono"]["N"]])
def test_monomials_hex(orc, N):
    m = MakeStructured3DMesh(N, hexes=True)
    l = vertex_lset(orc, m, planar(KA["planar3d"]["lset"]))
    for ref in KA["mono3d"]:
        for dim in range(3):
            e = [0, 0, 0]
            e[dim] = ref["alpha"]
            for name, dt in DTS[:2]:
                v, st = orc.quad_integrate(m, l, dt, 4, policy=orc.QUAD_OPTIMAL, exps=e)
                assert st == 0 and abs(v - ref[name]) < tol(4)


def test_orthogonal_cuts_hex(orc):
    m = MakeStructured3DMesh(1, hexes=True)
    s = KA["orth_axis3d"]["slope"]
    for axis in range(3):
        l = vertex_lset(orc, m, lambda x, y, z: 1 - s * (x, y, z)[axis])
        for name, dt in DTS:
            v, st = orc.quad_integrate(m, l, dt, 2)
            assert st == 0 and abs(v - KA["orth_axis3d"][name]) < tol(2)


def test_zero_value_challenge(orc):
    ref = KA["zero_val"]
    m = MakeStructured3DMesh(ref["N"], hexes=True)
    l = vertex_lset(orc, m, planar(KA["planar3d"]["lset"]))
    v, st = orc.quad_integrate(m, l, 1, ref["order"], policy=orc.QUAD_OPTIMAL, exps=(ref["alpha"], 0, 0))
    assert st == 0 and abs(v - ref["POS"]) < tol(ref["order"])


@pytest.mark.parametrize("dt_name,dt", DTS[:2])
def test_sphere_eoc_hexes(orc, dt_name, dt):
    ref = KA["sphere_eoc"]
    r = ref["r"]
    for order in ref["orders"]:
        errs = []
        for i in range(ref["n_ref"]):
            m = MakeStructured3DMesh(2 ** i, hexes=True)
            l = vertex_lset(orc, m, lambda x, y, z: math.sqrt(x * x + y * y + z * z) - r)
            v, st = orc.quad_integrate(m, l, dt, order)
            assert st == 0
            errs.append(abs(v - ref[dt_name]))
        eoc = [math.log(errs[i + 1] / errs[i]) / math.log(0.5) for i in range(ref["n_ref"] - 1)]
        assert sum(eoc[1:]) / (ref["n_ref"] - 2) > ref["min_mean_eoc"]


def test_tpmc_single_hex(orc):
    ref = KA["tpmc_hex"]
    m = MakeStructured3DMesh(1, hexes=True)
    l = np.array([ref["vals"][int(4 * x + 2 * y + z)] for x, y, z in m.coords], dtype=np.float64)
    for order in ref["orders"]:
        vals = {name: orc.quad_integrate(m, l, dt, order) for name, dt in DTS}
        assert all(st == 0 for _, st in vals.values())
        assert vals["IF"][0] < ref["IF_below"]
        assert abs(vals["NEG"][0] - ref["NEG"]) < ref["tol"]
        assert abs(vals["POS"][0] - ref["POS"]) < ref["tol"]


def test_tpmc_trilinear_10(orc):
    ref = KA["tpmc_10"]
    m = MakeStructured3DMesh(10, hexes=True)
    l = np.array([x * ((7 * y - 13) * z + 6) + y * (3 - 8 * z) + 8 * z - 4 for x, y, z in m.coords])
    for order in ref["orders"]:
        neg, _ = orc.quad_integrate(m, l, 0, order)
        pos, _ = orc.quad_integrate(m, l, 1, order)
        iff, _ = orc.quad_integrate(m, l, 2, order)
        assert abs(neg - ref["NEG"]) < ref["tol_vol"] and abs(pos - ref["POS"]) < ref["tol_vol"]
        assert abs(iff - ref["IF"]) < ref["tol_if"]


def test_policies_agree_on_exact_cases(orc):
    """The three direction policies integrate the planar hex cut exactly."""
    m = MakeStructured3DMesh(2, hexes=True)
    l = vertex_lset(orc, m, planar(KA["planar3d"]["lset"]))
    for pol in (orc.QUAD_FIRST, orc.QUAD_OPTIMAL, orc.QUAD_FALLBACK):
        for name, dt in DTS:
            v, st = orc.quad_integrate(m, l, dt, 4, policy=pol)
            assert st == 0 and abs(v - KA["planar3d"]["values"][name]) < tol(4), (pol, name)


def test_unit_rule_weights(orc):
    """An uncut element gets the tensor rule of the unit box (weights sum to 1);
    "no rule" for the other domain."""
    for nv in (4, 8):
        p, w = orc.quad_cut_rule(np.full(nv, -1.0), 0, 4)
        assert abs(w.sum() - 1.0) < 1e-15
        assert orc.quad_cut_rule(np.full(nv, -1.0), 1, 4) is None


def test_device_rule_code_matches_oracle_bitwise(orc, tmp_path):
    """csrc/xg_quadcut.cuh compiled as host code against the oracle
    (tests/native/quad_rule_check.cu)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    libdir = os.path.dirname(orc.LIB)
    exe = str(tmp_path / "quad_rule_check")
    subprocess.check_call([nvcc, "-x", "cu", "-std=c++17", "-O1", "-Xcompiler", "-ffp-contract=off",
                           "-diag-suppress", "20011,20014", "-I", os.path.join(ROOT, "ngsxfem_gb300", "csrc"),
                           "-I", os.path.join(ROOT, "include"), os.path.join(HERE, "native", "quad_rule_check.cu"),
                           "-L", libdir, "-loracle", "-Xlinker", "-rpath", "-Xlinker", libdir, "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout


def test_cutinfo_ratios_give_the_volumes(orc):
    """CutInfo on quads / hexes: the order-0 part volumes reproduce the planar
    cut's NEG measure (uniform elements: sum of ratio x element volume; exact
    in 2D), the domain types follow the ratios, and the bit rows are
    consistent."""
    for m, coef, ref in ((MakeStructured2DMesh(quads=True, nx=10, ny=10), KA["planar2d"]["lset"],
                          KA["planar2d"]["values"]["NEG"]),
                         (MakeStructured3DMesh(6, hexes=True), KA["planar3d"]["lset"], KA["planar3d"]["values"]["NEG"])):
        l = vertex_lset(orc, m, planar(coef))
        dom, ratio, bits = orc.quad_cutinfo(m, l)
        vol = 1.0 / m.ne
        # order-0 rules: the cut length of a quad is linear in the tensor
        # direction (exact), the cut area of a hex quadratic (not exact)
        assert abs(ratio.sum() * vol - ref) < (1e-13 if m.dim == 2 else 1e-3)
        # uncut elements have ratio 1 / 0 (a cut element with a sliver part may round to them too)
        assert (ratio[dom == 0] == 1.0).all() and (ratio[dom == 1] == 0.0).all()
        assert ((ratio > 0) & (ratio < 1) <= (dom == 2)).all()
        b = np.unpackbits(bits.view(np.uint8), axis=1, bitorder="little")[:, : m.ne].astype(bool)
        assert (b[1] == (dom == 0)).all() and (b[2] == (dom == 1)).all() and (b[4] == (dom == 2)).all()
        assert (b[3] == (b[1] | b[2])).all() and (b[5] == (b[1] | b[4])).all() and (b[6] == (b[2] | b[4])).all()
        assert b[7].all() and not b[0].any()

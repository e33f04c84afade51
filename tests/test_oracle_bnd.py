"""Boundary cut integrals dCut(lset, dt, vb=BND): the oracle
(orc_integrate_bnd, oracle/xg_oracle_mlset.cpp) against the closed forms of
ngsxfem's tests/pytests/test_bndcut.py, and the product's boundary rule
(csrc/xg_mlset.cuh ml::bnd_rule) against the oracle per element (host build,
tests/native/mlset_rule_check.cu, run by test_oracle_mlset.py).  CPU only."""
import json
import os

import numpy as np

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

HERE = os.path.dirname(os.path.abspath(__file__))
KA = json.load(open(os.path.join(HERE, "golden", "known_answers.json")))


def test_boundary_measures_2d(orc):
    ref = KA["bnd2d"]
    m = MakeStructured2DMesh(9, 9)
    for cut in ref["cuts"]:
        l = orc.interpolate_p1_perturb(m.coords[:, 0] - cut)
        neg, st = orc.integrate_bnd(m, l, orc.NEG, 2)
        pos, _ = orc.integrate_bnd(m, l, orc.POS, 2)
        npts, _ = orc.integrate_bnd(m, l, orc.IF, 0)
        assert st == 0
        assert abs(neg - (2 * cut + 1)) < ref["tol"]
        assert abs(neg + pos - ref["perimeter"]) < ref["tol"]
        assert abs(npts - ref["IF_points"]) < ref["tol"]
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - 0.5)
    assert abs(orc.integrate_bnd(m, l, orc.IF, 0, (1, 0, 0))[0] - ref["if_x_at_half"]) < ref["tol"]
    assert abs(orc.integrate_bnd(m, l, orc.IF, 0, (0, 1, 0))[0] - ref["if_y_at_half"]) < ref["tol"]


def test_boundary_measures_3d(orc):
    ref = KA["bnd3d"]
    m = MakeStructured3DMesh(7)
    l = orc.interpolate_p1_perturb(m.coords[:, 0] - ref["cut"])
    neg, st = orc.integrate_bnd(m, l, orc.NEG, 2)
    assert st == 0 and abs(neg - ref["NEG"]) < ref["tol"]
    # the interface on boundary triangles (codimension 2) is not supported
    assert orc.integrate_bnd(m, l, orc.IF, 2)[1] == 6

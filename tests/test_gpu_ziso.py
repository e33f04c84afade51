"""Mesh-level isoparametric integration on the GPU (xg_iso_integrate_mesh,
LevelSetMeshAdaptation) against the oracle's orc_iso_integrate_mesh (pinned
on the reference's curved-circle test) and against the exact circle
measures of tests/pytests/test_intcurved.py.  Bar: 1e-12 relative to the
oracle (the device code equals the oracle's within 4e-16 on the CPU,
tests/test_oracle_iso.py)."""
import math

import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


def circle(*x):
    return np.sqrt(x[0] ** 2 + x[1] ** 2) - 0.5


def sphere(*x):
    return np.sqrt((x[0] - .5) ** 2 + (x[1] - .5) ** 2 + (x[2] - .5) ** 2) - 0.3


@pytest.mark.parametrize("D", [2, 3])
def test_matches_oracle(xg, orc, D):
    m = MakeStructured2DMesh(12, 12, -1, 1, -1, 1) if D == 2 else MakeStructured3DMesh(5)
    f = circle if D == 2 else sphere
    v = xg.P2ElementValues(m, f)
    for thr in (-1.0, 0.2):
        lma = xg.LevelSetMeshAdaptation(m, order=2, threshold=thr).CalcDeformation(v)
        for dt in (orc.NEG, orc.POS, orc.IF):
            for order, deform in ((2, True), (4, True), (2, False)):
                ref, nc = orc.iso_integrate_mesh(m, v, dt, order, threshold=thr, deform=deform)
                got = lma.Integrate(dt, order=order, deform=deform)
                assert abs(got - ref) <= 1e-12 * max(1.0, abs(ref)), (thr, dt, order, deform, got, ref)
                if deform:
                    assert lma.nonconverged == nc


def test_curved_circle_accuracy(xg, orc):
    """tests/pytests/test_intcurved.py (order 2): errors below 1e-5 at N = 64."""
    exact = {orc.NEG: 0.25 * math.pi, orc.POS: 4 - 0.25 * math.pi, orc.IF: math.pi}
    m = MakeStructured2DMesh(64, 64, -1, 1, -1, 1)
    lma = xg.LevelSetMeshAdaptation(m, order=2, threshold=0.2).CalcDeformation(circle)
    for dt, val in exact.items():
        assert abs(lma.Integrate(dt, order=2) - val) < 1e-5, dt

"""CutInfo on quadrilateral / hexahedral meshes on the GPU (xg_cutinfo_update
on a tensor mesh: order-0 rules of LevelsetCutQuadrilateral) against the
oracle (orc_quad_cutinfo): domain types and bits equal, ratios within 1e-14
(the two base-rule tables agree to ~4e-16)."""
import math

import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


def cases(orc):
    m1 = MakeStructured2DMesh(quads=True, nx=20, ny=20)
    yield m1, orc.interpolate_p1_perturb(np.array([math.hypot(x - .4, y - .5) - .3 for x, y in m1.coords]))
    m2 = MakeStructured3DMesh(8, hexes=True)
    yield m2, orc.interpolate_p1_perturb(np.array([math.sqrt(x * x + y * y + z * z) - .72 for x, y, z in m2.coords]))
    m3 = MakeStructured3DMesh(10, hexes=True)
    yield m3, np.array([x * ((7 * y - 13) * z + 6) + y * (3 - 8 * z) + 8 * z - 4 for x, y, z in m3.coords])


def test_cutinfo_matches_oracle(xg, orc):
    for m, l in cases(orc):
        gf = xg.GridFunction(xg.H1(m, order=1))
        gf.vec.copy_(torch.from_numpy(np.ascontiguousarray(l)))
        ci = xg.CutInfo(m, gf)
        dom, ratio, bits = orc.quad_cutinfo(m, l)
        assert (ci.dom.cpu().numpy() == dom).all()
        assert np.max(np.abs(ci.cut_ratio.cpu().numpy() - ratio)) <= 1e-14
        got = ci.bits.cpu().numpy().view(np.uint64)
        assert (got == bits).all()
        assert ci.GetElementsOfType(xg.IF).NumSet() == int((dom == 2).sum()) > 0
        with pytest.raises(NotImplementedError):
            ci.GetCutNeighboringNodes("vertex")

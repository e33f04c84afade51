"""CutInfo beyond the VOL elements, on the GPU through the C ABI and the Python
mirror, against the oracle: BND elements (xfem/cutinfo.cpp:83-131 with vb ==
BND), cut-neighbouring nodes and node domain types (:134-224), and
GetElementsWithThresholdContribution (:263-284).  Bit-exact."""
import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


def cases():
    m2 = MakeStructured2DMesh(24, 20, -1, 1, -1, 1)
    m3 = MakeStructured3DMesh(7, 6, 5)
    rng = np.random.default_rng(4)
    return {
        "circle2d": (m2, np.sqrt((m2.coords ** 2).sum(1)) - 1.2),
        "random2d": (m2, rng.standard_normal(m2.nv) + 0.2),
        "sphere3d": (m3, np.sqrt(((m3.coords - 0.4) ** 2).sum(1)) - 0.45),
        "random3d": (m3, rng.standard_normal(m3.nv) + 0.3),
    }


CASES = list(cases())


def words(t):
    return t.cpu().numpy().view(np.uint64)


@pytest.mark.parametrize("case", CASES)
def test_bnd_and_nodes_match_oracle(xg, orc, case):
    m, vals = cases()[case]
    l = orc.interpolate_p1_perturb(vals)
    gf = xg.GridFunction(xg.H1(m, 1))
    xg.InterpolateToP1(vals, gf)
    ci = xg.CutInfo(m, gf)
    torch.cuda.synchronize()
    sp = orc.Space(m, 1)
    # BND elements
    facets, _ = sp.boundary_elements()
    nb = np.zeros(len(facets), dtype=np.int32)
    import ctypes
    nbn = np.zeros(1, dtype=np.int64)
    xg._lib.call("xg_mesh_boundary", ci.dm.h, nbn.ctypes.data_as(ctypes.c_void_p), nb.ctypes.data_as(ctypes.c_void_p))
    assert nbn[0] == len(facets) and np.array_equal(nb, facets)
    dom_b, ratio_b, bits_b = sp.cutinfo_bnd(l)
    assert np.array_equal(ci.dom_bnd[: ci.nbnd].cpu().numpy(), dom_b)
    assert np.array_equal(ci.GetCutRatios(xg.BND).cpu().numpy().view(np.uint64), ratio_b.view(np.uint64))
    assert np.array_equal(words(ci.bits_bnd), bits_b)
    nw = (len(facets) + 63) // 64
    assert np.array_equal(words(ci.GetElementsOfType(xg.IF, xg.BND).words)[:nw], bits_b[4])
    assert np.array_equal(words(ci.GetElementsOfType(xg.HASNEG, xg.BND).words)[:nw], bits_b[5])
    assert (dom_b == 2).sum() > 0 and (dom_b != 2).sum() > 0
    # nodes
    dom, ratio, _ = sp.cutinfo(l)
    (nv, ne_, nf, nel), (dv, de, df, dc) = sp.cutinfo_nodes(dom, ratio)
    assert np.array_equal(words(ci.cut_nb_nodes["vertex"])[: len(nv)], nv)
    assert np.array_equal(words(ci.cut_nb_nodes["edge"])[: len(ne_)], ne_)
    assert np.array_equal(words(ci.cut_nb_nodes["element"])[: len(nel)], nel)
    assert np.array_equal(ci.GetDomainOfNodes("vertex").cpu().numpy(), dv)
    assert np.array_equal(ci.GetDomainOfNodes("edge").cpu().numpy(), de)
    assert np.array_equal(ci.GetDomainOfNodes("cell").cpu().numpy(), dc)
    if m.dim == 3:
        assert np.array_equal(words(ci.cut_nb_nodes["face"])[: len(nf)], nf)
        assert np.array_equal(ci.GetDomainOfNodes("face").cpu().numpy(), df)
    # threshold marking
    for dt, thr in ((0, 0.5), (0, 1.0), (1, 0.25), (1, 1.0)):
        got = ci.GetElementsWithThresholdContribution(dt, thr).numpy()
        t = 1 - thr if dt == 1 else thr
        ref = ratio >= t if dt == 0 else ratio <= t
        assert np.array_equal(got, ref)

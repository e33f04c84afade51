"""The space-time Python mirror (ScalarTimeFE, tfe * fes, SpaceTimeInterpolateToP1,
dtref, dCut(..., time_order=..., tref=...), delta_t * dCut, dFacetPatch(time_order=...),
BilinearForm(st_fes).Assemble()), written like demos/spacetime/spacetimeDG_unfitted.py:124-168,
against the oracle's space-time assembly (within 1e-12)."""
import math

import numpy as np
import pytest

from ngsxfem_gb300.meshes import MakeStructured2DMesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k_t", [1, 2])
def test_spacetime_demo_shape(xg, orc, k_t):
    m = MakeStructured2DMesh(14, 14)
    delta_t, slab = 1.0 / 16, 3
    t0 = slab * delta_t
    w_amp = 0.4 * math.pi

    def levelset(x, y, t):
        cx, cy = 0.5 + 0.2 * math.cos(2 * math.pi * t), 0.5 + 0.2 * math.sin(2 * math.pi * t)
        return np.sqrt((x - cx) ** 2 + (y - cy) ** 2) - 0.25

    fes1 = xg.H1(m, order=1, dgjumps=True)
    tfe = xg.ScalarTimeFE(k_t)
    st_fes = tfe * fes1
    lset_st = xg.GridFunction(xg.ScalarTimeFE(k_t) * xg.H1(m, order=1))
    xg.SpaceTimeInterpolateToP1(levelset, None, lset_st, t0=t0, dt=delta_t)
    ci = xg.CutInfo(m, time_order=0)
    ci.Update(lset_st, time_order=0)
    hasneg = ci.GetElementsOfType(xg.HASNEG)
    ba_facets = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=ci.GetElementsOfType(xg.IF))
    u, v = st_fes.TnT()
    h = xg.specialcf.mesh_size
    time_order = 2 * k_t
    dQ = delta_t * xg.dCut(lset_st, xg.NEG, time_order=time_order, definedonelements=hasneg)
    dOmold = xg.dCut(lset_st, xg.NEG, definedonelements=hasneg, tref=0)
    dw = delta_t * xg.dFacetPatch(definedonelements=ba_facets, time_order=time_order)
    wvec = xg.TimeVector(bc=(0.0, w_amp), bs=(-w_amp, 0.0), omega=2 * math.pi, t0=t0, dt=delta_t)

    def dt(f):
        return 1.0 / delta_t * xg.dtref(f)

    gamma = 0.05
    a = xg.BilinearForm(st_fes)
    a += v * dt(u) * dQ
    a += xg.InnerProduct(xg.grad(u), xg.grad(v)) * dQ
    a += v * xg.InnerProduct(wvec, xg.grad(u)) * dQ
    a += u * v * dOmold
    a += h ** (-2) * (1 + delta_t / h) * gamma * (u - u.Other()) * (v - v.Other()) * dw
    a.Assemble()
    r, c, vals = a.mat.global_coo()
    # oracle: the same terms written out
    lst = lset_st.vec.cpu().numpy().reshape(k_t + 1, m.nv)
    sp = orc.Space(m, 1)
    dom, _, bits = sp.cutinfo_st(lst, k_t)
    fb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
    terms = [dict(kind=orc.TERM_DT_U_V, domain=orc.NEG, coef=1.0),
             dict(kind=orc.TERM_LAPLACE, domain=orc.NEG, coef=delta_t),
             dict(kind=orc.TERM_CONV, domain=orc.NEG, coef=delta_t, b=(0.0, 0.0, 0.0), bc=(0.0, w_amp, 0.0),
                  bs=(-w_amp, 0.0, 0.0), omega=2 * math.pi, t0=t0, dt=delta_t),
             dict(kind=orc.TERM_MASS, domain=orc.NEG, coef=1.0, tref=0.0),
             dict(kind=orc.TERM_GHOST_MASS, coef=gamma * delta_t, hpow=-2),
             dict(kind=orc.TERM_GHOST_MASS, coef=gamma * delta_t * delta_t, hpow=-3)]
    for t in terms:
        t["defined_on"] = fb if t["kind"] == orc.TERM_GHOST_MASS else bits[5]
    rp, rc, rv = sp.assemble_st(lst, k_t, k_t, time_order, terms)
    rr = np.repeat(np.arange(len(rp) - 1), np.diff(rp))
    ref = {(int(i), int(j)): x for i, j, x in zip(rr, rc, rv)}
    got = {(int(i), int(j)): x for i, j, x in zip(r, c, vals)}
    assert set(ref) == set(got)
    scale = max(abs(x) for x in ref.values())
    assert max(abs(got[k] - ref[k]) for k in ref) <= 1e-12 * scale

"""xg_integrate_noalloc: the allocation-free Integrate for callers that cannot
allocate device memory while they run (stream capture into a CUDA graph,
real-time loops, foreign allocators).  Checked through the C ABI against the
allocating xg_integrate on two calls in a row; this file is collected last."""
import ctypes

import numpy as np
import pytest
import torch

from ngsxfem_gb300.meshes import MakeStructured2DMesh, MakeStructured3DMesh

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim", [2, 3])
def test_noalloc_matches_integrate(xg, dim):
    lib = xg._lib.load()
    if dim == 2:
        m = MakeStructured2DMesh(40, 40, -1, 1, -1, 1)
        vals = np.sqrt(m.coords[:, 0] ** 2 + m.coords[:, 1] ** 2) - 0.5
    else:
        m = MakeStructured3DMesh(12)
        c = m.coords - 0.5
        vals = np.sqrt((c ** 2).sum(1)) - 0.3
    gf = xg.GridFunction(xg.H1(m, 1))
    xg.InterpolateToP1(vals, gf)
    dm = xg.device_mesh(m)
    ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    got = torch.zeros(2, dtype=torch.float64, device="cuda")
    stream = xg._stream()
    for dt in (xg.NEG, xg.POS, xg.IF):
        for e in ((0, 0, 0), (1, 2, 0)):
            xg._lib.check(lib.xg_integrate(dm.h, xg._vp(gf.vec), dt, 4, e[0], e[1], e[2], None, xg._vp(ref), stream),
                          "xg_integrate")
            for k in range(2):  # two calls in a row share the static scratch
                out = ctypes.c_void_p(got.data_ptr() + 8 * k)
                xg._lib.check(lib.xg_integrate_noalloc(dm.h, xg._vp(gf.vec), dt, 4, e[0], e[1], e[2], None, out,
                                                       stream), "xg_integrate_noalloc")
            torch.cuda.synchronize()
            dm.check()
            r = float(ref.item())
            for k in range(2):
                assert abs(float(got[k].item()) - r) <= 1e-12 * max(1.0, abs(r)), (dt, e, k)

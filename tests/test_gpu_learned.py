"""P2 level sets on the GPU (through the C ABI): the isoparametric moment
kernel against the oracle, the learned quadrature's network (forward, loss and
gradient) against the numpy statement, and a short GPU training run that shows
what the trained network gains over the method without it."""
import ctypes

import numpy as np
import pytest
import torch

from oracle import learned_ref as L

pytestmark = pytest.mark.gpu


def dev(a, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(a)).to("cuda", dtype)


def gpu_moments(xg, vals, order, deform):
    d_v = dev(vals)
    out = torch.zeros((len(vals), 35), dtype=torch.float64, device="cuda")
    nc = torch.zeros(len(vals), dtype=torch.int32, device="cuda")
    xg._lib.call("xg_iso_moments_tet", xg._vp(d_v), len(vals), order, int(deform), xg._vp(out), xg._vp(nc),
                 xg._stream())
    torch.cuda.synchronize()
    return out.cpu().numpy(), nc.cpu().numpy()


@pytest.mark.parametrize("dist", ["spec", "resolved"])
@pytest.mark.parametrize("deform", [0, 1])
def test_iso_moments_parity(xg, orc, dist, deform):
    rng = np.random.default_rng(11)
    v = L.spec_values(3000, rng) if dist == "spec" else L.resolved_values(3000, rng)
    order = 8 if deform else 4
    got, gnc = gpu_moments(xg, v, order, deform)
    ref, rnc = orc.iso_moments_tet(v, order, bool(deform), 8)
    scale = np.maximum(np.abs(ref).max(1), 1e-300)
    err = np.abs(got - ref).max(1) / scale
    same = gnc == rnc
    # the rule families of the two sides agree to a few ulp; Newton searches
    # that stop at |defect| < 1e-14 may stop one step apart
    assert same.mean() > 0.995, same.mean()
    assert np.quantile(err[same], 0.999) < 1e-10, np.sort(err[same])[-5:]
    assert (ref[:, 0] > 0).sum() > 100


def params_of(xg, mlp):
    n = np.zeros(1, dtype=np.int64)
    xg._lib.call("xg_mlp_param_count", n.ctypes.data_as(ctypes.c_void_p))
    p = torch.zeros(int(n[0]), dtype=torch.float32, device="cuda")
    xg._lib.call("xg_mlp_get_params", mlp, xg._vp(p), xg._stream())
    torch.cuda.synchronize()
    return p


def test_points_match_oracle(xg):
    pts = np.zeros(72)
    xg._lib.call("xg_learned_points", pts.ctypes.data_as(ctypes.c_void_p))
    assert np.array_equal(pts.reshape(24, 3), L.point_set())


@pytest.mark.parametrize("B", [37, 4096])
def test_network_forward_and_gradient_vs_oracle(xg, B):
    mlp = ctypes.c_void_p()
    xg._lib.call("xg_mlp_create", 1234, ctypes.byref(mlp))
    p = params_of(xg, mlp)
    rng = np.random.default_rng(B)
    x = rng.uniform(-1, 1, (B, 10)).astype(np.float32)
    t = (rng.standard_normal((B, 35)) * 0.01).astype(np.float32)
    s = rng.uniform(0.5, 1.0, B).astype(np.float32)
    d_x, d_t, d_s = dev(x, torch.float32), dev(t, torch.float32), dev(s, torch.float32)
    y = torch.zeros((B, 24), dtype=torch.float32, device="cuda")
    xg._lib.call("xg_mlp_forward", mlp, xg._vp(d_x), B, xg._vp(y), xg._stream())
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    g = torch.zeros_like(p)
    xg._lib.call("xg_mlp_loss_grad", mlp, xg._vp(d_x), xg._vp(d_t), xg._vp(d_s), B, xg._vp(loss), xg._vp(g),
                 xg._stream())
    torch.cuda.synchronize()
    pn = p.cpu().numpy().astype(np.float64)
    y_ref, _ = L.forward(pn, x.astype(np.float64))
    assert np.max(np.abs(y.cpu().numpy() - y_ref)) <= 1e-5 * max(1.0, np.abs(y_ref).max())
    l_ref, g_ref = L.loss_grad(pn, x.astype(np.float64), t.astype(np.float64), s.astype(np.float64))
    assert abs(float(loss.item()) - l_ref) <= 1e-5 * l_ref
    gg = g.cpu().numpy()
    k = 0
    for name, shp in L.SHAPES:
        n = int(np.prod(shp))
        a, b = gg[k:k + n], g_ref[k:k + n]
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b), (name, np.linalg.norm(a - b) / np.linalg.norm(b))
        k += n
    xg._lib.call("xg_mlp_destroy", mlp)


@pytest.mark.parametrize("B", [1, 127, 128, 129, 40000])
def test_tensor_core_forward_vs_oracle(xg, B):
    """The fused tcgen05 inference kernel (BF16 operands and activations, FP32
    accumulation in tensor memory) against the numpy statement with the same
    BF16 roundings: within 2e-3 of the output scale (a few BF16 ulps of the
    activations that round differently after FP32 vs FP64 sums), and within
    3e-2 of the FP32-activation forward."""
    mlp = ctypes.c_void_p()
    xg._lib.call("xg_mlp_create", 99, ctypes.byref(mlp))
    p = params_of(xg, mlp)
    rng = np.random.default_rng(B + 5)
    x = rng.uniform(-1, 1, (B, 10)).astype(np.float32)
    d_x = dev(x, torch.float32)
    y_tc = torch.full((B, 24), float("nan"), dtype=torch.float32, device="cuda")
    y_ref32 = torch.zeros((B, 24), dtype=torch.float32, device="cuda")
    for _ in range(2):  # two calls in a row: the persistent kernel leaves nothing behind
        xg._lib.call("xg_mlp_forward_tc", mlp, xg._vp(d_x), B, xg._vp(y_tc), xg._stream())
        torch.cuda.synchronize()
        xg._lib.check(xg._lib.load().xg_mlp_check(mlp), "tensor-core forward")
    xg._lib.call("xg_mlp_forward", mlp, xg._vp(d_x), B, xg._vp(y_ref32), xg._stream())
    torch.cuda.synchronize()
    got = y_tc.cpu().numpy()
    assert np.all(np.isfinite(got))
    ref = L.forward_bf16_activations(p.cpu().numpy().astype(np.float64), x)
    scale = max(1.0, np.abs(ref).max())
    assert np.max(np.abs(got - ref)) <= 2e-3 * scale, np.max(np.abs(got - ref)) / scale
    assert np.max(np.abs(got - y_ref32.cpu().numpy())) <= 3e-2 * scale
    xg._lib.call("xg_mlp_destroy", mlp)


def test_features_match_oracle(xg):
    v = L.spec_values(500, np.random.default_rng(2))
    x = torch.zeros((500, 10), dtype=torch.float32, device="cuda")
    d_v = dev(v)
    xg._lib.call("xg_learned_features", xg._vp(d_v), 500, xg._vp(x), xg._stream())
    torch.cuda.synchronize()
    assert np.max(np.abs(x.cpu().numpy() - L.features(v))) < 1e-6


def rel_err(a, ref):
    """moment error in units of the element measure (1/6 for the reference tet)"""
    return np.abs(a - ref).max(1) * 6.0


def learned_moments(xg, mlp, vals, kappa=-1.0):
    out = torch.zeros((len(vals), 35), dtype=torch.float64, device="cuda")
    nf = torch.zeros(1, dtype=torch.int32, device="cuda")
    d_v = dev(vals)
    xg._lib.call("xg_learned_moments_tet", mlp, xg._vp(d_v), len(vals), ctypes.c_double(kappa), xg._vp(out),
                 xg._vp(nf), xg._stream())
    torch.cuda.synchronize()
    return out.cpu().numpy(), int(nf.item())


def test_fallback_takes_the_plain_rule(xg):
    """kappa_max = 0: every element in the relevant band takes the
    isoparametric rule, so the result equals the plain kernel's bit for bit."""
    v = L.resolved_values(2000, np.random.default_rng(9))
    mlp = ctypes.c_void_p()
    xg._lib.call("xg_mlp_create", 3, ctypes.byref(mlp))
    got, nf = learned_moments(xg, mlp, v, 0.0)
    ref, _ = gpu_moments(xg, v, 8, 1)
    p1 = v[:, :4]
    band = (np.where(np.abs(p1) < 1e-14, 1e-14, p1).min(1) < 0) & (np.where(np.abs(p1) < 1e-14, 1e-14, p1).max(1) > 0)
    assert nf == band.sum()
    assert np.array_equal(got, ref)
    xg._lib.call("xg_mlp_destroy", mlp)


def test_fallback_takes_the_subdivision_rule(xg, orc):
    """With the subdivision rule as the plain rule (plain_subdivlvl = 2) and
    kappa_max = 0 every element in the band takes that rule: the result
    equals xg_subdiv_moments_tet bit for bit, and the oracle's rule within
    1e-13."""
    v = L.resolved_values(2000, np.random.default_rng(19))
    d_v = dev(v)
    mlp = ctypes.c_void_p()
    xg._lib.call("xg_mlp_create", 3, ctypes.byref(mlp))
    out = torch.zeros((len(v), 35), dtype=torch.float64, device="cuda")
    nf = torch.zeros(1, dtype=torch.int32, device="cuda")
    xg._lib.call("xg_learned_moments_tet_ex", mlp, xg._vp(d_v), len(v), ctypes.c_double(0.0), 2, xg._vp(out),
                 xg._vp(nf), xg._stream())
    ref = torch.zeros_like(out)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    xg._lib.call("xg_subdiv_moments_tet", xg._vp(d_v), len(v), 2, xg._vp(ref), xg._vp(err), xg._stream())
    torch.cuda.synchronize()
    xg._lib.check(xg._lib.load().xg_mlp_check(mlp), "learned")
    assert int(err.item()) == 0
    p1 = v[:, :4]
    band = (np.where(np.abs(p1) < 1e-14, 1e-14, p1).min(1) < 0) & (np.where(np.abs(p1) < 1e-14, 1e-14, p1).max(1) > 0)
    assert int(nf.item()) == band.sum()
    got = out.cpu().numpy()
    assert np.array_equal(got[band], ref.cpu().numpy()[band])
    orc_m = orc.subdiv_moments_p2(v, 2, 8)
    assert np.abs(got[band] - orc_m[band]).max() < 1e-13
    xg._lib.call("xg_mlp_destroy", mlp)


def test_training_gains_over_the_method_without_it(xg):
    """A short GPU training run on mildly curved elements (targets: the
    isoparametric moments; training samples whose defect exceeds 5 % of the
    element measure or whose point searches did not all converge are left to
    the fallback): on held-out elements the learned rule's moment error is
    below that of the straight cut rule alone (the method without the network)
    and far below the untrained network's."""
    rng = np.random.default_rng(5)
    v_tr = L.resolved_values(120000, rng, curvature=0.1)
    v_te = L.resolved_values(4000, np.random.default_rng(6), curvature=0.1)
    iso_tr, nc_tr = gpu_moments(xg, v_tr, 8, 1)
    p1_tr, _ = gpu_moments(xg, v_tr, 4, 0)
    iso_te, _ = gpu_moments(xg, v_te, 8, 1)
    p1_te, _ = gpu_moments(xg, v_te, 4, 0)
    keep = (nc_tr == 0) & (np.abs(iso_tr - p1_tr).max(1) * 6 <= 0.05)
    v_tr, iso_tr, p1_tr = v_tr[keep], iso_tr[keep], p1_tr[keep]
    n = len(v_tr)
    d_x = torch.zeros((n, 10), dtype=torch.float32, device="cuda")
    d_vtr = dev(v_tr)
    xg._lib.call("xg_learned_features", xg._vp(d_vtr), n, xg._vp(d_x), xg._stream())
    d_t = dev(iso_tr - p1_tr, torch.float32)
    d_s = torch.full((n,), 1.0 / 6.0, dtype=torch.float32, device="cuda")
    mlp = ctypes.c_void_p()
    xg._lib.call("xg_mlp_create", 7, ctypes.byref(mlp))
    e_untrained = np.median(rel_err(learned_moments(xg, mlp, v_te)[0], iso_te))
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    B, step, losses, epochs = 2048, 0, [], 40
    for epoch in range(epochs):
        perm = torch.randperm(n, device="cuda")
        lr = 2e-3 * 0.5 ** (epoch * 5 // epochs)
        for b0 in range(0, n - B + 1, B):
            idx = perm[b0:b0 + B]
            xb, tb, sb = d_x[idx].contiguous(), d_t[idx].contiguous(), d_s[idx].contiguous()
            xg._lib.call("xg_mlp_loss_grad", mlp, xg._vp(xb), xg._vp(tb), xg._vp(sb), B, xg._vp(loss), None,
                         xg._stream())
            step += 1
            xg._lib.call("xg_mlp_adam_step", mlp, None, ctypes.c_float(lr), step, xg._stream())
        losses.append(float(loss.item()))
    e_trained = rel_err(learned_moments(xg, mlp, v_te)[0], iso_te)
    e_p1 = rel_err(p1_te, iso_te)
    xg._lib.call("xg_mlp_destroy", mlp)
    assert losses[-1] < 0.5 * losses[0], losses
    assert np.median(e_trained) < 0.9 * np.median(e_p1), (np.median(e_trained), np.median(e_p1))
    assert np.median(e_trained) < 0.5 * e_untrained, (np.median(e_trained), e_untrained)

"""Benchmark of the cut-element assembly step on one GB300.

One step = CutInfo marking + ghost-facet marking + cut rules + element and
facet-patch matrices + the deterministic scatter into a compressed-row
matrix (xg_cutfem_step / xg_st_cutfem_step), for every form of the workload,
replayed as one CUDA graph (xg_step_graph_launch).  metric = cut (IF)
elements per second.  All inputs are synthetic and seeded (the reference
publishes no dataset).

Workloads (--workload):
  c2 (default)  3D CutFEM Poisson: unit cube, 64^3 cubes x 6 Kuhn tetrahedra
                (1,572,864 tets), level set
                phi = |x - 0.5| - 0.3 + 0.02 sin(7x) sin(7y) sin(7z) as P1 (with
                InterpolateToP1's +1e-14 perturbation), P2 H1 space, NEG-domain
                stiffness, Nitsche interface terms (lambda = 10 k^2, scaled by
                1/h) on IF and ghost penalty 0.1/h^2 (u - u')(v - v') on the
                facets between HASNEG and IF elements.
  c1            the 2D circle case ([-1,1]^2, 40 x 40 x 2 triangles,
                phi = sqrt(x^2 + y^2) - 0.5, P1, u v + grad u . grad v on NEG and
                u v on IF) as 512 replicas in one mesh (one launch).
  c3            512 independent unit-cube tet meshes of log-uniform sizes
                1e3..2e5 tets, rotated-ellipsoid level sets, H1 order drawn from
                {1, 2, 3}; the meshes of one order form one disconnected mesh,
                the three order groups run as concurrent branches of one graph.
                Form: the c2 form (stiffness + Nitsche + ghost penalty).
  c5            space-time: [0,1]^2 with 256 x 256 x 2 triangles, P1 in space x
                P1 in time, circle of radius 0.25 moving on
                (0.5 + 0.2 cos 2 pi t, 0.5 + 0.2 sin 2 pi t), 16 slabs of
                dt = 1/16, convection-diffusion form of the unfitted space-time
                DG demo with ghost penalty; the 16 slab steps are one graph.
  hex           quadrilateral / hexahedral straight-cut rules: Integrate of
                the NEG volume, POS volume and IF area (order 4, direction
                policy OPTIMAL) on the unit cube with --n^3 hexahedra (default
                128^3 = 2,097,152) and the octant sphere |x| - 0.7234436998 of
                the reference's hex test; one step = the three integrals.

    python bench.py [--steps K] [--warmup W] [--precision fp64|mixed] [--workload c2|c1|c3|c4|c5|hex]
                    [--impl xg|reference]
"""
import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cut elems/s, rule+assembly, 1 GB300: plain FP64 vs learned/mixed at equal error"
UNIT = "cut_elems/s"
SEED = 20261203
C5_DT = 1.0 / 16
C5_SLABS = 16
C5_KT = [1]  # time order of the c5 level set (set from --kt)


# ----------------------------------------------------------------------------
# workloads (host side, shared by both arms)
# ----------------------------------------------------------------------------
def c2_mesh(n):
    from ngsxfem_gb300.meshes import MakeStructured3DMesh
    m = MakeStructured3DMesh(n)
    X, Y, Z = m.coords.T
    vals = np.sqrt((X - .5) ** 2 + (Y - .5) ** 2 + (Z - .5) ** 2) - 0.3 + 0.02 * np.sin(7 * X) * np.sin(7 * Y) * np.sin(
        7 * Z)
    return m, vals


def terms_c2(order):
    lam = 10.0 * order * order
    return [
        dict(kind=1, domain=0, coef=1.0, hpow=0),       # grad u . grad v on NEG
        dict(kind=2, domain=2, coef=-1.0, hpow=0),      # -(n.grad u) v on IF
        dict(kind=3, domain=2, coef=-1.0, hpow=0),      # -(n.grad v) u on IF
        dict(kind=0, domain=2, coef=lam, hpow=-1),      # lambda/h u v on IF
        dict(kind=5, domain=0, coef=0.1, hpow=-2),      # 0.1/h^2 (u-u')(v-v') on ghost facets
    ]


def terms_dg(order):
    """demos/fictdom_dg.py:120-135 (unfitted DG Poisson on an L2 space):
    stiffness on NEG, Nitsche on IF, the symmetric interior-penalty skeleton
    on the facets between HASNEG elements (cut to NEG), ghost penalty."""
    lam = 10.0 * order * order
    return [
        dict(kind=1, domain=0, coef=1.0, hpow=0),       # grad u . grad v on NEG
        dict(kind=2, domain=2, coef=-1.0, hpow=0),      # -(n.grad u) v on IF
        dict(kind=3, domain=2, coef=-1.0, hpow=0),      # -(n.grad v) u on IF
        dict(kind=0, domain=2, coef=lam, hpow=-1),      # lambda/h u v on IF
        dict(kind=7, domain=0, coef=lam, hpow=-1),      # lambda/h [u][v] on the NEG part of the facets
        dict(kind=8, domain=0, coef=-0.5, hpow=0),      # -{grad u . n_F}[v]
        dict(kind=9, domain=0, coef=-0.5, hpow=0),      # -[u]{grad v . n_F}
        dict(kind=5, domain=0, coef=0.1, hpow=-2),      # 0.1/h^2 (u-u')(v-v') on ghost facets
    ]


def terms_c1():
    return [
        dict(kind=0, domain=0, coef=1.0, hpow=0),       # u v on NEG (order 2)
        dict(kind=1, domain=0, coef=1.0, hpow=0),       # grad u . grad v on NEG (order 0)
        dict(kind=0, domain=2, coef=1.0, hpow=0),       # u v on IF (order 2)
    ]


def terms_c5(t0):
    """demos/spacetime/spacetimeDG_unfitted.py:158-168 without deformation:
    v dt(u) dQ + dt grad u.grad v dQ + dt v (w.grad u) dQ + u v dOmold
    + ghost penalty (gamma dt / h^2 and gamma dt^2 / h^3 patch terms)."""
    w = 0.4 * math.pi
    gamma = 0.05
    return [
        dict(kind=6, domain=0, coef=1.0),
        dict(kind=1, domain=0, coef=C5_DT),
        dict(kind=4, domain=0, coef=C5_DT, bc=(0.0, w, 0.0), bs=(-w, 0.0, 0.0), omega=2 * math.pi, t0=t0, dt=C5_DT),
        dict(kind=0, domain=0, coef=1.0, tref=0.0),
        dict(kind=5, coef=gamma * C5_DT, hpow=-2),
        dict(kind=5, coef=gamma * C5_DT * C5_DT, hpow=-3),
    ]


def c1_mesh(copies):
    from ngsxfem_gb300.meshes import replicated_circle_2d
    return replicated_circle_2d(copies)


def c3_groups(count):
    """The c3 meshes grouped by order: {order: (union mesh, vertex values)}."""
    from ngsxfem_gb300.meshes import MakeStructured3DMesh, batched_ellipsoids, concatenate, ellipsoid_values
    spec = batched_ellipsoids(count, seed=SEED)
    cache = {}
    groups = {}
    for n, order, centre, axes, rot in spec:
        if n not in cache:
            cache[n] = MakeStructured3DMesh(n)
        m = cache[n]
        groups.setdefault(order, ([], []))
        groups[order][0].append(m)
        groups[order][1].append(ellipsoid_values(m.coords, centre, axes, rot))
    return {k: (concatenate(ms), np.concatenate(vs)) for k, (ms, vs) in sorted(groups.items())}


def c5_mesh(n=256):
    from ngsxfem_gb300.meshes import MakeStructured2DMesh
    return MakeStructured2DMesh(n, n)


def c5_slab_values(m, slab, kt_l):
    """Vertex values of the moving circle at the slab's Gauss-Lobatto time nodes
    (time-major, (kt_l+1) x nv), not yet perturbed."""
    nodes = [0.0, 1.0] if kt_l == 1 else [0.0, 0.5, 1.0]
    out = []
    for x in nodes:
        t = (slab + x) * C5_DT
        cx, cy = 0.5 + 0.2 * math.cos(2 * math.pi * t), 0.5 + 0.2 * math.sin(2 * math.pi * t)
        out.append(np.sqrt((m.coords[:, 0] - cx) ** 2 + (m.coords[:, 1] - cy) ** 2) - 0.25)
    return np.stack(out)


def workload_config(args):
    if args.workload == "dg":
        return {"workload": "3D unfitted DG Poisson (fictdom_dg form), %d^3x6 Kuhn tets, L2 P%d: NEG stiffness + "
                            "Nitsche IF + interior-penalty / flux skeleton on the NEG part of the (HASNEG, HASNEG) "
                            "facets + ghost penalty 0.1/h^2" % (args.n, args.order)}
    if args.workload == "c2":
        return {"workload": "3D CutFEM Poisson, %d^3x6 Kuhn tets, P%d, NEG stiffness + Nitsche IF + ghost "
                            "penalty 0.1/h^2" % (args.n, args.order)}
    if args.workload == "c1":
        return {"workload": "2D circle r=0.5 on [-1,1]^2, 40x40x2 tris, P1, NEG mass+stiffness + IF mass, "
                            "%d replicas in one mesh" % args.copies}
    if args.workload == "c3":
        return {"workload": "%d unit-cube Kuhn tet meshes, log-uniform 1e3..2e5 tets, rotated ellipsoids, orders "
                            "U{1,2,3}, c2 form, one graph (3 concurrent order groups)" % args.meshes}
    return {"workload": "space-time 2D, 256^2x2 tris, P1 x P%d(time), moving circle r=0.25, %d slabs dt=1/16, "
                        "convection-diffusion + ghost penalty, one graph" % (args.kt, C5_SLABS)}


# ----------------------------------------------------------------------------
# reference arm / CPU baseline: the oracle (CPU statement of the path)
# ----------------------------------------------------------------------------
def cpu_prepare(args, sample):
    """The oracle's inputs for the workload (or its bounded sample): a list of
    jobs and a description of the sample.  Not timed."""
    from oracle import oracle as orc
    if args.workload == "c5":
        m = c5_mesh()
        sp = orc.Space(m, 1)
        slabs = list(range(C5_SLABS)) if not sample else [0, 5, 10, 15]
        jobs = []
        for s in slabs:
            lst = np.stack([orc.interpolate_p1_perturb(x) for x in c5_slab_values(m, s, args.kt)])
            jobs.append(("st", sp, lst, terms_c5(s * C5_DT)))
        desc = "all %d slabs" % C5_SLABS if len(slabs) == C5_SLABS else "slabs %s of %d" % (slabs, C5_SLABS)
        return jobs, desc
    if args.workload in ("c2", "dg"):
        m, vals = c2_mesh(args.n)
        tf = terms_dg if args.workload == "dg" else terms_c2
        groups = [(m, vals, args.order, tf(args.order), True)]
        desc = "full workload"
    elif args.workload == "c1":
        copies = args.copies if not sample else min(args.copies, 64)
        m, vals = c1_mesh(copies)
        groups = [(m, vals, 1, terms_c1(), False)]
        desc = "full workload" if copies == args.copies else "%d of %d replicas" % (copies, args.copies)
    else:
        count = args.meshes if not sample else min(args.meshes, 48)
        groups = [(m, v, k, terms_c2(k), True) for k, (m, v) in c3_groups(count).items()]
        desc = "full workload" if count == args.meshes else "the first %d of the %d meshes" % (count, args.meshes)
    jobs = []
    for m, vals, order, terms, ghost in groups:
        sp = orc.Space(m, order, l2=args.workload == "dg")
        jobs.append(("plain", sp, orc.interpolate_p1_perturb(vals), terms, ghost))
    return jobs, desc


def cpu_pass(jobs, nth):
    """One timed CPU pass over the prepared jobs: (seconds, cut elements)."""
    from oracle import oracle as orc
    t_tot, n_cut = 0.0, 0
    for job in jobs:
        if job[0] == "plain":
            _, sp, l, terms, ghost = job
            t0 = time.perf_counter()
            sp.pipeline(l, terms, ghost, nth)
            t_tot += time.perf_counter() - t0
            dom, _, _ = sp.cutinfo(l, nth)
        else:
            _, sp, lst, terms = job
            t0 = time.perf_counter()
            dom, _, bits = sp.cutinfo_st(lst, C5_KT[0], nth)
            fb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
            t2 = []
            for t in terms:
                t = dict(t)
                t["defined_on"] = fb if t["kind"] == orc.TERM_GHOST_MASS else bits[5]
                t2.append(t)
            sp.assemble_st(lst, C5_KT[0], 1, 2, t2, nth)
            t_tot += time.perf_counter() - t0
        n_cut += int((dom == 2).sum())
    return t_tot, n_cut


# ----------------------------------------------------------------------------
# c4: learned cut quadrature on P2 level sets
# ----------------------------------------------------------------------------
TET_EDGES = [(0, 1), (0, 2), (0, 3), (1, 2), (1, 3), (2, 3)]


def c4_eval_values(n=48, R=0.3, r=0.1):
    """Element-local P2 nodal values of the torus level set
    sqrt((sqrt((x-.5)^2 + (y-.5)^2) - R)^2 + (z-.5)^2) - r on the n^3 x 6 Kuhn
    mesh, restricted to the elements whose P1 interpolant (with the +1e-14
    perturbation) is cut."""
    from ngsxfem_gb300.meshes import MakeStructured3DMesh
    m = MakeStructured3DMesh(n)

    def phi(p):
        q = np.sqrt((p[..., 0] - .5) ** 2 + (p[..., 1] - .5) ** 2) - R
        return np.sqrt(q ** 2 + (p[..., 2] - .5) ** 2) - r
    P = m.coords[m.elements]
    vals = np.stack([phi(P[:, i]) for i in range(4)] + [phi(0.5 * (P[:, a] + P[:, b])) for a, b in TET_EDGES], 1)
    p1 = np.where(np.abs(vals[:, :4]) < 1e-14, 1e-14, vals[:, :4])
    cut = (p1.min(1) < 0) & (p1.max(1) > 0)
    return m, np.ascontiguousarray(vals[cut])


def c4_train_values(n, seed):
    """Training P2 values: half drawn as the configuration states (N(0,1), shifted to a
    zero crossing, scaled to max |v| = 1), half mildly curved (a level set that
    the mesh resolves, the regime of the evaluation mesh)."""
    from oracle import learned_ref as L
    rng = np.random.default_rng(seed)
    return np.concatenate([L.spec_values(n // 2, rng), L.resolved_values(n - n // 2, rng)])


def run_c4(args):
    ws, rank = dist_env()
    sub = args.plain == "subdiv"
    L = args.subdivlvl
    plain_name = ("subdivision rule, level %d (the reference's CutIntegrationRule for a P2 level set, "
                  "cutint/xintegration.cpp:1626-1754)" % L) if sub else \
        "isoparametric rule (LevelSetMeshAdaptation + straight cut, order 8)"
    cfg = {"workload": "learned cut quadrature, P2 torus (R=0.3, r=0.1) on 48^3x6 Kuhn tets; MLP 10-256-256-24 "
                       "trained on %d P2 value sets; plain = %s" % (args.train, plain_name)}
    m, vals = c4_eval_values()
    n = len(vals)
    cfg.update({"n_tets": int(m.ne), "n_cut": n})
    if args.impl == "reference":
        if rank != 0:
            return
        from oracle import oracle as orc
        nth = os.cpu_count() or 1
        def rule():
            if sub:
                orc.subdiv_moments_p2(vals, L, nth)
            else:
                orc.iso_moments_tet(vals, 8, True, nth)
        for _ in range(args.warmup):
            rule()
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            rule()
            times.append(time.perf_counter() - t0)
        t = float(np.mean(times))
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": n / t, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": n / t, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": "all cut elements per step: per-element %s (oracle)" % plain_name},
            "e2e": {"value": n / t, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    import torch
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    from ngsxfem_gb300 import build as xbuild
    xbuild.build()
    from ngsxfem_gb300 import _lib
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    vp = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731

    def moments(d_v, order, deform, out=None):
        out = out if out is not None else torch.zeros((d_v.shape[0], 35), dtype=torch.float64, device="cuda")
        _lib.call("xg_iso_moments_tet", vp(d_v), d_v.shape[0], order, deform, vp(out), None, sp)
        return out

    sd_err = torch.zeros(1, dtype=torch.int32, device="cuda")

    def subdiv_moments(d_v, level, out=None):
        out = out if out is not None else torch.zeros((d_v.shape[0], 35), dtype=torch.float64, device="cuda")
        _lib.call("xg_subdiv_moments_tet", vp(d_v), d_v.shape[0], level, vp(out), vp(sd_err), sp)
        return out

    # ---- training set and its targets (GPU isoparametric rule) ----
    t0 = time.perf_counter()
    v_tr = torch.from_numpy(c4_train_values(args.train, SEED)).cuda()
    nc_tr = torch.zeros(args.train, dtype=torch.int32, device="cuda")
    if sub:
        iso_tr = subdiv_moments(v_tr, L)
    else:
        iso_tr = moments(v_tr, 8, 1)
        _lib.call("xg_iso_moments_tet", vp(v_tr), args.train, 8, 1, vp(iso_tr), vp(nc_tr), sp)
    p1_tr = moments(v_tr, 4, 0)
    t_tr = (iso_tr - p1_tr).float()
    # samples the network is not meant to take (the fallback's): defects above
    # 5 % of the element measure or searches that did not converge
    keep = (t_tr.abs().amax(1) * 6 <= 0.05) & (nc_tr == 0)
    v_tr, t_tr = v_tr[keep].contiguous(), t_tr[keep].contiguous()
    n_tr = int(v_tr.shape[0])
    n_tr_all = args.train
    x_tr = torch.zeros((n_tr, 10), dtype=torch.float32, device="cuda")
    _lib.call("xg_learned_features", vp(v_tr), n_tr, vp(x_tr), sp)
    s_tr = torch.full((n_tr,), 1.0 / 6.0, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    t_targets = time.perf_counter() - t0
    del iso_tr, p1_tr, nc_tr
    mlp = ctypes.c_void_p()
    _lib.call("xg_mlp_create", SEED, ctypes.byref(mlp))
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    B, step, losses = 8192, 0, []
    g = torch.Generator(device="cuda")
    g.manual_seed(SEED)
    t0 = time.perf_counter()
    for ep in range(args.epochs):
        perm = torch.randperm(n_tr, device="cuda", generator=g)
        lr = 2e-3 * (0.5 ** (ep * 5 // max(args.epochs, 1)))
        for b0 in range(0, n_tr - B + 1, B):
            idx = perm[b0:b0 + B]
            xb, tb, sb = x_tr[idx].contiguous(), t_tr[idx].contiguous(), s_tr[idx].contiguous()
            _lib.call("xg_mlp_loss_grad", mlp, vp(xb), vp(tb), vp(sb), B, vp(loss), None, sp)
            step += 1
            _lib.call("xg_mlp_adam_step", mlp, None, ctypes.c_float(lr), step, sp)
        losses.append(float(loss.item()))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t0
    del v_tr, x_tr, t_tr, s_tr

    # ---- the network alone: tensor-core fused kernel vs the FP32 SIMT products ----
    nb = min(n_tr_all, 2_000_000)
    xb_all = torch.from_numpy(np.random.default_rng(SEED).uniform(-1, 1, (nb, 10)).astype(np.float32)).cuda()
    y_tc = torch.zeros((nb, 24), dtype=torch.float32, device="cuda")
    y_simt = torch.zeros_like(y_tc)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    for _ in range(3):
        _lib.call("xg_mlp_forward_tc", mlp, vp(xb_all), nb, vp(y_tc), sp)
        _lib.call("xg_mlp_forward", mlp, vp(xb_all), nb, vp(y_simt), sp)
    ev[0].record(stream)
    for _ in range(5):
        _lib.call("xg_mlp_forward_tc", mlp, vp(xb_all), nb, vp(y_tc), sp)
    ev[1].record(stream)
    for _ in range(5):
        _lib.call("xg_mlp_forward", mlp, vp(xb_all), nb, vp(y_simt), sp)
    ev[2].record(stream)
    torch.cuda.synchronize()
    _lib.check(_lib.load().xg_mlp_check(mlp), "tensor-core forward")
    ms_tc = ev[0].elapsed_time(ev[1]) / 5
    ms_simt = ev[1].elapsed_time(ev[2]) / 5
    fl = 2.0 * (10 * 256 + 256 * 256 + 256 * 24) * nb
    diff = float((y_tc - y_simt).abs().max() / y_simt.abs().max())
    mlp_fwd = {"rows": nb, "tensor_core_ms": ms_tc, "simt_fp32_ms": ms_simt, "speedup": ms_simt / ms_tc,
               "tensor_core_tflops": fl / (ms_tc * 1e-3) / 1e12, "simt_tflops": fl / (ms_simt * 1e-3) / 1e12,
               "max_rel_diff_tc_vs_simt": diff,
               "note": "tcgen05 BF16 (activations too) with FP32 accumulation vs SIMT FP32 FMA with BF16 weights"}
    del xb_all, y_tc, y_simt

    # ---- evaluation on the torus mesh ----
    d_v = torch.from_numpy(vals).cuda()
    out_plain = torch.zeros((n, 35), dtype=torch.float64, device="cuda")
    out_learn = torch.zeros_like(out_plain)
    out_p1 = torch.zeros_like(out_plain)

    def plain():
        if sub:
            subdiv_moments(d_v, L, out_plain)
        else:
            moments(d_v, 8, 1, out_plain)

    nfb = torch.zeros(1, dtype=torch.int32, device="cuda")

    def learned(kappa=args.kappa):
        _lib.call("xg_learned_moments_tet_ex", mlp, vp(d_v), n, ctypes.c_double(kappa), L if sub else -1,
                  vp(out_learn), vp(nfb), sp)

    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timeit(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        st = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        en = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        for k in range(args.steps):
            flush.fill_(float(k))
            st[k].record(stream)
            fn()
            en[k].record(stream)
        torch.cuda.synchronize()
        return float(np.mean([a.elapsed_time(b) for a, b in zip(st, en)]))

    with Clocks(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms_learn = timeit(learned)
        ms_plain = timeit(plain)
    moments(d_v, 4, 0, out_p1)
    torch.cuda.synchronize()
    n_fallback = int(nfb.item())
    ref = out_plain.cpu().numpy()
    # moment errors in units of the element measure (1/6 for the reference tet)
    e_learn = np.abs(out_learn.cpu().numpy() - ref).max(1) * 6
    e_p1 = np.abs(out_p1.cpu().numpy() - ref).max(1) * 6

    def stats(e):
        return {"median": float(np.median(e)), "p99": float(np.quantile(e, 0.99)), "max": float(e.max()),
                "frac_le_1e-6": float((e <= 1e-6).mean()), "frac_le_1e-4": float((e <= 1e-4).mean()),
                "frac_le_1e-3": float((e <= 1e-3).mean())}
    errs = {"definition": "max over the 35 moments of |m - m_plain| / (measure of the element)",
            "learned_vs_plain": stats(e_learn), "straight_cut_vs_plain": stats(e_p1)}
    if sub:
        # the isoparametric rule and the finer subdivision against the plain rule
        out_iso = moments(d_v, 8, 1)
        out_fine = subdiv_moments(d_v, L + 1)
        torch.cuda.synchronize()
        errs["isoparametric_vs_plain"] = stats(np.abs(out_iso.cpu().numpy() - ref).max(1) * 6)
        errs["subdivision_level_%d_vs_plain" % (L + 1)] = stats(np.abs(out_fine.cpu().numpy() - ref).max(1) * 6)
        assert int(sd_err.item()) == 0, "subdivision rule error %d" % int(sd_err.item())
        del out_iso, out_fine
    sweep = {}
    for kap in (0.0, 0.01, 0.02, 0.05, -1.0):
        learned(kap)
        torch.cuda.synchronize()
        e = np.abs(out_learn.cpu().numpy() - ref).max(1) * 6
        sweep[str(kap)] = {"fallback_frac": float(nfb.item()) / n, "median": float(np.median(e)),
                           "p99": float(np.quantile(e, 0.99)), "max": float(e.max())}
    errs["fallback_sweep (kappa_max: result)"] = sweep
    # ---- end to end: host values in, moments out ----
    h_v = torch.from_numpy(vals).pin_memory()
    h_out = torch.empty((n, 35), dtype=torch.float64).pin_memory()
    e2e = []
    for k in range(args.steps + 2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d_v.copy_(h_v, non_blocking=True)
        learned()
        h_out.copy_(out_learn, non_blocking=True)
        stream.synchronize()
        if k >= 2:
            e2e.append(time.perf_counter() - t0)
    e2e_s = float(np.mean(e2e))
    flops_mlp = 2.0 * (10 * 256 + 256 * 256 + 256 * 24) * n
    pk = peaks()
    peak_tc = pk["bf16_tflops"] if pk else 1900.0
    ach = flops_mlp / (ms_learn * 1e-3) / 1e12
    cfg.update({"train": {"samples": args.train, "epochs": args.epochs, "batch": B, "steps": step,
                          "targets_s": t_targets, "train_s": t_train, "loss_first_last": [losses[0], losses[-1]]},
                "plain_ms": ms_plain, "learned_ms": ms_learn, "learned_speedup_vs_plain": ms_plain / ms_learn,
                "kappa_max": args.kappa, "fallback_frac": n_fallback / n, "train_kept": n_tr,
                "errors": errs, "l2": "flushed between timed steps (512 MB write)",
                "plain": "GPU " + plain_name + " (FP64), also the fallback and the judge of the error"})
    out = {
        "metric": METRIC, "value": n / (ms_learn * 1e-3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_learn, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 weights, f32 accumulation, f64 moments", "data": "synthetic",
        "config": cfg,
        "e2e": {"value": n / e2e_s, "unit": UNIT, "h2d_bytes_per_step": n * 80, "d2h_bytes_per_step": n * 280,
                "ms_per_step": e2e_s * 1e3},
        "roofline": {"bound": "tensor", "kernel": "k_mlp_tc (fused three-layer MLP, tcgen05 BF16)",
                     "achieved": mlp_fwd["tensor_core_tflops"], "peak": peak_tc, "unit": "TFLOP/s",
                     "frac": mlp_fwd["tensor_core_tflops"] / peak_tc, "traffic": None,
                     "peak_source": "measured bf16" if pk else "fallback",
                     "learned_path_whole": {"achieved": ach, "frac": ach / peak_tc},
                     "dominant_stage": "the fallback's subdivision rule (k_sd_fill, FP64-bound: 88 % of the FP64 "
                                       "pipe with full warps in the ncu capture of the same kernels)"
                     if sub else "the fallback's isoparametric rule (k_tet_moments, FP64)"},
        "mlp_forward": mlp_fwd,
        "clocks": clk.summary(),
        # moments, features, the fused network, correction; the fallback: memset and list, then
        # (subdivision) per tree level classify + three scans of three kernels + emit, the plain and
        # cut leaf fills and the per-element sums (one chunk of at most 32,768 elements), or
        # (isoparametric) one kernel
        "gpu_launches": args.steps * (4 + ((2 + ((L + 1) * 11 + 3 if sub else 1)) if args.kappa >= 0 else 0)),
    }
    if args.cpu_baseline:
        from oracle import oracle as orc
        nth = os.cpu_count() or 1
        def rule():
            if sub:
                orc.subdiv_moments_p2(vals, L, nth)
            else:
                orc.iso_moments_tet(vals, 8, True, nth)
        rule()
        t0 = time.perf_counter()
        rule()
        tc = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / tc, "unit": UNIT, "cores": nth, "kind": "port",
                               "sample": "all cut elements: per-element %s (oracle), 1 timed pass" % plain_name}
    _lib.call("xg_mlp_destroy", mlp)
    print(json.dumps(out))


HEX_R = 0.7234436998


def hex_values(n):
    """n^3 hexahedra of the unit cube and the vertex values of |x| - r with
    InterpolateToP1's |v| < 1e-14 -> 1e-14 perturbation."""
    from ngsxfem_gb300.meshes import MakeStructured3DMesh
    m = MakeStructured3DMesh(n, hexes=True)
    v = np.sqrt((m.coords ** 2).sum(1)) - HEX_R
    v[np.abs(v) < 1e-14] = 1e-14
    return m, v


def hex_cut_count(m, v):
    s = v[m.elements] >= 0
    return int((s.any(1) & ~s.all(1)).sum())


def hex_cpu_sample(n_cpu, nth):
    """Oracle Integrate (nth host threads) of the three domains on an n_cpu^3
    sample: (cut elements / s, seconds)."""
    from oracle import oracle as orc
    m, v = hex_values(n_cpu)
    orc.quad_integrate(m, v, 0, 4, nthreads=nth)
    t0 = time.perf_counter()
    for dt in (0, 1, 2):
        orc.quad_integrate(m, v, dt, 4, nthreads=nth)
    t = time.perf_counter() - t0
    return hex_cut_count(m, v) / t, t


def run_hex(args):
    ws, rank = dist_env()
    n = args.n if args.n != 64 else 128
    m, v = hex_values(n)
    n_cut = hex_cut_count(m, v)
    cfg = {"workload": "quad/hex straight-cut rules: Integrate NEG, POS, IF (order 4, OPTIMAL) on %d^3 hexahedra, "
                       "octant sphere r=%.10f" % (n, HEX_R), "n_hex": int(m.ne), "n_cut": n_cut,
           "l2": "flushed between timed steps (512 MB write)"}
    n_cpu = n  # the full workload: the cut fraction changes with the resolution
    nth = os.cpu_count() or 1
    if args.impl == "reference":
        if rank != 0:
            return
        for _ in range(args.warmup):
            hex_cpu_sample(8, nth)
        vals = [hex_cpu_sample(n_cpu, nth)[0] for _ in range(args.steps)]
        val = float(np.mean(vals))
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": nth, "kind": "port",
                             "sample": "the same integrals on %d^3 hexahedra (oracle, %d threads)" % (n_cpu, nth)},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    from ngsxfem_gb300 import build as xbuild
    xbuild.build()
    from ngsxfem_gb300 import _lib, xfem
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    dm = xfem.device_mesh(m)
    d_l = torch.from_numpy(v).cuda()
    res = torch.zeros(3, dtype=torch.float64, device="cuda")

    def step():
        for dt in range(3):
            _lib.call("xg_integrate_ex", dm.h, ctypes.c_void_p(d_l.data_ptr()), dt, 4, xfem.OPTIMAL, 0, 0, 0, None,
                      ctypes.c_void_p(res.data_ptr() + 8 * dt), sp)

    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for _ in range(args.warmup):
        step()
    dm.check()
    st = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    en = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))
            st[k].record(stream)
            step()
            en[k].record(stream)
        torch.cuda.synchronize()
    ms = float(np.mean([a.elapsed_time(b) for a, b in zip(st, en)]))
    dm.check()
    r = res.cpu().numpy()
    exact = {"NEG": math.pi * HEX_R ** 3 / 6, "POS": 1 - math.pi * HEX_R ** 3 / 6, "IF": math.pi * HEX_R ** 2 / 2}
    cfg["integrals"] = {k: float(r[i]) for i, k in enumerate(("NEG", "POS", "IF"))}
    cfg["error_vs_exact_sphere"] = {k: float(r[i] - exact[k]) for i, k in enumerate(("NEG", "POS", "IF"))}
    # end to end: host vertex values in, the three integrals out
    h_l = torch.from_numpy(v).pin_memory()
    h_r = torch.empty(3, dtype=torch.float64).pin_memory()
    e2e = []
    for k in range(args.steps + 2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d_l.copy_(h_l, non_blocking=True)
        step()
        h_r.copy_(res, non_blocking=True)
        stream.synchronize()
        if k >= 2:
            e2e.append(time.perf_counter() - t0)
    e2e_s = float(np.mean(e2e))
    # algorithmic bytes per step: per integral the vertex ids (32 B), the
    # corner coordinates and values (8 x 4 x 8 B) of every hexahedron
    alg = 3 * m.ne * (32 + 256)
    pk = peaks()
    peak = pk["hbm_gbs"] if pk else 6800.0
    ach = alg / (ms * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": n_cut / (ms * 1e-3), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "config": cfg,
        "elements_per_s": m.ne / (ms * 1e-3),
        "e2e": {"value": n_cut / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(v.nbytes), "d2h_bytes_per_step": 24,
                "ms_per_step": e2e_s * 1e3},
        "roofline": {"bound": "hbm", "kernel": "k_qint_uncut<3> + k_qint_cut<3>", "achieved": ach, "peak": peak,
                     "unit": "GB/s", "frac": ach / peak, "traffic": None,
                     "peak_source": "measured" if pk else "fallback",
                     "note": "bound by the FP64 pipe (per-point element map and cut rules), not by HBM"},
        "clocks": clk.summary(),
        # per integral: uncut pass, cut pass, block sums, final sum
        "gpu_launches": args.steps * 12,
    }
    if args.cpu_baseline:
        val, t = hex_cpu_sample(n_cpu, nth)
        out["cpu_baseline"] = {"value": val, "unit": UNIT, "cores": nth, "kind": "port",
                               "sample": "the same integrals on %d^3 hexahedra (oracle, %d threads, %.2f s)"
                                         % (n_cpu, nth, t)}
    print(json.dumps(out))


def run_reference(args):
    """The reference arm: the CPU statement of the path (the reference itself
    needs NGSolve and cannot be built), all host threads, same workload."""
    ws, rank = dist_env()
    if rank != 0:
        return
    nth = os.cpu_count() or 1
    C5_KT[0] = args.kt
    jobs, desc = cpu_prepare(args, args.workload in ("c3", "c5"))
    for _ in range(args.warmup):
        cpu_pass(jobs, nth)
    times, n_cut = [], 0
    for _ in range(args.steps):
        t, n_cut = cpu_pass(jobs, nth)
        times.append(t)
    t = float(np.mean(times))
    value = n_cut / t
    cfg = workload_config(args)
    cfg["n_cut_per_step"] = n_cut
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": cfg,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port",
                         "sample": desc + " per step (oracle C++ restatement of ngsxfem's path; the reference needs "
                                          "NGSolve, which cannot be built here)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


# ----------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, dev_index):
        self.dev = dev_index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.p is not None:
            time.sleep(0.25)
            self.p.terminate()
            out, _ = self.p.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# DRAM bytes (read + write) per launch of a stage's dominant kernel from one
# ncu capture (dram__bytes_read.sum + dram__bytes_write.sum, one pass, on the
# full-size workload).  Each entry names the first 16 hex digits of the
# sha256 of the source file it was captured on; when that file has changed
# since, the line reports traffic null instead of a stale figure.
TRAFFIC = {
    ("c2", "patch"): {"bytes": 74575872 + 196613376, "source": "ngsxfem_gb300/csrc/xg_asm.cu",
                      "sha16": "913d9771b561e503"},
}


def traffic_for(workload, stage):
    t = TRAFFIC.get((workload, stage))
    if t is None:
        return None
    import hashlib
    with open(os.path.join(ROOT, t["source"]), "rb") as f:
        sha = hashlib.sha256(f.read()).hexdigest()[:16]
    return t["bytes"] if sha == t["sha16"] else None


def patch_exact_flops(dim, k):
    """FP64 operations of one facet patch in the basis-change kernel as
    executed: the node images (2 (D+1)^2 per node and side), the columns of
    both basis changes (an evaluation of about 3 operations per function and
    node, about 4 per coefficient of the hierarchical solve), W = Mh C over the
    rows of degree <= the column's degree, and the entries (block sums over
    the same rows, 4 more per diagonal-block entry, 4 per coupling entry)."""
    n = (k + 1) * (k + 2) // 2 if dim == 2 else (k + 1) * (k + 2) * (k + 3) // 6
    nedge = 3 if dim == 2 else 6
    deg = [1] * (dim + 1)
    if k == 2:
        deg += [2] * nedge
    elif k == 3:
        deg += [2, 3] * nedge + [3] * (1 if dim == 2 else 4)
    cnt = {d: sum(1 for x in deg if x <= d) for d in (1, 2, 3)}
    nodes = 2 * n * 2 * (dim + 1) * (dim + 1) / (dim + 1)
    cols = 2 * n * (3 * n + 4 * n)
    w = 2 * n * sum(2 * cnt[deg[j]] for j in range(n))
    blocks = 2 * sum((n - a) * (2 * cnt[deg[a]] + 4) for a in range(n))
    cross = n * n * 4
    return nodes + cols + w + blocks + cross


def fp64_peak(torch):
    a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    best = None
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        t = s.elapsed_time(e) * 1e-3
        best = t if best is None else min(best, t)
    return 2 * 4096 ** 3 / best / 1e12


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


class Gpu:
    """The GPU side of one workload: forms, device level sets, outputs."""

    def __init__(self, args):
        import torch
        from ngsxfem_gb300 import _lib
        from ngsxfem_gb300 import xfem as xg
        self.torch, self._lib, self.xg = torch, _lib, xg
        self.args = args
        self.prec = 0 if args.precision == "fp64" else 1
        self.stream = torch.cuda.current_stream()
        self.sp = ctypes.c_void_p(self.stream.cuda_stream)
        self.keep = []
        self.entries = []  # dicts: form, lset, st, out, counts

    # --- objects
    def lset(self, vals):
        t = self.torch.from_numpy(np.ascontiguousarray(vals, dtype=np.float64)).cuda()
        self._lib.call("xg_interpolate_p1_perturb", ctypes.c_void_p(t.data_ptr()), t.numel(), 1e-14, self.sp)
        return t

    def form(self, space_h, terms):
        arr = (self._lib.Term * len(terms))()
        for k, t in enumerate(terms):
            arr[k].kind, arr[k].domain, arr[k].order = t["kind"], t["domain"], -1
            arr[k].hpow, arr[k].coef = t["hpow"], t["coef"]
            arr[k].d_defined_on = None
        f = ctypes.c_void_p()
        self._lib.call("xg_form_create", space_h, arr, len(terms), self.prec, ctypes.byref(f))
        return f

    def st_form(self, space_h, kt_l, order_time, terms):
        arr = (self._lib.StTerm * len(terms))()
        for k, t in enumerate(terms):
            B = arr[k].base
            B.kind, B.domain, B.order, B.hpow, B.coef = t["kind"], t.get("domain", 0), -1, t.get("hpow", 0), t["coef"]
            for j in range(3):
                B.b[j] = 0.0
                arr[k].bc[j] = t.get("bc", (0, 0, 0))[j]
                arr[k].bs[j] = t.get("bs", (0, 0, 0))[j]
            B.d_defined_on = None
            arr[k].tref = t.get("tref", -1.0)
            arr[k].omega, arr[k].t0, arr[k].dt = t.get("omega", 0.0), t.get("t0", 0.0), t.get("dt", 1.0)
        f = ctypes.c_void_p()
        self._lib.call("xg_st_form_create", space_h, kt_l, order_time, arr, len(terms), self.prec, ctypes.byref(f))
        return f

    def out(self, cap_rows, cap_nnz):
        torch = self.torch
        o = {"row_dof": torch.zeros(cap_rows, dtype=torch.int32, device="cuda"),
             "rowptr": torch.zeros(cap_rows + 1, dtype=torch.int64, device="cuda"),
             "cols": torch.zeros(max(cap_nnz, 1), dtype=torch.int32, device="cuda"),
             "vals": torch.zeros(max(cap_nnz, 1), dtype=torch.float64, device="cuda"),
             "counts": torch.zeros(2, dtype=torch.int64, device="cuda")}
        c = self._lib.Csr()
        c.d_row_dof, c.d_rowptr = o["row_dof"].data_ptr(), o["rowptr"].data_ptr()
        c.d_cols, c.d_vals, c.d_counts = o["cols"].data_ptr(), o["vals"].data_ptr(), o["counts"].data_ptr()
        c.cap_rows, c.cap_nnz = cap_rows, cap_nnz
        o["csr"] = c
        return o

    def eager_step(self, e):
        name = "xg_st_cutfem_step" if e["st"] else "xg_cutfem_step"
        self._lib.call(name, e["form"], ctypes.c_void_p(e["lset"].data_ptr()), ctypes.byref(e["out"]["csr"]),
                       self.sp)

    def add(self, form, lset, st, marking):
        """Registers one step, sizes its output by an eager step (the full
        pattern when small, else the step's own count plus 5 %) and records
        the marking counts of its level set."""
        cap = np.zeros(2, dtype=np.int64)
        self._lib.call("xg_form_capacity", form, cap.ctypes.data_as(ctypes.c_void_p))
        e = {"form": form, "lset": lset, "st": st}
        first = int(cap[1]) if cap[1] * 12 <= (1 << 31) else 1024
        e["out"] = self.out(int(cap[0]), first)
        self.eager_step(e)
        self.torch.cuda.synchronize()
        st_ = self._lib.load().xg_form_check(form)
        nnz = int(e["out"]["counts"][1].item())
        if st_ == self._lib.XG_ERR_CAPACITY or nnz > first:
            e["out"] = self.out(int(cap[0]), int(nnz * 1.05) + 4096)
            self.eager_step(e)
            self.torch.cuda.synchronize()
            st_ = self._lib.load().xg_form_check(form)
        self._lib.check(st_, "bench step")
        e["nrows"], e["nnz"] = (int(x) for x in e["out"]["counts"].cpu().tolist())
        e.update(marking)
        self.entries.append(e)
        return e

    def marking_plain(self, dm, lset, skeleton=False):
        """Counts of the step's sets; with skeleton=True the facet count is that
        of the ghost facets joined with the (HASNEG, HASNEG) skeleton facets."""
        torch, xg = self.torch, self.xg
        ne, nf = dm.ne, dm.nfacets
        dom = torch.zeros(ne, dtype=torch.uint8, device="cuda")
        ratio = torch.zeros(ne, dtype=torch.float64, device="cuda")
        bits = torch.zeros((8, (ne + 63) // 64), dtype=torch.int64, device="cuda")
        fb = torch.zeros((nf + 63) // 64, dtype=torch.int64, device="cuda")
        self._lib.call("xg_cutinfo_update", dm.h, xg._vp(lset), xg._vp(dom), xg._vp(ratio), xg._vp(bits), self.sp)
        self._lib.call("xg_facets_with_neighbor_types", dm.h, xg._vp(bits[5]), xg._vp(bits[4]), 1, 1, 1, xg._vp(fb),
                       self.sp)
        if skeleton:
            fs = torch.zeros_like(fb)
            self._lib.call("xg_facets_with_neighbor_types", dm.h, xg._vp(bits[5]), xg._vp(bits[5]), 1, 1, 1,
                           xg._vp(fs), self.sp)
            fb = fb | fs
        dm.check()
        return self._counts(dom, fb, nf, dm)

    def marking_st(self, dm, lset, kt_l):
        torch, xg = self.torch, self.xg
        ne, nf = dm.ne, dm.nfacets
        dom = torch.zeros(ne, dtype=torch.uint8, device="cuda")
        ratio = torch.zeros(ne, dtype=torch.float64, device="cuda")
        bits = torch.zeros((8, (ne + 63) // 64), dtype=torch.int64, device="cuda")
        fb = torch.zeros((nf + 63) // 64, dtype=torch.int64, device="cuda")
        self._lib.call("xg_cutinfo_update_st", dm.h, xg._vp(lset), kt_l, xg._vp(dom), xg._vp(ratio), xg._vp(bits),
                       self.sp)
        self._lib.call("xg_facets_with_neighbor_types", dm.h, xg._vp(bits[5]), xg._vp(bits[4]), 1, 1, 1, xg._vp(fb),
                       self.sp)
        dm.check()
        return self._counts(dom, fb, nf, dm)

    def _counts(self, dom, fb, nf, dm):
        d = dom.cpu().numpy()
        w = fb.cpu().numpy().view(np.uint64)
        n_fa = int(np.unpackbits(w.view(np.uint8), bitorder="little")[:nf].sum())
        return {"n_if": int((d == 2).sum()), "n_neg": int((d == 0).sum()), "n_facets": n_fa, "ne": dm.ne,
                "dim": dm.dim}

    def autotune(self):
        """xg_form_autotune on every spatial entry (its own level set and
        output); returns the per-process table."""
        for e in self.entries:
            if not e["st"]:
                self._lib.call("xg_form_autotune", e["form"], ctypes.c_void_p(e["lset"].data_ptr()),
                               ctypes.byref(e["out"]["csr"]), self.sp)
        self.torch.cuda.synchronize()
        L = self._lib.load()
        need = L.xg_autotune_table(None, 0)
        buf = ctypes.create_string_buffer(int(need))
        L.xg_autotune_table(buf, need)
        return json.loads(buf.value.decode() or "{}")

    # --- graph
    def graph(self):
        n = len(self.entries)
        forms = (ctypes.c_void_p * n)(*[e["form"].value for e in self.entries])
        lsets = (ctypes.c_void_p * n)(*[e["lset"].data_ptr() for e in self.entries])
        outs = (self._lib.Csr * n)(*[e["out"]["csr"] for e in self.entries])
        g = ctypes.c_void_p()
        self._lib.call("xg_step_graph_create", forms, lsets, outs, n, ctypes.byref(g))
        kc = np.zeros(1, dtype=np.int64)
        self._lib.call("xg_step_graph_kernel_count", g, kc.ctypes.data_as(ctypes.c_void_p))
        self.g, self.kernels = g, int(kc[0])
        return g

    def launch(self):
        self._lib.call("xg_step_graph_launch", self.g, self.sp)

    def graph_on(self, key):
        """A second graph of the same steps writing the outputs e[key]
        (double-buffered end-to-end runs); the steps' level sets are shared."""
        n = len(self.entries)
        forms = (ctypes.c_void_p * n)(*[e["form"].value for e in self.entries])
        lsets = (ctypes.c_void_p * n)(*[e["lset"].data_ptr() for e in self.entries])
        outs = (self._lib.Csr * n)(*[e[key]["csr"] for e in self.entries])
        g = ctypes.c_void_p()
        self._lib.call("xg_step_graph_create", forms, lsets, outs, n, ctypes.byref(g))
        return g

    def check_forms(self):
        self.torch.cuda.synchronize()
        for f in {e["form"].value for e in self.entries}:
            self._lib.check(self._lib.load().xg_form_check(ctypes.c_void_p(f)), "bench form")


def fetch_csr(gpu, e):
    """The entry's output as (global rows, global cols, vals) numpy arrays,
    row-major with ascending columns."""
    o = e["out"]
    n, z = (int(x) for x in o["counts"].cpu().tolist())
    rd = o["row_dof"][:n].cpu().numpy()
    rp = o["rowptr"][: n + 1].cpu().numpy()
    c = o["cols"][:z].cpu().numpy()
    v = o["vals"][:z].cpu().numpy()
    return np.repeat(rd.astype(np.int64), np.diff(rp)), rd[c], v


def oracle_csr(e, nth):
    """The oracle's matrix of the entry's step (CutInfo -> element and facet
    sets -> assembly) on all host threads."""
    from oracle import oracle as orc
    kind, m, vals, order, terms = e["host"]
    if kind == "st":
        lst = np.stack([orc.interpolate_p1_perturb(x) for x in vals])
        sp = orc.Space(m, 1)
        _, _, bits = sp.cutinfo_st(lst, len(vals) - 1, nthreads=nth)
        fb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
        t2 = [dict(t, defined_on=fb if t["kind"] == orc.TERM_GHOST_MASS else bits[5]) for t in terms]
        rp, cols, rv = sp.assemble_st(lst, len(vals) - 1, 1, 2, t2, nthreads=nth)
    else:
        l = orc.interpolate_p1_perturb(vals)
        sp = orc.Space(m, order, l2=e.get("l2", False))
        _, _, bits = sp.cutinfo(l, nthreads=nth)
        fb = sp.facets_with_neighbor_types(bits[5], bits[4], True, True, True)
        # skeleton terms: NEG on (HASNEG, HASNEG) facets, POS on (HASPOS, HASPOS), whole facets on the ghost facets
        fsk = {orc.NEG: sp.facets_with_neighbor_types(bits[5], bits[5], True, True, True),
               orc.POS: sp.facets_with_neighbor_types(bits[6], bits[6], True, True, True), orc.WHOLE: fb}
        t2 = [dict(t, defined_on=fb if t["kind"] == orc.TERM_GHOST_MASS else
                   (fsk[t["domain"]] if t["kind"] >= orc.TERM_SKEL_JUMP else
                    {orc.NEG: bits[5], orc.IF: bits[4], orc.POS: bits[6]}[t["domain"]])) for t in terms]
        rp, cols, rv = sp.assemble(l, t2, nthreads=nth)
    return np.repeat(np.arange(len(rp) - 1, dtype=np.int64), np.diff(rp)), cols, rv


def max_rel_err(got, ref):
    """(same pattern, max |got - ref| / max |ref|) of two row-major CSRs."""
    same = len(got[2]) == len(ref[2]) and np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    if not same:
        return False, None
    scale = float(np.max(np.abs(ref[2]))) if len(ref[2]) else 1.0
    return True, float(np.max(np.abs(got[2] - ref[2]))) / max(scale, 1e-300) if len(ref[2]) else 0.0


def time_graph(gpu, steps, warmup, flush, clk=None):
    """Mean device time (ms) of `steps` graph replays, L2 flushed before each."""
    torch = gpu.torch
    stream = gpu.stream
    for _ in range(warmup):
        gpu.launch()
    gpu.check_forms()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    torch.cuda.synchronize()
    if clk is not None:
        clk.__enter__()
    for k in range(steps):
        flush.fill_(float(k))  # L2 flush between timed steps (not timed)
        starts[k].record(stream)
        gpu.launch()
        ends[k].record(stream)
    torch.cuda.synchronize()
    if clk is not None:
        clk.__exit__(None, None, None)
    gpu.check_forms()
    return float(np.mean([a.elapsed_time(b) for a, b in zip(starts, ends)]))



def setup(args, gpu):
    """Builds the workload's forms and steps on the device; returns the config."""
    xg = gpu.xg
    cfg = workload_config(args)
    if args.workload in ("c2", "c1", "c3", "dg"):
        if args.workload in ("c2", "dg"):
            m, vals = c2_mesh(args.n)
            groups = {args.order: (m, vals)}
            tf = terms_dg if args.workload == "dg" else terms_c2
        elif args.workload == "c1":
            m, vals = c1_mesh(args.copies)
            groups = {1: (m, vals)}
            tf = lambda k: terms_c1()  # noqa: E731
        else:
            t0 = time.perf_counter()
            groups = c3_groups(args.meshes)
            cfg["host_mesh_gen_s"] = time.perf_counter() - t0
        for order, (m, vals) in groups.items():
            V = xg.L2(m, order=order) if args.workload == "dg" else xg.H1(m, order=order)
            lset = gpu.lset(vals)
            form = gpu.form(V.h, (terms_c2 if args.workload == "c3" else tf)(order))
            gpu.keep += [V, m]
            mk = gpu.marking_plain(V.dm, lset, skeleton=args.workload == "dg")
            mk["ndof_el"] = V.ndof_el
            mk["order"] = order
            if args.workload == "c1":
                mk["n_facets"] = 0  # no patch terms
            e = gpu.add(form, lset, False, mk)
            e["host"] = ("plain", m, vals, order, (terms_c2 if args.workload == "c3" else tf)(order))
            e["l2"] = args.workload == "dg"
        if args.workload == "c3":
            cfg["groups"] = {str(k): {"n_tets": int(m.ne)} for k, (m, _) in groups.items()}
    else:
        m = c5_mesh()
        dm = xg.device_mesh(m)
        sh = ctypes.c_void_p()
        gpu._lib.call("xg_space_create_st", dm.h, 1, 1, ctypes.byref(sh))
        info = np.zeros(6, dtype=np.int64)
        gpu._lib.call("xg_space_info_st", sh, info.ctypes.data_as(ctypes.c_void_p))
        gpu.keep += [m, dm]
        # one form per slab: the convection field's time origin is a form
        # parameter (t0 of b(t)), so each slab's form differs in t0 only
        for s in range(C5_SLABS):
            st_vals = c5_slab_values(m, s, args.kt)
            lset = gpu.lset(st_vals)
            form = gpu.st_form(sh, args.kt, 2, terms_c5(s * C5_DT))
            mk = gpu.marking_st(dm, lset, args.kt)
            mk["ndof_el"] = int(info[1])
            mk["order"] = 1
            e = gpu.add(form, lset, True, mk)
            e["host"] = ("st", m, st_vals, 1, terms_c5(s * C5_DT))
        gpu.st_space = sh
    return cfg


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="xg", choices=["xg", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--workload", default="c2", choices=["c2", "c1", "c3", "c4", "c5", "hex", "dg"])
    ap.add_argument("--train", type=int, default=2000000)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--kappa", type=float, default=0.05)
    ap.add_argument("--plain", default="subdiv", choices=["subdiv", "iso"],
                    help="c4: the plain rule (targets, fallback, judge): subdivision or isoparametric")
    ap.add_argument("--subdivlvl", type=int, default=3, help="c4: level of the subdivision rule")
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--order", type=int, default=2)
    ap.add_argument("--copies", type=int, default=512)
    ap.add_argument("--meshes", type=int, default=512)
    ap.add_argument("--kt", type=int, default=1, choices=[1, 2])
    ap.add_argument("--cpu-baseline", type=int, default=1)
    ap.add_argument("--check", type=int, default=1, help="error of the step against the oracle")
    ap.add_argument("--mixed", type=int, default=1, help="also time the mixed form (fp64 runs)")
    ap.add_argument("--autotune", type=int, default=1, help="tune the launch choices before timing")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.workload == "c4":
        return run_c4(args)
    if args.workload == "hex":
        return run_hex(args)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    ws, rank = dist_env()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from ngsxfem_gb300 import build as xbuild
    xbuild.build()
    gpu = Gpu(args)
    _lib = gpu._lib
    stream = gpu.stream
    cfg = setup(args, gpu)
    E = gpu.entries
    n_cut = sum(e["n_if"] for e in E)
    if args.autotune:
        cfg["autotune"] = gpu.autotune()
    gpu.graph()

    # ---------------- device-resident timing (graph replay) ----------------
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)
    if ws > 1:
        torch.distributed.barrier()
    clk = Clocks(local)
    ms = time_graph(gpu, args.steps, args.warmup, flush, clk)
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = ws * n_cut / (ms * 1e-3)

    # ---------------- stage breakdown (eager steps with stage events) ----------------
    stage_ms = np.zeros(7)
    names = ["marking", "lists", "elmat_uncut", "elmat_cut", "patch", "pattern", "scatter"]
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(8)]
    for e in evs:  # torch creates the CUDA event on first record
        e.record(stream)
    torch.cuda.synchronize()
    ev_arr = (ctypes.c_void_p * 8)(*[ctypes.c_void_p(e.cuda_event) for e in evs])
    for e in E:
        _lib.call("xg_form_stage_events", e["form"], ev_arr, 8)
        reps = max(1, min(args.steps, 5))
        for _ in range(reps):
            flush.fill_(1.0)
            gpu.eager_step(e)
            evs[7].synchronize()
            stage_ms += np.array([evs[i].elapsed_time(evs[i + 1]) for i in range(7)]) / reps
        _lib.call("xg_form_stage_events", e["form"], None, 0)
    gpu.check_forms()

    # ---------------- end to end through the C ABI with host buffers ----------------
    for e in E:
        e["h_lset"] = torch.empty(e["lset"].shape, dtype=torch.float64).pin_memory()
        e["h_lset"].copy_(e["lset"].cpu())
        o = e["out"]
        e["h_out"] = {k: torch.empty(n, dtype=o[k].dtype).pin_memory()
                      for k, n in (("row_dof", e["nrows"]), ("rowptr", e["nrows"] + 1), ("cols", e["nnz"]),
                                   ("vals", e["nnz"]), ("counts", 2))}
    e2e_times = []
    for k in range(args.steps + 2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for e in E:
            e["lset"].copy_(e["h_lset"], non_blocking=True)
        gpu.launch()
        for e in E:
            e["h_out"]["counts"].copy_(e["out"]["counts"], non_blocking=True)
        stream.synchronize()
        for e in E:
            r, z = int(e["h_out"]["counts"][0]), int(e["h_out"]["counts"][1])
            h, o = e["h_out"], e["out"]
            h["row_dof"][:r].copy_(o["row_dof"][:r], non_blocking=True)
            h["rowptr"][: r + 1].copy_(o["rowptr"][: r + 1], non_blocking=True)
            h["cols"][:z].copy_(o["cols"][:z], non_blocking=True)
            h["vals"][:z].copy_(o["vals"][:z], non_blocking=True)
        stream.synchronize()
        if k >= 2:
            e2e_times.append(time.perf_counter() - t0)
    gpu.check_forms()
    e2e_serial_s = float(np.mean(e2e_times))
    h2d = sum(e["lset"].numel() * 8 for e in E)
    d2h = sum(16 + e["nrows"] * 4 + (e["nrows"] + 1) * 8 + e["nnz"] * 12 for e in E)

    # pipelined: two output sets and two graphs; the read-back of step k runs
    # on a copy stream while step k + 1 computes into the other set (every
    # step still copies its level set in and its whole matrix out)
    e2e_pipe_s = None
    try:
        for e in E:
            e["out2"] = gpu.out(int(e["out"]["csr"].cap_rows), int(e["out"]["csr"].cap_nnz))
            e["h_out2"] = {k: torch.empty_like(v).pin_memory() for k, v in e["h_out"].items()}
        g2 = gpu.graph_on("out2")
    except (RuntimeError, torch.cuda.OutOfMemoryError):
        g2 = None
    if g2 is not None:
        cs = torch.cuda.Stream()
        done = [torch.cuda.Event(), torch.cuda.Event()]
        freed = [torch.cuda.Event(), torch.cuda.Event()]
        for ev in freed:
            ev.record(stream)
        keys = (("out", "h_out"), ("out2", "h_out2"))

        def issue_copy(k):
            """Host waits for step k's counts, then queues its read-back on the
            copy stream after the step's graph."""
            b = k % 2
            done[b].synchronize()
            with torch.cuda.stream(cs):
                cs.wait_event(done[b])
                for e in E:
                    o, h = e[keys[b][0]], e[keys[b][1]]
                    r, z = int(h["counts"][0]), int(h["counts"][1])
                    h["row_dof"][:r].copy_(o["row_dof"][:r], non_blocking=True)
                    h["rowptr"][: r + 1].copy_(o["rowptr"][: r + 1], non_blocking=True)
                    h["cols"][:z].copy_(o["cols"][:z], non_blocking=True)
                    h["vals"][:z].copy_(o["vals"][:z], non_blocking=True)
                freed[b].record(cs)

        nsteps, warm = args.steps, 2
        for k in range(nsteps + warm):
            if k == warm:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
            b = k % 2
            stream.wait_event(freed[b])  # the read-back of step k - 2 left this output set
            for e in E:
                e["lset"].copy_(e["h_lset"], non_blocking=True)
            _lib.call("xg_step_graph_launch", gpu.g if b == 0 else g2, gpu.sp)
            for e in E:
                e[keys[b][1]]["counts"].copy_(e[keys[b][0]]["counts"], non_blocking=True)
            done[b].record(stream)
            if k > 0:
                issue_copy(k - 1)
        issue_copy(nsteps + warm - 1)
        torch.cuda.synchronize()
        e2e_pipe_s = (time.perf_counter() - t0) / nsteps
        gpu.check_forms()
        # the last step's copy equals the serial read-back's size
        for e in E:
            b = (nsteps + warm - 1) % 2
            assert int(e[keys[b][1]]["counts"][1]) == e["nnz"]
        _lib.load().xg_step_graph_destroy(g2)
        for e in E:
            e.pop("out2", None)
            e.pop("h_out2", None)
    e2e_s = e2e_pipe_s if e2e_pipe_s is not None else e2e_serial_s

    # ---------------- the mixed arm on the same workload ----------------
    fp64_out = [fetch_csr(gpu, e) for e in E] if rank == 0 else None
    # the timed forms are released first: the largest workloads do not fit twice
    for f in {e["form"].value for e in E}:
        _lib.load().xg_form_destroy(ctypes.c_void_p(f))
    _lib.load().xg_step_graph_destroy(gpu.g)
    for e in E:
        for k in ("out", "lset", "h_out", "h_lset"):
            e.pop(k, None)
    gpu.keep.clear()
    torch.cuda.empty_cache()
    mixed = None
    if args.precision == "fp64" and args.mixed:
        a2 = argparse.Namespace(**vars(args))
        a2.precision = "mixed"
        gm = Gpu(a2)
        setup(a2, gm)
        if args.autotune:
            gm.autotune()
        gm.graph()
        if ws > 1:
            torch.distributed.barrier()
        ms_m = time_graph(gm, args.steps, args.warmup, flush)
        if ws > 1:
            t = torch.tensor([ms_m], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms_m = float(t.item())
        mixed = {"value": ws * n_cut / (ms_m * 1e-3), "unit": UNIT, "ms_per_step": ms_m, "speedup_vs_fp64": ms / ms_m,
                 "dtype": "f32 contractions (compensated), f64 geometry and sums"}
        if rank == 0:
            res = [max_rel_err(fetch_csr(gm, e), ref) for e, ref in zip(gm.entries, fp64_out)]
            mixed["same_pattern_as_fp64"] = all(r[0] for r in res)
            mixed["max_rel_err_vs_fp64"] = max((r[1] for r in res if r[1] is not None), default=None)
            mixed["err_definition"] = "max |A_mixed - A_fp64| / max |A_fp64| over all entries of the step's matrices"
        for f in {e["form"].value for e in gm.entries}:
            _lib.load().xg_form_destroy(ctypes.c_void_p(f))
        _lib.load().xg_step_graph_destroy(gm.g)
        del gm

    # ---------------- error of this arm against the oracle ----------------
    check = None
    if rank == 0 and args.check:
        nth = os.cpu_count() or 1
        t0 = time.perf_counter()
        res = [max_rel_err(got, oracle_csr(e, nth)) for e, got in zip(E, fp64_out)]
        check = {"same_pattern": all(r[0] for r in res),
                 "max_rel_err": max((r[1] for r in res if r[1] is not None), default=None),
                 "against": "oracle (C++ restatement of the reference path, FP64), whole workload",
                 "definition": "max |A_gpu - A_oracle| / max |A_oracle| over all entries of each step's matrix",
                 "host_s": time.perf_counter() - t0}

    # ---------------- roofline ----------------
    # algorithmic bytes per stage: vertex ids, coordinates + level set per vertex,
    # dof ids and the element matrix written once (element kernels), the same
    # for both elements of a patch, and the CSR write (scatter)
    alg = dict.fromkeys(names, 0.0)
    for e in E:
        D, nd, ne = e["dim"], e["ndof_el"], e["ne"]
        b_el = 4 * (D + 1) + 8 * (D + 1) * (D + 1) + 4 * nd + 8 * nd * nd
        b_fa = 4 * 2 * (D + 1) + 8 * 2 * (D + 1) * (D + 1) + 4 * 2 * nd + 8 * (2 * nd) ** 2
        alg["marking"] += ne * (4 * (D + 1) + 8 * (D + 1) + 1 + 8)
        alg["lists"] += ne / 8 * 3
        alg["elmat_uncut"] += e["n_neg"] * b_el
        alg["elmat_cut"] += e["n_if"] * b_el
        alg["patch"] += e["n_facets"] * b_fa
        alg["pattern"] += e["nnz"] * 4 + e["nrows"] * 8
        alg["scatter"] += e["nnz"] * 12 + (e["n_neg"] + e["n_if"]) * nd * nd * 8 + e["n_facets"] * (2 * nd) ** 2 * 8
    pk = peaks()
    peak_bw = pk["hbm_gbs"] if pk else 6800.0
    if args.workload == "c5":  # the space-time element kernel covers uncut and cut elements in one launch
        stage_ms[3] += stage_ms[2]
        stage_ms[2] = 0.0
        alg["elmat_cut"] += alg["elmat_uncut"]
        alg["elmat_uncut"] = 0.0
    dom_i = int(np.argmax(stage_ms))
    dname = names[dom_i]
    achieved = alg[dname] / (stage_ms[dom_i] * 1e-3) / 1e9
    step_bytes = sum(alg.values())
    # the FP64 element kernels run on the FP64 pipe.  Patch stage of a spatial
    # form: FLOPs of the basis-change kernel as executed (patch_exact_flops);
    # space-time patches use the quadrature kernel: the packed upper triangle
    # of the (2n)^2 patch matrix, one FMA = 2 FLOPs per entry and point,
    # 2 x NQ(2k) points per facet
    fp64 = None
    if dname == "patch" and gpu.prec == 0 and args.workload != "dg":
        nq = {(2, 2): 3, (2, 4): 6, (2, 6): 16, (3, 2): 4, (3, 4): 14, (3, 6): 64}
        flops = 0.0
        for e in E:
            k = e["order"]
            if e["st"]:
                nd = e["ndof_el"] // 2  # patches are spatial (P1 x P1 in time)
                flops += e["n_facets"] * 2 * nq[(e["dim"], 2 * k)] * 2 * (2 * nd) * (2 * nd + 1) / 2
            else:
                flops += e["n_facets"] * patch_exact_flops(e["dim"], k)
        peak_fp64 = fp64_peak(torch)
        ach = flops / (stage_ms[dom_i] * 1e-3) / 1e12
        fp64 = {"bound": "fp64", "kernel": dname, "achieved": ach, "peak": peak_fp64, "unit": "TFLOP/s",
                "frac": ach / peak_fp64, "flops_per_step": flops,
                "peak_source": "measured here: cuBLAS DGEMM 4096^3 (torch.matmul float64), best of 3"}
    cfg.update({
        "n_tets_or_tris": int(sum(e["ne"] for e in E)), "n_cut": n_cut, "n_neg_uncut": sum(e["n_neg"] for e in E),
        "n_ghost_facets": sum(e["n_facets"] for e in E), "nrows": sum(e["nrows"] for e in E),
        "nnz": sum(e["nnz"] for e in E), "precision": args.precision, "steps_per_graph": len(E),
        "l2": "flushed between timed steps (512 MB write)", "parallelism": "replicas only",
        "timing": "CUDA graph replay of the whole step, CUDA events on the launching stream"})
    if args.workload in ("c2", "dg"):
        cfg["order"] = args.order
    if args.workload == "dg":
        cfg["facets_note"] = "n_ghost_facets counts the ghost facets joined with the (HASNEG, HASNEG) skeleton facets"
        cfg["space"] = "L2 (element-local dofs)"
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if gpu.prec == 0 else "f32+f64", "data": "synthetic", "config": cfg,
        "e2e": {"value": ws * n_cut / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_s * 1e3,
                "mode": "pipelined: two output sets, the read-back of step k on a copy stream overlaps step k + 1"
                if e2e_pipe_s is not None else "serial",
                "serial": {"value": ws * n_cut / e2e_serial_s, "ms_per_step": e2e_serial_s * 1e3,
                           "mode": "copy in, step, counts, copy out, synchronise; one step at a time"}},
        "stages_ms": {n: float(v) for n, v in zip(names, stage_ms)},
        "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak_bw, "unit": "GB/s",
                     "frac": achieved / peak_bw, "traffic": traffic_for(args.workload, dname) if
                     (args.workload, args.n, args.order) == ("c2", 64, 2) or args.workload != "c2" else None,
                     "peak_source": "measured" if pk else "fallback",
                     "whole_step": {"achieved": step_bytes / (ms * 1e-3) / 1e9,
                                    "frac": step_bytes / (ms * 1e-3) / 1e9 / peak_bw}},
        "clocks": clk.summary(),
        "gpu_launches": args.steps * gpu.kernels,
    }
    if check is not None:
        out["max_rel_err"] = check["max_rel_err"]
        out["error_check"] = check
    if mixed is not None:
        out["mixed"] = mixed
    if fp64 is not None:  # the bound that binds for the dominant kernel
        fp64["traffic"] = out["roofline"]["traffic"]
        fp64["hbm"] = out["roofline"]
        out["roofline"] = fp64
    if rank == 0 and args.cpu_baseline:
        try:
            nth = os.cpu_count() or 1
            C5_KT[0] = args.kt
            jobs, desc = cpu_prepare(args, args.workload in ("c3", "c5"))
            cpu_pass(jobs, nth)  # warm-up
            reps = 2
            t_cpu, n_cpu = 0.0, 0
            for _ in range(reps):
                t, nc = cpu_pass(jobs, nth)
                t_cpu += t
                n_cpu += nc
            out["cpu_baseline"] = {"value": n_cpu / t_cpu, "unit": UNIT, "cores": nth, "kind": "port",
                                   "sample": "%s, %d timed pass(es)" % (desc, reps)}
        except Exception as ex:  # the baseline is reported, never required
            out["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": repr(ex)}
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

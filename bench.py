"""Benchmark of the cut-element assembly step on one GB300.

Workload (the 3D CutFEM Poisson configuration): unit cube, 64^3 cubes x 6
Kuhn tetrahedra (1,572,864 tets), level set
phi = |x - 0.5| - 0.3 + 0.02 sin(7x) sin(7y) sin(7z) interpolated to P1 (with
InterpolateToP1's +1e-14 perturbation), P2 H1 space, NEG-domain stiffness,
Nitsche interface terms (lambda = 10 k^2 = 40, scaled by 1/h) on IF and ghost
penalty 0.1/h^2 (u - u')(v - v') on the facets between HASNEG and IF
elements.  Synthetic, seeded data (the reference publishes no dataset).

One step = CutInfo marking + ghost-facet marking + cut rules + element and
facet-patch matrices + the deterministic scatter into a compressed-row
matrix (xg_cutfem_step).  metric = cut (IF) elements per second.

    python bench.py [--steps K] [--warmup W] [--precision fp64|mixed] [--impl xg|reference]
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cut elems/s, rule+assembly, 1 GB300: plain FP64 vs learned/mixed at equal error"
UNIT = "cut_elems/s"


def workload(n):
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


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except (OSError, ValueError):
        return None


def run_reference(args):
    """The reference arm: the CPU statement of the path (the reference itself
    needs NGSolve and cannot be built), all host threads, same workload."""
    ws, rank = dist_env()
    if rank != 0:
        return
    from oracle import oracle as orc
    m, vals = workload(args.n)
    l = orc.interpolate_p1_perturb(vals)
    sp = orc.Space(m, args.order)
    nth = os.cpu_count() or 1
    dom, _, _ = sp.cutinfo(l, nth)
    n_if = int((dom == 2).sum())
    for _ in range(args.warmup):
        sp.pipeline(l, terms_c2(args.order), True, nth)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        sp.pipeline(l, terms_c2(args.order), True, nth)
        times.append(time.perf_counter() - t0)
    t = float(np.mean(times))
    value = n_if / t
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "3D CutFEM Poisson, 64^3x6 Kuhn tets, P2, NEG stiffness + Nitsche IF + ghost penalty",
                   "n_tets": int(m.ne), "n_cut": n_if, "order": args.order},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nth, "kind": "port",
                         "sample": "full workload per step (oracle C++ restatement of ngsxfem's path; the reference "
                                   "needs NGSolve, which cannot be built here)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="xg", choices=["xg", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--n", type=int, default=64)
    ap.add_argument("--order", type=int, default=2)
    ap.add_argument("--cpu-baseline", type=int, default=1)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    args.warmup = max(args.warmup, 3)

    import torch
    ws, rank = dist_env()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    from ngsxfem_gb300 import build as xbuild
    xbuild.build()
    from ngsxfem_gb300 import _lib
    from ngsxfem_gb300 import xfem as xg

    m, vals = workload(args.n)
    gf = xg.GridFunction(xg.H1(m, 1))
    xg.InterpolateToP1(vals, gf)
    V = xg.H1(m, order=args.order)
    terms = terms_c2(args.order)
    arr = (_lib.Term * len(terms))()
    for k, t in enumerate(terms):
        arr[k].kind, arr[k].domain, arr[k].order = t["kind"], t["domain"], -1
        arr[k].hpow, arr[k].coef = t["hpow"], t["coef"]
        arr[k].d_defined_on = None
    prec = 0 if args.precision == "fp64" else 1
    form = ctypes.c_void_p()
    _lib.call("xg_form_create", V.h, arr, len(terms), prec, ctypes.byref(form))
    cap = np.zeros(2, dtype=np.int64)
    _lib.call("xg_form_capacity", form, cap.ctypes.data_as(ctypes.c_void_p))
    bf = xg.BilinearForm(V)
    bf._alloc(int(cap[0]), int(cap[1]))
    stream = torch.cuda.current_stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    lset = gf.vec

    # stage events (profiling hook, recorded on the launching stream)
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(8)]
    for e in evs:  # torch creates the CUDA event on first record
        e.record(stream)
    torch.cuda.synchronize()
    ev_arr = (ctypes.c_void_p * 8)(*[ctypes.c_void_p(e.cuda_event) for e in evs])

    def step():
        _lib.call("xg_cutfem_step", form, ctypes.c_void_p(lset.data_ptr()), ctypes.byref(bf._csr), sp)

    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # > L2 (129 MB)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    _lib.check(_lib.load().xg_form_check(form), "bench form")
    nrows, nnz = (int(x) for x in bf._counts.cpu().tolist())
    # counts of the workload
    dom_p = ctypes.c_void_p()
    _lib.call("xg_cutfem_marking", form, ctypes.byref(dom_p), None, None, None)
    ci = xg.CutInfo(m, gf)
    dom = ci.dom.cpu().numpy()
    n_if = int((dom == 2).sum())
    n_neg = int((dom == 0).sum())
    hasneg, hasif = ci.GetElementsOfType(xg.HASNEG), ci.GetElementsOfType(xg.IF)
    n_facets = xg.GetFacetsWithNeighborTypes(m, a=hasneg, b=hasif).NumSet()

    # ---------------- device-resident timing ----------------
    _lib.call("xg_form_stage_events", form, ev_arr, 8)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    stage_ms = np.zeros(7)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for k in range(args.steps):
            flush.fill_(float(k))  # L2 flush between timed steps (not timed)
            starts[k].record(stream)
            step()
            ends[k].record(stream)
            ends[k].synchronize()
            stage_ms += np.array([evs[i].elapsed_time(evs[i + 1]) for i in range(7)])
    torch.cuda.synchronize()
    _lib.call("xg_form_stage_events", form, None, 0)
    ms = float(np.mean([s.elapsed_time(e) for s, e in zip(starts, ends)]))
    if ws > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    stage_ms /= args.steps
    _lib.check(_lib.load().xg_form_check(form), "bench form")
    value = ws * n_if / (ms * 1e-3)

    # ---------------- end to end through the C ABI with host buffers ----------------
    h_lset = torch.empty_like(lset, device="cpu").pin_memory()
    h_lset.copy_(lset.cpu())
    h_rowdof = torch.empty(nrows, dtype=torch.int32).pin_memory()
    h_rowptr = torch.empty(nrows + 1, dtype=torch.int64).pin_memory()
    h_cols = torch.empty(nnz, dtype=torch.int32).pin_memory()
    h_vals = torch.empty(nnz, dtype=torch.float64).pin_memory()
    h_counts = torch.empty(2, dtype=torch.int64).pin_memory()
    d_lset = torch.empty_like(lset)
    e2e_times = []
    for k in range(args.steps + 2):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d_lset.copy_(h_lset, non_blocking=True)
        _lib.call("xg_cutfem_step", form, ctypes.c_void_p(d_lset.data_ptr()), ctypes.byref(bf._csr), sp)
        h_counts.copy_(bf._counts, non_blocking=True)
        stream.synchronize()
        r, z = int(h_counts[0]), int(h_counts[1])
        h_rowdof[:r].copy_(bf._row_dof[:r], non_blocking=True)
        h_rowptr[: r + 1].copy_(bf._rowptr[: r + 1], non_blocking=True)
        h_cols[:z].copy_(bf._cols[:z], non_blocking=True)
        h_vals[:z].copy_(bf._vals[:z], non_blocking=True)
        stream.synchronize()
        if k >= 2:
            e2e_times.append(time.perf_counter() - t0)
    e2e_s = float(np.mean(e2e_times))
    h2d = lset.numel() * 8
    d2h = 16 + nrows * 4 + (nrows + 1) * 8 + nnz * 12

    # ---------------- roofline of the dominant stage ----------------
    names = ["marking", "lists", "elmat_uncut", "elmat_cut", "patch", "pattern", "scatter"]
    dom_i = int(np.argmax(stage_ms))
    D, nd = 3, V.ndof_el
    b_el = 4 * (D + 1) + 8 * (D + 1) * (D + 1) + 4 * nd + 8 * nd * nd
    b_fa = 4 * 2 * (D + 1) + 8 * 2 * (D + 1) * (D + 1) + 4 * 2 * nd + 8 * (2 * nd) ** 2
    n_uncut_active = n_neg
    alg = {
        "marking": m.ne * (4 * (D + 1) + 8 * (D + 1) + 1 + 8),
        "lists": m.ne / 8 * 3,
        "elmat_uncut": n_uncut_active * b_el,
        "elmat_cut": n_if * b_el,
        "patch": n_facets * b_fa,
        "pattern": nnz * 4 + nrows * 8,
        "scatter": nnz * 12 + (n_uncut_active + n_if) * nd * nd * 8 + n_facets * (2 * nd) ** 2 * 8,
    }
    pk = peaks()
    peak_bw = pk["hbm_gbs"] if pk else 6800.0
    dname = names[dom_i]
    achieved = alg[dname] / (stage_ms[dom_i] * 1e-3) / 1e9
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == 0 else "f32+f64", "data": "synthetic",
        "config": {"workload": "3D CutFEM Poisson, %d^3x6 Kuhn tets, P%d, NEG stiffness + Nitsche IF + ghost "
                               "penalty 0.1/h^2" % (args.n, args.order),
                   "n_tets": int(m.ne), "n_cut": n_if, "n_neg_uncut": n_neg, "n_ghost_facets": n_facets,
                   "nrows": nrows, "nnz": nnz, "precision": args.precision,
                   "l2": "flushed between timed steps (512 MB write)", "parallelism": "replicas only"},
        "e2e": {"value": ws * n_if / e2e_s, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "ms_per_step": e2e_s * 1e3},
        "stages_ms": {n: float(v) for n, v in zip(names, stage_ms)},
        "roofline": {"bound": "hbm", "kernel": dname, "achieved": achieved, "peak": peak_bw, "unit": "GB/s",
                     "frac": achieved / peak_bw, "traffic": None,
                     "peak_source": "measured" if pk else "fallback"},
        "clocks": clk.summary(),
        "gpu_launches": None,
    }
    # kernel launches per step: cutinfo 1, facets 1, active 2, compactions 3x4, elmat 2, patch 1,
    # dof mark 1 (+memset), rowcount 1, scan 3, rowfill 1
    out["gpu_launches"] = args.steps * 25
    if rank == 0 and args.cpu_baseline:
        try:
            from oracle import oracle as orc
            l = orc.interpolate_p1_perturb(vals)
            spc = orc.Space(m, args.order)
            nth = os.cpu_count() or 1
            spc.pipeline(l, terms, True, nth)
            t0 = time.perf_counter()
            reps = 2
            for _ in range(reps):
                spc.pipeline(l, terms, True, nth)
            tc = (time.perf_counter() - t0) / reps
            out["cpu_baseline"] = {"value": n_if / tc, "unit": UNIT, "cores": nth, "kind": "port",
                                   "sample": "full workload, mean of 2 pipeline runs after 1 warm-up"}
        except Exception as e:  # the baseline is reported, never required
            out["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": 0, "kind": "port", "sample": repr(e)}
    _lib.load().xg_form_destroy(form)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

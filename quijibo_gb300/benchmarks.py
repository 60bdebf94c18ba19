"""Measurements of the mesher, the energies and the server (beside bench.py,
which measures the headline field).  Each prints one JSON object.

    python -m quijibo_gb300.benchmarks mesh   [--res 512] [--workload precision|large]
    python -m quijibo_gb300.benchmarks energy [--samples 200000] [--steps 50]
    python -m quijibo_gb300.benchmarks serve  [--requests 400] [--scale 0.25]
    python -m quijibo_gb300.benchmarks large  [--res 2200] [--slab 64] [--check-slices 4]
    python -m quijibo_gb300.benchmarks classify [--res 2200] [--slab 64] [--reps 5]
    python -m quijibo_gb300.benchmarks lagrange [--res 256]

All inputs are synthetic (quijibo_gb300/rootsets.py, samples.py).
"""
import argparse
import json
import statistics
import time

import numpy as np


def hbm_peak_gbs():
    """(GB/s, source): the measured copy bandwidth of MEASURED_PEAKS.json at
    the repository root, else the pool's earlier GB300 measurement."""
    import os
    path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                        "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback (earlier GB300 copy measurement)"


def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def bench_mesh(args):
    """Streaming mesher (field slab + classify/scan/emit + FP64 bisection) on
    the precision or large workload; reports triangles/s and the time split."""
    import torch

    from . import lib
    from .rootsets import large_workload, precision_workload
    ctx = lib.Context(0)
    wl = precision_workload if args.workload == "precision" else large_workload
    args.res = args.res or 512
    rs, g, p = wl(args.res)
    h = ctx.upload(rs)
    it = ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP32_REFINE,
                         refine_pow=lib.QJG_REFINE_INT)
    # capacities from a coarse pass scale with the surface (about res^2)
    vcap = int(args.vert_cap or 12 * g.res[0] * g.res[1])
    tcap = int(args.tri_cap or 24 * g.res[0] * g.res[1])
    v32 = torch.empty(3 * vcap, dtype=torch.float32, device="cuda")
    tris = torch.empty(3 * tcap, dtype=torch.int32, device="cuda")
    kw = dict(d_verts32=v32.data_ptr(), vert_cap=vcap, d_tris=tris.data_ptr(), tri_cap=tcap,
              slab_nz=args.slab)
    rc, st = ctx.mesh_stream(h, g, it, check=False, **kw)  # warm-up, and sizes
    if rc == -5:
        raise SystemExit("raise --vert-cap/--tri-cap: needs %d / %d" % (st["n_verts"], st["n_tris"]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _, st = ctx.mesh_stream(h, g, it, **kw)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    # the field alone over the same grid, for the split
    f = torch.empty(g.res[0] * g.res[1] * min(g.res[2], args.slab + 1), dtype=torch.float64,
                    device="cuda")
    ctx.set_timing(True)
    field_ms = 0.0
    for z0 in range(0, g.res[2], args.slab + 1):
        z1 = min(z0 + args.slab + 1, g.res[2])
        ctx.field(h, g, it, f.data_ptr(), z0=z0, z1=z1)
        b, r = ctx.last_timings()
        field_ms += b + r
    return {"workload": "%s %d^3" % (args.workload, args.res), "voxels": g.n_voxels,
            "triangles": st["n_tris"], "vertices": st["n_verts"], "wall_s": wall,
            "triangles_per_s": st["n_tris"] / wall, "gvox_s": g.n_voxels / wall / 1e9,
            "field_only_s": field_ms / 1e3, "mesher_s": wall - field_ms / 1e3,
            "bisection_map_evals_fp64": st["map_evals"],
            "bisection_map_evals_fp32": st["map_evals_fp32"],
            "bisection_map_evals_ff": st["map_evals_ff"], "unbracketed": st["n_unbracketed"],
            "degenerate": st["n_degenerate"], "slabs": st["slabs"],
            "refined": st["field"]["refined"],
            "lane_efficiency": st["field"]["voxel_iters"] / max(1, st["field"]["lane_iters"])}


def bench_classify(args):
    """The mesher's classification alone on one stored slab of the large
    workload: the precision field of 65 planes of the 2200^3 grid (48/24
    roots, 60 iterations) computed once, then meshed repeatedly as a stored
    field with linear edge vertices, so the classify and triangle phases are
    timed without the field and the bisection.  Algorithmic bytes: the FP64
    field read once (8 B per voxel), 12 B per vertex and per triangle."""
    import torch

    from . import lib
    from .rootsets import Grid, large_workload
    ctx = lib.Context(0)
    res = args.res or 2200
    rs, g, p = large_workload(res)
    h = ctx.upload(rs)
    planes = args.slab + 1
    z0 = args.z0 if args.z0 >= 0 else res // 2
    XY = g.res[0] * g.res[1]
    f = torch.empty(planes * XY, dtype=torch.float64, device="cuda")
    it = ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP32_REFINE,
                         refine_pow=lib.QJG_REFINE_INT, rel_tol=args.rel_tol)
    ctx.field(h, g, it, f.data_ptr(), z0=z0, z1=z0 + planes)
    torch.cuda.synchronize()
    slab = Grid((g.res[0], g.res[1], planes), lengths=(g.lengths[0], g.lengths[1],
                                                      g.lengths[2] * planes / res))
    vcap, tcap = 8 * XY, 16 * XY
    v32 = torch.empty(3 * vcap, dtype=torch.float32, device="cuda")
    tris = torch.empty(3 * tcap, dtype=torch.int32, device="cuda")
    ctx.set_timing(True)
    runs = []
    for k in range(args.reps + 1):
        _, st = ctx.mesh_field(None, slab, None, f.data_ptr(), lib.QJG_EDGE_LINEAR,
                               d_verts32=v32.data_ptr(), vert_cap=vcap, d_tris=tris.data_ptr(),
                               tri_cap=tcap, slab_nz=args.slab)
        if k:
            runs.append(st)
    n = slab.n_voxels
    cls = statistics.median(r["ms_classify"] for r in runs)
    tri = statistics.median(r["ms_triangles"] for r in runs)
    st = runs[-1]
    alg = mesh_algorithmic_bytes(n, st["n_verts"], st["n_tris"] + st["n_degenerate"])
    out = {"workload": "large workload, planes [%d, %d) of the %d^3 grid as one stored slab"
                       % (z0, z0 + planes, res),
           "voxels": n, "vertices": st["n_verts"], "triangles": st["n_tris"],
           "ms_classify": cls, "ms_triangles": tri, "ms_vertices": st["ms_vertices"],
           "algorithmic_bytes": alg, "gb_s": alg / ((cls + tri) * 1e-3) / 1e9,
           "frac_hbm": alg / ((cls + tri) * 1e-3) / 1e9 / args.hbm_gbs, "hbm_peak_gb_s": args.hbm_gbs}
    ctx.free(h)
    ctx.close()
    return out


def bench_mesh_fixed(args):
    """The streaming mesher three ways on the precision workload at small
    grids (a mesh request's sizes): qjg_mesh_stream (host reads between
    slabs), qjg_mesh_stream_async (the fixed launch sequence, one wait) and
    that sequence replayed from a captured CUDA graph; wall-clock ms per mesh
    (median of --reps), same mesh each way."""
    import torch

    from . import lib
    from .rootsets import precision_workload
    ctx = lib.Context(0)
    out = {"workload": "precision workload map, FP32 + double-float + FP64 band, rel_tol 1e-6"}
    for res in (64, 128, 256):
        rs, g, p = precision_workload(res)
        h = ctx.upload(rs)
        it = ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP32_REFINE,
                             refine_pow=lib.QJG_REFINE_INT, rel_tol=1e-6)
        vcap, tcap = 12 * res * res + 4096, 24 * res * res + 4096
        v64 = torch.empty(3 * vcap, dtype=torch.float64, device="cuda")
        tris = torch.empty(3 * tcap, dtype=torch.int32, device="cuda")
        kw = dict(d_verts64=v64.data_ptr(), vert_cap=vcap, d_tris=tris.data_ptr(), tri_cap=tcap)
        s = torch.cuda.Stream()
        ctx.mesh_prepare(g, vcap, tcap)

        def timed(fn):
            fn()
            torch.cuda.synchronize()
            ts = []
            for _ in range(args.reps):
                t0 = time.perf_counter()
                fn()
                torch.cuda.synchronize()
                ts.append(1e3 * (time.perf_counter() - t0))
            return float(np.median(ts))

        def host():
            ctx.mesh_stream(h, g, it, stream=s.cuda_stream, **kw)

        def fixed():
            ctx.mesh_stream_async(h, g, it, stream=s.cuda_stream, **kw)
            s.synchronize()

        r = {"host_ms": timed(host)}
        _, st_h = ctx.mesh_stream(h, g, it, stream=s.cuda_stream, **kw)
        r["fixed_ms"] = timed(fixed)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=s, capture_error_mode="thread_local"):
            ctx.mesh_stream_async(h, g, it, stream=s.cuda_stream, **kw)
        r["graph_ms"] = timed(graph.replay)
        _, st = ctx.mesh_async_result()
        r.update(triangles=st["n_tris"], same_counts=st["n_tris"] == st_h["n_tris"] and
                 st["n_verts"] == st_h["n_verts"], slabs=st["slabs"])
        out["%d^3" % res] = r
        ctx.free(h)
    return out


def bench_lagrange(args):
    """The Lagrange order of the map (RATIONAL_4D::evaluateLagrange, the
    lagrangeBunny3D driver's) on the precision workload's map (16 top / 8
    bottom roots, 40 iterations, escape 2) at res^3: the plain FP64 form
    against the precision form (FP32 bulk, double-float re-run at rel_tol,
    FP64 band): time, sign map, error."""
    import torch

    from . import lib
    from .rootsets import precision_workload
    ctx = lib.Context(0)
    res = args.res or 256
    rs, g, p = precision_workload(res)
    h = ctx.upload(rs)
    n = g.n_voxels
    a = torch.empty(n, dtype=torch.float64, device="cuda")
    b = torch.empty(n, dtype=torch.float64, device="cuda")
    forms = {"fp64": ctx.iter_params(p["max_it"], p["escape"], refine_pow=lib.QJG_REFINE_INT,
                                     lagrange=True),
             "fp32_refine": ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP32_REFINE,
                                            refine_pow=lib.QJG_REFINE_INT, rel_tol=args.rel_tol,
                                            lagrange=True)}
    out = {"workload": "Lagrange order, precision workload map, %d^3, 40 iterations" % res,
           "voxels": n, "rel_tol": args.rel_tol}
    for name, it in forms.items():
        buf = a if name == "fp64" else b
        ctx.field(h, g, it, buf.data_ptr())  # warm
        torch.cuda.synchronize()
        e0, e1 = _events(torch)
        e0.record()
        ctx.field(h, g, it, buf.data_ptr())
        e1.record()
        e1.synchronize()
        ms = e0.elapsed_time(e1)
        out[name] = {"ms": ms, "gvox_s": n / (ms * 1e-3) / 1e9, "stats": ctx.stats()}
    rel = (b - a).abs() / a.abs().clamp_min(1e-300)
    out["sign_map_disagreements"] = int(((a > 0) != (b > 0)).sum().item())
    out["max_rel_err"] = float(rel.max().item())
    out["speedup"] = out["fp64"]["ms"] / out["fp32_refine"]["ms"]
    ctx.free(h)
    ctx.close()
    return out


def bench_energy(args):
    """Differentiation workload: 64 top / 16 bottom roots, Poisson-disk
    samples, 30 iterations; FP32 forward, FP32 recompute adjoint, device
    L-BFGS."""
    import torch

    from . import lib
    from .samples import differentiation_workload
    ctx = lib.Context(0)
    rs, xyz, t, p = differentiation_workload(args.samples)
    P = torch.from_numpy(lib.params_of(rs)).cuda()
    X = torch.from_numpy(xyz).cuda()
    T = torch.from_numpy(t).cuda()
    G = torch.empty_like(P)
    n = len(t)
    out = {"samples": n, "params": int(P.numel()), "max_it": p["max_it"]}
    from .roofline import energy_flops
    peak = lib.fma_probe(0)
    forms = (("forward_fp32", lib.QJG_FP32, False), ("adjoint_fp32", lib.QJG_FP32, True),
             ("forward_fp64", lib.QJG_FP64, False), ("adjoint_fp64", lib.QJG_FP64, True))
    if args.energy_pairs:
        lib.set_energy_pairs(True)
        out["forward_kernel"] = "two samples per lane"
    lib.set_energy_fast(not args.energy_accurate)
    out["polar_power"] = ("accurate device functions" if args.energy_accurate else
                          "fast: hardware log2 and sin/cos, polynomial atan")
    if getattr(args, "sweep_blocks", ""):
        # forward and forward + adjoint calls per forward block count: median
        # of 7 FP32 calls after one warm-up call (wall clock, ms)
        sweep = {}
        fargs = (P.data_ptr(), rs.n_top, rs.n_bottom, n, X.data_ptr(), T.data_ptr(), p["max_it"],
                 p["escape"])
        try:
            for per_sm in [int(v) for v in args.sweep_blocks.split(",")]:
                lib.set_energy_forward_blocks(per_sm)
                row = {}
                for name, g in (("forward_ms", 0), ("gradient_ms", G.data_ptr())):
                    ctx.energy(*fargs, precision=lib.QJG_FP32, d_grad=g)
                    torch.cuda.synchronize()
                    ts = []
                    for _ in range(7):
                        t0 = time.perf_counter()
                        e = ctx.energy(*fargs, precision=lib.QJG_FP32, d_grad=g)
                        ts.append(time.perf_counter() - t0)
                    row[name] = sorted(ts)[3] * 1e3
                    row["energy"] = e
                sweep[per_sm] = row
        finally:
            lib.set_energy_forward_blocks(0)
        out["forward_blocks_sweep"] = sweep
        return out
    for name, prec, grad in forms[:2] if args.fp32_only else forms:
        kw = dict(precision=prec, d_grad=G.data_ptr() if grad else 0)
        ctx.energy(P.data_ptr(), rs.n_top, rs.n_bottom, n, X.data_ptr(), T.data_ptr(), p["max_it"],
                   p["escape"], **kw)
        torch.cuda.synchronize()
        reps = 3
        t0 = time.perf_counter()
        for _ in range(reps):
            e = ctx.energy(P.data_ptr(), rs.n_top, rs.n_bottom, n, X.data_ptr(), T.data_ptr(),
                           p["max_it"], p["escape"], **kw)
        dt = (time.perf_counter() - t0) / reps
        out[name] = {"s": dt, "samples_per_s": n / dt, "energy": e}
        # algorithmic work of the call (counted on the device) against the
        # FP32 FMA probe: per-call wall time, so a lower bound of the kernels'
        apps, steps = ctx.energy_last_work()
        fl, sp = energy_flops(rs.n_top, rs.n_bottom, apps, steps)
        out[name].update({"map_applications": apps, "adjoint_steps": steps,
                          "root_terms": apps * (rs.n_top + rs.n_bottom), "flops": fl,
                          "special_ops": sp, "tflops": fl / dt / 1e12})
        if prec == lib.QJG_FP32:
            out[name]["frac_fma_probe"] = fl / dt / 1e12 / peak
    out["fma_probe_tflops"] = peak
    out["gradients_per_s"] = 1.0 / out["adjoint_fp32"]["s"]
    # the FP32 adjoint with one lane per sample walking the roots, for comparison
    lib.set_energy_adjoint_roots(False)
    try:
        kw = dict(precision=lib.QJG_FP32, d_grad=G.data_ptr())
        args_e = (P.data_ptr(), rs.n_top, rs.n_bottom, n, X.data_ptr(), T.data_ptr(), p["max_it"],
                  p["escape"])
        ctx.energy(*args_e, **kw)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            ctx.energy(*args_e, **kw)
        out["adjoint_fp32_one_lane"] = {"s": (time.perf_counter() - t0) / 3}
    finally:
        lib.set_energy_adjoint_roots(True)
    if args.steps <= 0:
        return out
    Pfit = P.clone()
    t0 = time.perf_counter()
    en, st = ctx.fit_lbfgs(Pfit.data_ptr(), rs.n_top, rs.n_bottom, n, X.data_ptr(), T.data_ptr(),
                           p["max_it"], p["escape"], steps=args.steps, precision=lib.QJG_FP32)
    out["lbfgs"] = dict(st, wall_s=time.perf_counter() - t0,
                        energies=[float(v) for v in en[:: max(1, len(en) // 10)]])
    return out


def bench_energy_batch(args):
    """One qjg_energy_backward_batch pass over 8 FP32 energy + gradient calls
    (25k Poisson-disk samples each, 64/16, 32/8, 16/4 and 48/12 roots, 30
    iterations): median of 5 batch calls with the adjoint's roots over
    16-lane groups and with one lane per sample, and how far apart the two
    forms' gradients are."""
    import torch

    from . import lib
    from .rootsets import Grid, conformal_scale, draw_rootset
    from .samples import ShapeSDF, poisson_disk
    ctx = lib.Context(0)
    items = []
    for j in range(8):
        nt, nb = [(64, 16), (32, 8), (16, 4), (48, 12)][j % 4]
        rs = draw_rootset(40 + j, nt, nb, -1.2, 1.2, exps=(1, 2))
        rs.scale = conformal_scale(rs, Grid((16, 16, 16), lengths=(2.0, 2.0, 2.0)))
        xyz, _ = poisson_disk(args.batch_samples, seed=j)
        t = ShapeSDF(j)(xyz)
        p = torch.from_numpy(lib.params_of(rs)).cuda()
        X, T = torch.from_numpy(xyz).cuda(), torch.from_numpy(t).cuda()
        g = torch.empty(5 * (nt + nb) + 1, dtype=torch.float64, device="cuda")
        items.append(dict(d_params=p.data_ptr(), n_top=nt, n_bot=nb, n=len(t),
                          d_xyz=X.data_ptr(), d_target=T.data_ptr(), max_it=30, escape=2.0,
                          d_sat=1.0, d_grad=g.data_ptr(), keep=(p, X, T, g)))
    out = {"items": len(items), "samples_per_item": args.batch_samples}
    grads = {}
    try:
        for roots in (False, True):
            lib.set_energy_adjoint_roots(roots)
            ctx.energy_batch(items)
            torch.cuda.synchronize()
            ts = []
            for _ in range(5):
                t0 = time.perf_counter()
                ctx.energy_batch(items)
                ts.append(time.perf_counter() - t0)
            name = "grouped_adjoint_ms" if roots else "one_lane_adjoint_ms"
            out[name] = sorted(ts)[2] * 1e3
            grads[roots] = [it["keep"][3].cpu().numpy().copy() for it in items]
    finally:
        lib.set_energy_adjoint_roots(True)
    out["max_rel_gradient_difference"] = max(
        float(np.linalg.norm(a - b) / np.linalg.norm(a)) for a, b in zip(grads[False], grads[True]))
    return out


def _stream(seed, n, scale):
    """Poisson-arrival mix of field, field+mesh and energy+gradient requests:
    grid sides log-uniform in [32, 512] (field) and [128, 1024] (mesh) times
    `scale`, 10k-200k samples times `scale`, 4-64 roots, 10-60 iterations."""
    from . import lib
    from .rootsets import Grid, conformal_scale, draw_rootset
    from .samples import ShapeSDF, poisson_disk
    rng = np.random.RandomState(seed)
    reqs = []
    # sample sets: two seeded Poisson-disk sets of the largest size, each
    # with its own target shape; a request takes a prefix of one (dart
    # throwing accepts points uniformly over the box, so a prefix is spread
    # over it too)
    big = int(200_000 * scale)
    pools = {}
    for i in range(n):
        kind = rng.choice([lib.QJG_REQ_FIELD, lib.QJG_REQ_MESH, lib.QJG_REQ_ENERGY], p=[0.5, 0.2, 0.3])
        nr = int(rng.randint(4, 65))
        nb = int(rng.randint(0, nr // 3 + 1))
        rs = draw_rootset(1000 + i, nr - nb if nr - nb >= 1 else 1, nb, -1.2, 1.2, exps=(1, 2))
        max_it = int(rng.randint(10, 61))
        if kind == lib.QJG_REQ_ENERGY:
            ns = max(64, int(np.exp(rng.uniform(np.log(10_000), np.log(200_000))) * scale))
            pool = i % 2
            if pool not in pools:
                xyz = poisson_disk(max(big, 64), seed=pool)[0]
                pools[pool] = (xyz, ShapeSDF(pool)(xyz))
            xyz, target = pools[pool][0][:ns], pools[pool][1][:ns]
            rs.scale = conformal_scale(rs, Grid((16, 16, 16), lengths=(2.0, 2.0, 2.0)), 16)
            reqs.append(dict(kind=kind, rs=rs, params=lib.params_of(rs), xyz=xyz,
                             target=target, max_it=max_it, precision=lib.QJG_FP32))
        else:
            lo, hi = (32, 512) if kind == lib.QJG_REQ_FIELD else (128, 1024)
            res = max(8, int(np.exp(rng.uniform(np.log(lo), np.log(hi))) * scale))
            g = Grid((res, res, res))
            rs.scale = conformal_scale(rs, g, 16)
            r = dict(kind=kind, rs=rs, grid=g, max_it=max_it, precision=lib.QJG_FP32_REFINE)
            if kind == lib.QJG_REQ_MESH:
                r.update(vert_cap=24 * res * res + 4096, tri_cap=48 * res * res + 4096)
            reqs.append(r)
    return reqs


def _failures(reqs, results):
    """Requests that did not complete: index, kind, size, status and error."""
    from . import lib
    out = []
    for i, (q, r) in enumerate(zip(reqs, results)):
        if r["status"] != lib.QJG_STATUS_DONE:
            size = q["grid"].res[0] if "grid" in q else len(q["target"])
            out.append({"i": i, "kind": int(q["kind"]), "size": int(size), "roots": q["rs"].n_top +
                        q["rs"].n_bottom, "status": int(r["status"]), "error": int(r["error"])})
    return out


def _retry_capacity(srv, reqs, results):
    """Mesh requests whose mesh outgrew their caps come back failed with
    QJG_ERR_CAPACITY and the counts they need; a client resubmits them with
    those caps.  The retried request's latency is both attempts' (the retry
    runs after the stream).  Returns how many were retried."""
    from . import lib
    idx = [i for i, r in enumerate(results) if r["status"] != lib.QJG_STATUS_DONE and
           r["error"] == lib.QJG_ERR_CAPACITY and reqs[i]["kind"] == lib.QJG_REQ_MESH]
    tickets = []
    for i in idx:
        q = dict(reqs[i])
        q["vert_cap"] = max(q["vert_cap"], int(results[i]["n_verts"]))
        q["tri_cap"] = max(q["tri_cap"], int(results[i]["n_tris"]))
        tickets.append(srv.submit(**q))
    for i, t in zip(idx, tickets):
        r = srv.wait(t)
        r["latency_ms"] += results[i]["latency_ms"]
        results[i] = r
    return len(idx)


def bench_serve(args):
    """Serving: Poisson arrivals into the continuous-batching server vs the
    same requests as plain FP64 launches one after another."""
    from . import lib
    reqs = _stream(args.seed, args.requests, args.scale)
    # offered load: mean gap chosen so the stream arrives over --span seconds
    rng = np.random.RandomState(args.seed + 1)
    gaps = rng.exponential(args.span / len(reqs), size=len(reqs))
    srv = lib.Server(workers=args.workers, hbm_budget=int(args.budget_gb * (1 << 30)))
    # warm the workers' modules
    srv.wait(srv.submit(**reqs[0]))
    t0 = time.perf_counter()
    tickets = []
    for r, gap in zip(reqs, gaps):
        target = time.perf_counter() + gap
        while time.perf_counter() < target:
            pass
        tickets.append(srv.submit(**r))
    results = [srv.wait(t) for t in tickets]
    span = time.perf_counter() - t0
    st = srv.stats()
    retried = _retry_capacity(srv, reqs, results)
    srv.close()
    lat = np.array([r["latency_ms"] for r in results])
    vox = sum(r["grid"].n_voxels for r in reqs if "grid" in r)
    out = {"requests": len(reqs), "scale": args.scale, "workers": args.workers,
           "offered_req_s": len(reqs) / args.span,
           "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
           "max_ms": float(lat.max()), "throughput_req_s": len(reqs) / span,
           "gvox_s": vox / span / 1e9, "span_s": span, "peak_running": st["peak_running"],
           "failed": st["failed"], "batched": st["batched"], "batches": st["batches"],
           "max_batch": st["max_batch"], "energy_batched": st["energy_batched"],
           "energy_batches": st["energy_batches"], "max_energy_batch": st["max_energy_batch"],
           "mesh_batched": st["mesh_batched"], "by_kind": {}, "capacity_retries": retried, "failures": _failures(reqs, results)}
    for kind, name in ((lib.QJG_REQ_FIELD, "field"), (lib.QJG_REQ_MESH, "mesh"),
                       (lib.QJG_REQ_ENERGY, "energy")):
        lk = np.array([r["latency_ms"] for r, q in zip(results, reqs) if q["kind"] == kind])
        if len(lk):
            out["by_kind"][name] = {"n": int(len(lk)), "p50_ms": float(np.percentile(lk, 50)),
                                    "p99_ms": float(np.percentile(lk, 99))}
    # capacity: the same requests submitted at once
    srv = lib.Server(workers=args.workers, hbm_budget=int(args.budget_gb * (1 << 30)))
    srv.wait(srv.submit(**reqs[0]))
    t0 = time.perf_counter()
    tickets = [srv.submit(**r) for r in reqs]
    results_b = [srv.wait(t) for t in tickets]
    span_b = time.perf_counter() - t0
    st_b = srv.stats()
    retried_b = _retry_capacity(srv, reqs, results_b)
    srv.close()
    lat_b = np.array([r["latency_ms"] for r in results_b])
    out["burst"] = {"throughput_req_s": len(reqs) / span_b, "gvox_s": vox / span_b / 1e9,
                    "span_s": span_b, "p50_ms": float(np.percentile(lat_b, 50)),
                    "p99_ms": float(np.percentile(lat_b, 99)), "peak_running": st_b["peak_running"],
                    "batched": st_b["batched"], "batches": st_b["batches"],
                    "max_batch": st_b["max_batch"], "energy_batched": st_b["energy_batched"],
                    "energy_batches": st_b["energy_batches"],
                    "max_energy_batch": st_b["max_energy_batch"],
                    "mesh_batched": st_b["mesh_batched"], "failed": st_b["failed"],
                    "capacity_retries": retried_b, "failures": _failures(reqs, results_b)}
    # baseline: a sample of the same requests, plain FP64, one at a time
    ctx = lib.Context(0)
    # evenly spaced requests, leaving out grids above baseline_max_voxels (a
    # 1024^3 mesh in the plain FP64 form runs for many minutes)
    small = [i for i, r in enumerate(reqs)
             if "grid" not in r or r["grid"].n_voxels <= args.baseline_max_voxels]
    idx = small[::max(1, len(small) // args.baseline_sample)]
    base_t, serve_t = [], []
    for i in idx:
        r = reqs[i]
        t1 = time.perf_counter()
        if "grid" in r:
            h = ctx.upload(r["rs"])
            it = ctx.iter_params(r["max_it"], 2.0, precision=lib.QJG_FP64)
            if r["kind"] == lib.QJG_REQ_FIELD:
                ctx.field_host(h, r["grid"], it)
            else:
                import torch
                v = torch.empty(3 * r["vert_cap"], dtype=torch.float64, device="cuda")
                tt = torch.empty(3 * r["tri_cap"], dtype=torch.int32, device="cuda")
                ctx.mesh_stream(h, r["grid"], it, d_verts64=v.data_ptr(), vert_cap=r["vert_cap"],
                                d_tris=tt.data_ptr(), tri_cap=r["tri_cap"])
            ctx.free(h)
        else:
            import torch
            P = torch.from_numpy(r["params"]).cuda()
            X = torch.from_numpy(r["xyz"]).cuda()
            T = torch.from_numpy(r["target"]).cuda()
            G = torch.empty_like(P)
            ctx.energy(P.data_ptr(), r["rs"].n_top, r["rs"].n_bottom, len(r["target"]), X.data_ptr(),
                       T.data_ptr(), r["max_it"], 2.0, precision=lib.QJG_FP64, d_grad=G.data_ptr())
        base_t.append(time.perf_counter() - t1)
        serve_t.append(results[i]["run_ms"] / 1e3)
    out["baseline_fp64_serial"] = {
        "sampled_requests": len(idx), "max_voxels": args.baseline_max_voxels,
        "mean_s": statistics.mean(base_t),
        "throughput_req_s_est": 1.0 / statistics.mean(base_t),
        "served_run_s_same_requests": statistics.mean(serve_t)}
    return out


def mesh_algorithmic_bytes(n_voxels, n_verts, n_tris):
    """Algorithmic HBM bytes of the mesher's classify and triangle phases:
    the FP64 field read once (8 B per voxel) plus the FP32 vertices and
    int32 triangles written (12 B each)."""
    return 8 * n_voxels + 12 * n_verts + 12 * n_tris


def bench_large(args):
    """The large-grid configuration: 48 top / 24 bottom roots, 60 iterations,
    a res^3 grid (2200 by default) in 64-slice z-slabs.  (1) ONE pass of the
    precision field (FP32 bulk, double-float re-run at rel_tol, FP64 band)
    streamed through the mesher to FP32 vertices and int32 triangles, with
    the device time of each phase and the FP32 bulk kernel's FMA roofline
    from the same pass; (2) optionally (args.field_pass) the field alone over
    the same slabs; (3) evenly spaced z-slices in the precision form, the
    plain FP64 form (the reference's polar pow per root term) and the FP64
    form with integer powers as repeated products (the precision form's
    algebra in FP64): sign map, error, and the speed of each, so the
    speed-up splits into algorithm (pow -> products) and precision."""
    import torch

    from . import lib
    from .rootsets import large_workload
    from .roofline import field_flops
    ctx = lib.Context(0)
    args.res = args.res or 2200
    rs, g, p = large_workload(args.res)
    h = ctx.upload(rs)
    n = g.n_voxels
    XY = g.res[0] * g.res[1]
    it = ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP32_REFINE,
                         refine_pow=lib.QJG_REFINE_INT, rel_tol=args.rel_tol)
    out = {"workload": "large %d^3: 48 top / 24 bottom roots U[-1.2,1.2]^4 (seed 0), exponents "
                       "{1,2}, s = u * conformal scale, 60 iterations, escape 2" % args.res,
           "voxels": n, "slab": args.slab, "rel_tol": args.rel_tol}
    # warm the modules on a small grid
    from .rootsets import Grid
    small = Grid((64, 64, 64))
    ws = torch.empty(64 ** 3, dtype=torch.float64, device="cuda")
    ctx.field(h, small, it, ws.data_ptr())
    torch.cuda.synchronize()
    del ws
    peak = lib.fma_probe(0)
    field_gvox = None

    # (1) one streamed field + mesh pass
    if not args.no_mesh:
        vcap = int(args.vert_cap or 40 * XY)
        tcap = int(args.tri_cap or 80 * XY)
        v32 = torch.empty(3 * vcap, dtype=torch.float32, device="cuda")
        tris = torch.empty(3 * tcap, dtype=torch.int32, device="cuda")
        ctx.set_timing(True)
        torch.cuda.synchronize()
        e0, e1 = _events(torch)
        t0 = time.perf_counter()
        e0.record()
        rc, st = ctx.mesh_stream(h, g, it, check=False, d_verts32=v32.data_ptr(), vert_cap=vcap,
                                 d_tris=tris.data_ptr(), tri_cap=tcap, slab_nz=args.slab)
        e1.record()
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        if rc == -5:
            raise SystemExit("raise --vert-cap/--tri-cap: needs %d / %d" % (st["n_verts"], st["n_tris"]))
        V, T = st["n_verts"], st["n_tris"] + st["n_degenerate"]
        mesh_ms = st["ms_classify"] + st["ms_triangles"]
        alg = mesh_algorithmic_bytes(n, V, T)
        fs = st["field"]
        flops = field_flops(rs, fs["voxel_iters"])
        bulk = st["ms_field_bulk"]
        field_gvox = n / (st["ms_field"] * 1e-3) / 1e9
        out["mesh"] = {"passes": 1, "triangles": st["n_tris"], "vertices": V,
                       "degenerate": st["n_degenerate"], "unbracketed": st["n_unbracketed"],
                       "wall_s": wall, "device_ms": e0.elapsed_time(e1),
                       "triangles_per_s": st["n_tris"] / wall,
                       "ms_field": st["ms_field"], "ms_field_bulk": bulk,
                       "ms_classify": st["ms_classify"], "ms_vertices": st["ms_vertices"],
                       "ms_triangles": st["ms_triangles"], "ms_filter": st["ms_filter"],
                       "classify_emit_algorithmic_bytes": alg,
                       "classify_emit_gb_s": alg / (mesh_ms * 1e-3) / 1e9,
                       "classify_emit_frac_hbm": alg / (mesh_ms * 1e-3) / 1e9 / args.hbm_gbs,
                       "hbm_peak_gb_s": args.hbm_gbs,
                       "bisection_map_evals_fp64": st["map_evals"],
                       "bisection_map_evals_fp32": st["map_evals_fp32"],
                       "bisection_map_evals_ff": st["map_evals_ff"], "slabs": st["slabs"],
                       "field": fs}
        out["field"] = {"gvox_s": field_gvox, "source": "the streamed pass's field phase "
                        "(65 slices computed per 64-slice slab: one-plane overlap)",
                        "gvoxel_iterations_s": fs["voxel_iters"] / (st["ms_field"] * 1e-3) / 1e9,
                        "roofline": {"bound": "fma", "kernel": "field32x2_kernel",
                                     "achieved_tflops": flops / (bulk * 1e-3) / 1e12,
                                     "peak_tflops": peak,
                                     "frac": flops / (bulk * 1e-3) / 1e12 / peak},
                        "lane_efficiency": fs["voxel_iters"] / max(1, fs["lane_iters"])}
        del v32, tris
        torch.cuda.empty_cache()

    # (2) the field alone, slab by slab
    if args.field_pass or args.no_mesh:
        ctx.set_timing(True)
        buf = torch.empty(args.slab * XY, dtype=torch.float64, device="cuda")
        bulk = rest = 0.0
        tot = {}
        for z0 in range(0, g.res[2], args.slab):
            z1 = min(z0 + args.slab, g.res[2])
            ctx.field(h, g, it, buf.data_ptr(), z0=z0, z1=z1)
            b, r = ctx.last_timings()
            bulk, rest = bulk + b, rest + r
            for k, v in ctx.stats().items():
                tot[k] = tot.get(k, 0) + v
        del buf
        flops = field_flops(rs, tot["voxel_iters"])
        field_gvox = n / ((bulk + rest) * 1e-3) / 1e9
        out["field_alone"] = {
            "gvox_s": field_gvox, "bulk_ms": bulk, "rest_ms": rest,
            "gvoxel_iterations_s": tot["voxel_iters"] / ((bulk + rest) * 1e-3) / 1e9,
            "roofline": {"achieved_tflops": flops / (bulk * 1e-3) / 1e12, "peak_tflops": peak,
                         "frac": flops / (bulk * 1e-3) / 1e12 / peak},
            "stats": tot, "lane_efficiency": tot["voxel_iters"] / max(1, tot["lane_iters"])}

    # (3) sampled slices: precision form against both FP64 forms
    if args.check_slices > 0:
        forms = {"fp64_pow": ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP64),
                 "fp64_int": ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP64,
                                             refine_pow=lib.QJG_REFINE_INT),
                 "fp32_refine": it}
        zs = [int(v) for v in np.linspace(0, g.res[2] - 1, args.check_slices)]
        buf = {k: torch.empty(XY, dtype=torch.float64, device="cuda") for k in forms}
        ms = {k: 0.0 for k in forms}
        acc = {k: dict(sign=0, mx=0.0, ss=0.0) for k in ("fp64_pow", "fp64_int")}
        for z in zs:
            for k, itk in forms.items():
                e0, e1 = _events(torch)
                e0.record()
                ctx.field(h, g, itk, buf[k].data_ptr(), z0=z, z1=z + 1)
                e1.record()
                e1.synchronize()
                ms[k] += e0.elapsed_time(e1)
            a = buf["fp32_refine"]
            for k in acc:
                b = buf[k]
                acc[k]["sign"] += int(((a > 0) != (b > 0)).sum().item())
                rel = (a - b).abs() / b.abs().clamp_min(1e-300)
                acc[k]["mx"] = max(acc[k]["mx"], float(rel.max().item()))
                acc[k]["ss"] += float(rel.pow(2).sum().item())
        nv = len(zs) * XY
        gv = {k: nv / (ms[k] * 1e-3) / 1e9 for k in forms}
        ref_gvox = field_gvox or gv["fp32_refine"]
        chk = {"slices": zs, "voxels": nv}
        for k in acc:
            chk["vs_" + k] = {"sign_map_disagreements": acc[k]["sign"],
                              "max_rel_err": acc[k]["mx"], "rms_rel_err": (acc[k]["ss"] / nv) ** 0.5}
        chk.update({"gvox_s": gv,
                    "fp64_pow_full_grid_s_est": n / gv["fp64_pow"] / 1e9,
                    "speedup_vs_fp64_pow": ref_gvox / gv["fp64_pow"],
                    "speedup_vs_fp64_int": ref_gvox / gv["fp64_int"],
                    "speedup_algorithm_fp64_int_over_pow": gv["fp64_int"] / gv["fp64_pow"]})
        out["fp64_check"] = chk
    ctx.free(h)
    ctx.close()
    return out


def tooth_problem(path, n_top=12, n_bot=6, dres=64, seed=3):
    """A toothOptimizer input in the unit-cube frame of its state files: the
    signed distance of an ellipsoid (negative inside) on a dres^3 grid over
    [0, 1]^3, the first top root at the origin, the others around the shape,
    exponents 1 or 2; written as an .o3d state file."""
    import numpy as np

    from . import lib
    from .rootsets import Grid, RootSet, cell_centers
    rng = np.random.RandomState(seed)
    top = np.zeros((n_top, 4))
    top[1:, :3] = 0.5 + rng.uniform(-0.2, 0.2, (n_top - 1, 3))
    top[1:, 3] = rng.uniform(-0.05, 0.05, n_top - 1)
    bot = np.zeros((n_bot, 4))
    bot[:, :3] = 0.5 + rng.uniform(-0.3, 0.3, (n_bot, 3))
    bot[0, :3] = 0.03
    rs = RootSet(top_roots=top, top_powers=rng.choice([1.0, 2.0], n_top), bottom_roots=bot,
                 bottom_powers=rng.choice([1.0, 2.0], n_bot), scale=1.0)
    dg = Grid((dres,) * 3, center=(0.5, 0.5, 0.5), lengths=(1.0, 1.0, 1.0))
    c = cell_centers(dg) - 0.5
    dist = (np.sqrt(((c / np.array([0.3, 0.24, 0.2])) ** 2).sum(1)) - 1.0) * 0.22
    lib.o3d_write(path, rs, (4, 4, 4), (0.5, 0.5, 0.5), (1.0, 1.0, 1.0),
                  {"fractal": ((4, 4, 4), (0.5,) * 3, (1.0,) * 3, np.zeros(64)),
                   "distance": (dg.res, dg.center, dg.lengths, dist),
                   "curvature": (dg.res, dg.center, dg.lengths, dist)})
    return rs


def bench_tooth(args):
    """toothOptimizer's run (qjg_tooth_optimize) at levels 25, 50, 97 on a
    synthetic 12 top / 6 bottom root problem with a 64^3 target distance
    field (the reweighted solve needs an external signed-distance program and
    is left out): evaluations, time per level and per evaluation, against
    the C restatement's score-and-gradient evaluation on one host core."""
    import os
    import tempfile

    import numpy as np

    from . import lib
    from .rootsets import Grid
    levels = (25, 50, 97)
    ctx = lib.Context(0)
    tmp = tempfile.mkdtemp()
    path = os.path.join(tmp, "tooth_bench.o3d")
    tooth_problem(path)
    ctx.tooth_optimize(path, (12,), 4.0, 0.8)  # warm-up (module load, allocator)
    t0 = time.perf_counter()
    out = ctx.tooth_optimize(path, levels, 4.0, 0.8, output_prefix=os.path.join(tmp, "run"))
    wall = time.perf_counter() - t0
    res = {"workload": "toothOptimizer run, levels 25/50/97, 12 top / 6 bottom roots, 64^3 "
                       "target, fractal radius 4, amp 0.8, no reweighted solve",
           "wall_s": wall, "levels": []}
    # CPU: the oracle's one-pass score and gradients at each level's end state
    from oracle.oracle import Oracle, build
    build()
    o = Oracle()
    cpu_total = 0.0
    for L in out:
        ev = sum(sv["evaluations"] for sv in L["solve"])
        st = lib.o3d_read(os.path.join(tmp, "run_res_%d.o3d" % L["res"]))
        rs = lib.RootSet(top_roots=st["top_roots"], top_powers=st["top_powers"],
                         sigma_top=st["sigma_top"], bottom_roots=st["bottom_roots"],
                         bottom_powers=st["bottom_powers"], sigma_bottom=st["sigma_bottom"],
                         scale=st["scale"])
        dres, dc, dl, dd = st["distance"]
        g = Grid((L["res"],) * 3, dc, dl)
        wg = Grid(dres, dc, dl)
        w = np.abs(dd).ravel() + 0.01  # any weights: the cost does not depend on them
        t1 = time.perf_counter()
        o.tanh_score_grad(rs, g, wg, w, 1)
        cpu_eval = time.perf_counter() - t1
        cpu_total += cpu_eval * ev
        res["levels"].append({"res": L["res"], "evaluations": ev, "ms": L["ms"],
                              "gpu_ms_per_eval": L["ms"] / max(1, ev),
                              "cpu_ms_per_eval_1core": cpu_eval * 1e3,
                              "final_score": L["final_score"],
                              "solves": [sv["reason"] for sv in L["solve"]]})
    res["cpu_projected_s_1core"] = cpu_total
    res["speedup_vs_cpu_port"] = cpu_total / wall
    # one evaluation at the last level's end state, timed alone, without and
    # with the field written
    import torch
    L = out[-1]
    st = lib.o3d_read(os.path.join(tmp, "run_res_%d.o3d" % L["res"]))
    rs = lib.RootSet(top_roots=st["top_roots"], top_powers=st["top_powers"],
                     sigma_top=st["sigma_top"], bottom_roots=st["bottom_roots"],
                     bottom_powers=st["bottom_powers"], sigma_bottom=st["sigma_bottom"],
                     scale=st["scale"])
    dres, dc, dl, dd = st["distance"]
    g = Grid((L["res"],) * 3, dc, dl)
    wg = Grid(dres, dc, dl)
    dist = torch.from_numpy(np.ascontiguousarray(dd.ravel())).cuda()
    w = torch.empty_like(dist)
    ctx.inverted_distance(dres, dist.data_ptr(), True, w.data_ptr())
    f = torch.empty(g.n_voxels, dtype=torch.float64, device="cuda")
    h = ctx.upload(rs)
    npar = 3 + rs.n_top + rs.n_bottom
    for tag, fp in (("no_field", 0), ("with_field", f.data_ptr())):
        ctx.tanh_score_grad(h, g, 1, wg, w.data_ptr(), npar, d_field=fp)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        for _ in range(5):
            _, _, sst = ctx.tanh_score_grad(h, g, 1, wg, w.data_ptr(), npar, d_field=fp)
        res["eval_%s" % tag] = {"ms": (time.perf_counter() - t1) / 5 * 1e3, **sst}
    ctx.free(h)
    return res


def bench_tanh(args):
    """toothOptimizer's objective alone: one pass of the tanh score and its
    21 gradients (FP64, reference rounding) on the synthetic tooth problem of
    `bench_tooth` moved to the fractal frame, sigma 1 and the conformal
    scale, on a res^3 grid (97 by default); `--steps` timed passes."""
    import os
    import tempfile

    import numpy as np
    import torch

    from . import lib
    from .rootsets import Grid
    res = args.res or 97
    ctx = lib.Context(0)
    path = os.path.join(tempfile.mkdtemp(), "tanh_bench.o3d")
    tooth_problem(path)
    st = lib.o3d_read(path)
    R = 4.0
    tr, br = st["top_roots"].copy(), st["bottom_roots"].copy()
    tr[1:, :3] += -0.5
    br[1:, :3] += -0.5
    rs = lib.RootSet(top_roots=tr * R, top_powers=st["top_powers"], bottom_roots=br * R,
                     bottom_powers=st["bottom_powers"], scale=1.0)
    dres, dc, dl, dd = st["distance"]
    c = tuple((np.array(dc) - 0.5) * R)
    wg = Grid(dres, c, tuple(np.array(dl) * R))
    g = Grid((res,) * 3, c, wg.lengths)
    dist = torch.from_numpy(np.ascontiguousarray(dd.ravel()) * R).cuda()
    w = torch.empty_like(dist)
    ctx.inverted_distance(dres, dist.data_ptr(), True, w.data_ptr())
    h = ctx.upload(rs)
    _, _, rs.scale = ctx.conformal_radius(h, g, wg, dist.data_ptr())
    ctx.free(h)
    h = ctx.upload(rs)
    npar = 3 + rs.n_top + rs.n_bottom
    ctx.tanh_score_grad(h, g, 1, wg, w.data_ptr(), npar)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        score, _, sst = ctx.tanh_score_grad(h, g, 1, wg, w.data_ptr(), npar)
    ms = (time.perf_counter() - t0) / args.steps * 1e3
    ctx.free(h)
    return {"workload": "tanh score + %d gradients, 12 top / 6 bottom roots, %d^3" % (npar, res),
            "ms_per_eval": ms, "voxels_per_s": g.n_voxels / ms * 1e3, "score": score, **sst}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("what", choices=["mesh", "energy", "serve", "large", "tooth", "tanh",
                                     "classify", "lagrange", "mesh_fixed", "energy_batch"])
    ap.add_argument("--res", type=int, default=0, help="grid edge (mesh: 512, large: 2200)")
    ap.add_argument("--workload", default="precision", choices=["precision", "large"])
    ap.add_argument("--slab", type=int, default=64)
    ap.add_argument("--vert-cap", type=int, default=0)
    ap.add_argument("--tri-cap", type=int, default=0)
    ap.add_argument("--samples", type=int, default=200_000)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--fp32-only", action="store_true", help="energy: skip the FP64 forms")
    ap.add_argument("--requests", type=int, default=400)
    ap.add_argument("--scale", type=float, default=0.25)
    ap.add_argument("--span", type=float, default=20.0)
    ap.add_argument("--workers", type=int, default=8)
    ap.add_argument("--budget-gb", type=float, default=64.0)
    ap.add_argument("--baseline-sample", type=int, default=40)
    ap.add_argument("--baseline-max-voxels", type=int, default=1 << 24)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--rel-tol", type=float, default=1e-6)
    ap.add_argument("--check-slices", type=int, default=4)
    ap.add_argument("--no-mesh", action="store_true")
    ap.add_argument("--field-pass", action="store_true", help="large: also time the field alone")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--energy-accurate", action="store_true",
                    help="energy: the FP32 polar power with the accurate device functions")
    ap.add_argument("--energy-pairs", action="store_true",
                    help="energy: the forward kernel with two samples per lane")
    ap.add_argument("--batch-samples", type=int, default=25_000,
                    help="energy_batch: samples per item")
    ap.add_argument("--sweep-blocks", default="",
                    help="energy: comma-separated forward blocks per SM to time (0: the rule)")
    ap.add_argument("--z0", type=int, default=-1, help="classify: first plane of the slab")
    ap.add_argument("--hbm-gbs", type=float, default=0.0,
                    help="HBM roofline denominator (default: MEASURED_PEAKS.json, else 6800)")
    args = ap.parse_args()
    args.hbm_gbs = args.hbm_gbs or hbm_peak_gbs()[0]
    fn = {"mesh": bench_mesh, "energy": bench_energy, "serve": bench_serve,
          "large": bench_large, "tooth": bench_tooth, "tanh": bench_tanh,
          "classify": bench_classify, "lagrange": bench_lagrange,
          "mesh_fixed": bench_mesh_fixed, "energy_batch": bench_energy_batch}[args.what]
    print(json.dumps(fn(args)), flush=True)


if __name__ == "__main__":
    main()

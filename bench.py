"""Benchmark of the QUIJIBO hot path on GB300.

Workload (the precision-form configuration the headline metric is quoted
on): a rational quaternion map with 16 top / 8 bottom roots drawn uniform in
[-1.2,1.2]^4 (MT19937 seed 0), exponents in {1,2}, scale s = u * conformal
scale with u drawn in [0.5,2], 40 iterations, escape radius 2, on a 512^3
grid over [-1.5,1.5]^3 at slice w = 0.  One step = one FP32-bulk +
FP64-band-refine field pass over the whole grid (|d| < 2h re-evaluated in
FP64), output the FP64 field in HBM.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0).  Inputs are synthetic; see quijibo_gb300/rootsets.py.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from quijibo_gb300.roofline import field_flops  # noqa: E402

METRIC = "Julia field Gvox/s (FP32+refine vs FP64, same sign map); p50/p99 req latency"
RES = 512
WORKLOAD = ("precision form: 16 top / 8 bottom roots U[-1.2,1.2]^4 (seed 0), exponents {1,2}, "
            "s = u * conformal scale (u in [0.5,2]), 40 iterations, escape 2, %d^3 grid over "
            "[-1.5,1.5]^3, slice 0; FP32 bulk, double-float-head re-run of voxels whose tracked "
            "FP32 error exceeds rel_tol, FP64 re-evaluation of |d| < 2h")
# DRAM bytes of one field32x2_kernel launch on the 512^3 workload (ncu,
# dram__bytes_read.sum + dram__bytes_write.sum, one pass at full size): the
# FMA-bound kernel moves ~7.7 B per voxel, the FP64 field it writes
TRAFFIC_PER_VOXEL = (19.15e6 + 1.01e9) / 512 ** 3


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms; start()
    returns once the first sample is written, so the timed region that
    follows is covered from its start."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        rows = []
        for line in open(self.path):
            f = [v.strip() for v in line.split(",")]
            if len(f) >= 8 and f[0].isdigit():
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[4 + k] == "Active"})
        return {"sm_mhz": statistics.median(float(r[0]) for r in rows),
                "sm_max_mhz": max(float(r[1]) for r in rows),
                "power_w_max": max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit()),
                "samples": len(rows), "reasons": reasons}


def cpu_sample(rs, g, p, slices, nthreads=0):
    """Time the oracle port (double, OpenMP) on the listed z-slices."""
    from oracle.oracle import Oracle, build
    build()
    o = Oracle()
    t0 = time.perf_counter()
    vox = 0
    for z in slices:
        o.field(rs, g, p["max_it"], p["escape"], z0=z, z1=z + 1, nthreads=nthreads)
        vox += g.res[0] * g.res[1]
    dt = time.perf_counter() - t0
    return vox, dt


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("QJ_BENCH_GLOO") is None else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, v):
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, world, rank):
    """The reference arm: the CPU implementation of the path (the oracle port
    of the reference's double build) on the host cores, one bounded z-slice
    sample of the same workload per step."""
    from quijibo_gb300.rootsets import precision_workload
    if rank != 0:
        return
    rs, g, p = precision_workload(args.res)
    cores = os.cpu_count()
    # steps walk evenly spaced slices so each step samples the whole height
    per_step = max(1, args.ref_slices)
    order = [int(v) for v in np.linspace(0, g.res[2] - 1, per_step * (args.steps + args.warmup))]
    for w in range(args.warmup):
        cpu_sample(rs, g, p, order[w * per_step:(w + 1) * per_step])
    vox, dt = 0, 0.0
    for k in range(args.steps):
        s = order[(args.warmup + k) * per_step:(args.warmup + k + 1) * per_step]
        v, t = cpu_sample(rs, g, p, s)
        vox, dt = vox + v, dt + t
    value = vox / dt / 1e9
    line = {"metric": METRIC, "value": value, "unit": "Gvox/s", "impl": "reference",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD % args.res, "res": args.res,
                       "sample": "%d z-slices of %d^2 voxels per step" % (per_step, args.res)},
            "cpu_baseline": {"value": value, "unit": "Gvox/s", "cores": cores, "kind": "port",
                             "sample": "%d z-slices per step, %d steps" % (per_step, args.steps)},
            "e2e": {"value": value, "unit": "Gvox/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import torch

    from quijibo_gb300 import lib
    from quijibo_gb300.rootsets import precision_workload

    torch.cuda.set_device(local)
    ctx = lib.Context(local)
    rs, g, p = precision_workload(args.res)
    h = ctx.upload(rs)
    n = g.n_voxels
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    field = torch.empty(n, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > L2 (129 MB)
    it = ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP32_REFINE,
                         refine_pow=lib.QJG_REFINE_INT, band_h=2.0, rel_tol=args.rel_tol)
    ctx.set_timing(True)

    for _ in range(args.warmup):
        ctx.field(h, g, it, field.data_ptr(), stream=sptr)
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    if rank == 0:
        clocks.start()
    launches0 = ctx.launch_count()
    step_ms, bulk_ms, refine_ms = [], [], []
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.field(h, g, it, field.data_ptr(), stream=sptr)
        e1.record(stream)
        b, r = ctx.last_timings()
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        bulk_ms.append(b)
        refine_ms.append(r)
    torch.cuda.synchronize()
    barrier(world)
    wall = time.perf_counter() - t_wall
    launches = ctx.launch_count() - launches0
    clk = clocks.stop() if rank == 0 else None
    st = ctx.stats(sptr)
    ms = max_over_ranks(world, statistics.mean(step_ms))
    value = world * n / (ms * 1e-3) / 1e9

    # FP64 plain form on the same workload: speed and sign-map / error check
    fp64 = None
    if not args.no_fp64:
        it64 = ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP64)
        f64 = torch.empty(n, dtype=torch.float64, device="cuda")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.field(h, g, it64, f64.data_ptr(), stream=sptr)
        e1.record(stream)
        e1.synchronize()
        ms64 = e0.elapsed_time(e1)
        st64 = ctx.stats(sptr)
        sign_diff = int(((field > 0) != (f64 > 0)).sum().item())
        rel = (field - f64).abs() / f64.abs().clamp_min(1e-300)
        fp64 = {"gvox_s": n / (ms64 * 1e-3) / 1e9, "ms": ms64, "speedup_fp32_refine": ms64 / ms,
                "sign_map_disagreements": sign_diff, "max_rel_err": float(rel.max().item()),
                "rms_rel_err": float(rel.pow(2).mean().sqrt().item()),
                "frac_rel_err_le_1e-6": float((rel <= 1e-6).double().mean().item()),
                "voxel_iters": st64["voxel_iters"],
                "form": "plain FP64: the reference's polar QUATERNION::pow per root term"}
        del rel
        # the same algebra as the precision form (integer powers as repeated
        # products) in FP64: splits the speed-up into algorithm and precision
        iti = ctx.iter_params(p["max_it"], p["escape"], precision=lib.QJG_FP64,
                              refine_pow=lib.QJG_REFINE_INT)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.field(h, g, iti, f64.data_ptr(), stream=sptr)
        e1.record(stream)
        e1.synchronize()
        msi = e0.elapsed_time(e1)
        rel = (field - f64).abs() / f64.abs().clamp_min(1e-300)
        fp64["int_powers"] = {
            "form": "FP64 with integer powers as repeated products (the precision form's algebra)",
            "gvox_s": n / (msi * 1e-3) / 1e9, "ms": msi, "speedup_fp32_refine": msi / ms,
            "speedup_algorithm_int_over_pow": ms64 / msi,
            "sign_map_disagreements": int(((field > 0) != (f64 > 0)).sum().item()),
            "max_rel_err": float(rel.max().item()),
            "rms_rel_err": float(rel.pow(2).mean().sqrt().item())}
        del f64, rel

    # roofline of the FP32 bulk kernel (FMA-pipe bound)
    peak = lib.fma_probe(local)
    bulk = statistics.mean(bulk_ms)
    flops = field_flops(rs, st["voxel_iters"])
    achieved = flops / (bulk * 1e-3) / 1e12

    # end to end through the host-buffer entry point, pinned host output
    host = torch.empty(n, dtype=torch.float64, pin_memory=True).numpy().reshape(g.res[::-1])
    e2e_t = []
    for k in range(args.e2e_steps + 1 if args.e2e_steps else 0):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        hh = ctx.upload(rs)  # the root set crosses to the device every step
        ctx.field_host(hh, g, it, out=host)
        ctx.free(hh)
        if k:  # the first call warms the staging buffers
            e2e_t.append(time.perf_counter() - t0)
    h2d = 8 * (5 * (rs.n_top + rs.n_bottom)) + 8 * 4
    e2e = None
    if e2e_t:
        e2e = {"value": world * n / max_over_ranks(world, statistics.mean(e2e_t)) / 1e9,
               "unit": "Gvox/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 8 * n}

    # serving: a Poisson-arrival stream of field / field+mesh / energy+gradient
    # requests at the serving configuration's sizes (fields 32^3-512^3, meshes
    # 128^3-1024^3, 10k-200k samples) and its offered rate (22 req/s), p50/p99
    serving = None
    if rank == 0 and not args.no_serve:
        from quijibo_gb300.benchmarks import bench_serve
        sargs = argparse.Namespace(seed=0, requests=args.serve_requests, scale=1.0,
                                   span=args.serve_requests / 22.2,
                                   workers=8, budget_gb=64.0, baseline_sample=10,
                                   baseline_max_voxels=1 << 24)
        serving = bench_serve(sargs)

    # the large-grid configuration (48/24 roots, 60 iterations, 2200^3 in
    # 64-slice slabs): one streamed field + mesh pass, its FMA roofline and
    # mesher GB/s, and sampled slices against both FP64 forms
    large = None
    if rank == 0 and not args.no_large:
        from quijibo_gb300.benchmarks import bench_large, hbm_peak_gbs
        largs = argparse.Namespace(res=args.large_res, slab=64, rel_tol=args.rel_tol, vert_cap=0,
                                   tri_cap=0, no_mesh=False, field_pass=False,
                                   check_slices=args.large_slices, hbm_gbs=hbm_peak_gbs()[0])
        large = bench_large(largs)

    # the differentiation configuration (200k Poisson-disk samples, 64 top /
    # 16 bottom roots, 30 iterations): FP32 forward + recompute-free adjoint
    # per call (gradients/s), both FP64 forms beside it, the algorithmic FLOP
    # rate of each against the FMA probe, and 50 device L-BFGS steps
    energy = None
    if rank == 0 and not args.no_energy:
        from quijibo_gb300.benchmarks import bench_energy
        eargs = argparse.Namespace(samples=200_000, steps=50, fp32_only=False,
                                   energy_pairs=False, energy_accurate=False)
        energy = bench_energy(eargs)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        slices = [int(v) for v in np.linspace(0, g.res[2] - 1, args.cpu_slices)]
        vox, dt = cpu_sample(rs, g, p, slices)
        cpu = {"value": vox / dt / 1e9, "unit": "Gvox/s", "cores": os.cpu_count(), "kind": "port",
               "sample": "%d evenly spaced z-slices (%d voxels, %.1f s)" % (len(slices), vox, dt)}

    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": "Gvox/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
        "config": {"workload": WORKLOAD % args.res, "res": args.res, "voxels": n,
                   "rel_tol": args.rel_tol,
                   "l2": "L2 flushed (256 MiB write) between timed steps; output 1 GiB > L2",
                   "parallelism": "one grid per GPU" if world > 1 else "single GPU"},
        "fp64_plain": fp64,
        "field_stats": dict(st, bulk_ms=bulk, refine_ms=statistics.mean(refine_ms),
                            wall_s=wall, refined_frac=st["refined"] / n,
                            gvoxel_iterations_s=world * st["voxel_iters"] / (ms * 1e-3) / 1e9,
                            lane_efficiency=st["voxel_iters"] / max(1, st["lane_iters"])),
        "roofline": {"bound": "fma", "kernel": "field32x2_kernel", "achieved": achieved,
                     "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                     "traffic": TRAFFIC_PER_VOXEL * n,
                     "traffic_source": "ncu dram bytes of one 512^3 launch, per voxel x voxels",
                     "peak_source": "measured FP32 FMA-chain probe (qjg_fma_probe), same run",
                     "flops_per_launch": flops},
        "cpu_baseline": cpu,
        "serving": serving,
        "large": large,
        "energy": energy,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--res", type=int, default=RES)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--rel-tol", type=float, default=1e-6,
                    help="target relative field error of the precision form (0: band rule only)")
    ap.add_argument("--cpu-slices", type=int, default=12)
    ap.add_argument("--ref-slices", type=int, default=3)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 plain-form comparison")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving stream")
    ap.add_argument("--serve-requests", type=int, default=400)
    ap.add_argument("--no-large", action="store_true", help="skip the 2200^3 large-grid record")
    ap.add_argument("--large-res", type=int, default=2200)
    ap.add_argument("--large-slices", type=int, default=4)
    ap.add_argument("--no-energy", action="store_true",
                    help="skip the 200k-sample energy + gradient record")
    args = ap.parse_args()
    world, rank, local = dist_init()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

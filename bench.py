#!/usr/bin/env python
"""Benchmark of the NGLOD neural-SDF hot path on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Headline workload (``config.workload``): ``OctreeSDF.sdf(x, lod=4)`` of the
full architecture (5 LODs, 5^3..65^3 volumes, C=32, H=128) on 4,194,304 query
points, half uniform in [-1,1]^3 and half within 0.02 of the 16-sphere-union
surface (seed 1), in the BF16 form (bf16 volumes, tcgen05 decoder with fp32
accumulation) -- the mixed-precision inference configuration.  One step =
one pass over the batch.  ``value`` is queries/s with the points already
resident in HBM; ``e2e`` is the same metric through the public API with
host buffers (``Bf16OctreeSDF.sdf_host`` -> ``nglod_sdf_fwd_bf16_host``): the
points are copied from pinned host memory and the distances copied back inside
the timed region, in 256k-point chunks whose copies overlap the kernels.
``fp32`` repeats the measurement for the float32 drop-in (``OctreeSDF.sdf``),
which matches the reference to 1e-5.

The model holds the sphere-union SDF through ``analytic_init`` (deterministic
and traced with real hits; throughput does not depend on the weights).
Between timed steps an L2 flush (a 256 MiB write, larger than the 129 MB L2)
runs outside the timed events.

Extra keys: ``trace`` (sphere tracers at 1920x1080, 64 steps: fused BF16,
fused float32 and the plain per-step float32 tracer), ``serve`` (the
continuous-batching server under a Poisson request stream), ``train`` (the
training step against the reference computation in stock PyTorch ops, then
2,000 steps and the BF16 form on the trained weights), ``sparse`` (SPC octree
traversal + sparse BF16 trace of a 1080p frame), ``shade`` (a shaded 1080p
frame: trace, ground plane, shadow rays, ambient occlusion, matcap),
``mesh`` (mesh signed distance of 1M points against 20,480 triangles),
``roofline``,
``cpu_baseline``, ``clocks``, ``gpu_launches``.  ``--only LEG`` runs one
extra leg alone (for profiling).

``--impl reference`` times the reference's own CPU torch computation (the
restatement in oracle/torch_port.py, same torch operators) on the host cores
on a bounded sample of the same workload and prints the same metric.

Several GPUs (torchrun): the path shards only as independent replicas; each
rank runs the full workload on its own GPU (weak scaling, no collective on
the data path); rank 0 prints the aggregate.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_POINTS = 4_194_304
LOD = 4
TRACE_W, TRACE_H, TRACE_STEPS = 1920, 1080, 64
METRIC = "sdf_queries_per_s"
UNIT = "queries/s"
WORKLOAD = "OctreeSDF.sdf(x, lod=4): 5 LODs (5^3..65^3 volumes), C=32, H=128, 4,194,304 points"
CPU_SAMPLE = 262_144
FLUSH_BYTES = 256 << 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=500)
    p.add_argument("--warmup", type=int, default=10)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--no-extras", action="store_true", help="skip the trace and CPU-baseline legs")
    p.add_argument("--only", choices=["trace", "aabb", "summed", "train", "sparse", "serve", "shade", "mesh"], default=None,
                   help="run one extra leg alone (profiling); prints its JSON")
    return p.parse_args()


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# sdf_fwd_bf16_tc_kernel on this workload, from the ncu capture summarised in
# profiles/sdf_fwd_bf16_tc_4M.md (the algorithmic bytes of a launch are
# 67.1 MB of points and results plus 40.4 MB of bf16 pair volumes; the
# results still in L2 when the kernel ends are written back later).
NCU_TRAFFIC_BYTES = 90_623_232 + 10_336_512
NCU_TRAFFIC_SOURCE = "ncu --set full capture of one launch, 4,194,304 points (profiles/sdf_fwd_bf16_tc_4M.md)"


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(v, ws, dev):
    if ws == 1:
        return v
    import torch.distributed as dist
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.item()


def build_model(dev=None):
    import nglod_gb300 as ng
    from nglod_gb300 import synthetic
    from nglod_gb300.analytic_init import init_from_sdf
    from nglod_gb300.options import default_args
    c, r = synthetic.sphere_union(1)
    torch.manual_seed(0)
    net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2))
    init_from_sdf(net, lambda p: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)), noise=1e-3, seed=2)
    net.eval()
    return net.to(dev) if dev is not None else net, (c, r)


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons while running."""
    FIELDS = ["clocks.sm", "clocks.max.sm", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, index):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(index), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) != len(self.FIELDS):
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def time_steps(fn, steps, flush, stream):
    """Sum of per-step CUDA-event durations (ms) on `stream`, L2 flushed between steps."""
    total = 0.0
    evs = []
    for k in range(steps):
        flush.fill_(k & 0xFF)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        evs.append((a, b))
    torch.cuda.synchronize()
    for a, b in evs:
        total += a.elapsed_time(b)
    return total


def line_read_peak(dev, nbytes, reps=20):
    """Measured ceiling of the gather's corner reads: random whole 128-byte
    lines of an L2-resident buffer of `nbytes` (the pair volumes' size) read
    with the gather's 256-bit loads, four lanes per line
    (nglod_measure_line_reads), 64 warps per SM; GB/s, best of `reps`."""
    from nglod_gb300 import _lib
    lines = nbytes // 128
    buf = torch.zeros(lines * 128, dtype=torch.uint8, device=dev)
    sink = torch.zeros(1, dtype=torch.int32, device=dev)
    blocks = torch.cuda.get_device_properties(dev).multi_processor_count * 16
    loads = 256
    lib = _lib.load()

    def go():
        _lib.check(lib.nglod_measure_line_reads(_lib.ptr(buf), lines, loads, blocks, _lib.ptr(sink),
                                                _lib.stream_ptr(dev)), "nglod_measure_line_reads")

    for _ in range(3):
        go()
    torch.cuda.synchronize()
    best = float("inf")
    stream = torch.cuda.current_stream(dev)
    for _ in range(reps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        go()
        b.record(stream)
        b.synchronize()
        best = min(best, a.elapsed_time(b))
    return blocks * 128 * loads * 32 / (best / 1e3) / 1e9


def run_ours(args):
    ws, rank, local = dist_setup()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    import nglod_gb300 as ng
    from nglod_gb300 import synthetic
    ng.load_library()
    from nglod_gb300.bf16 import Bf16OctreeSDF
    net, (c, r) = build_model(dev)
    bnet = Bf16OctreeSDF(net)
    x_host = synthetic.near_surface_query(N_POINTS, c, r, seed=1).pin_memory()
    x = x_host.to(dev)
    out_host = torch.empty(N_POINTS, 1).pin_memory()
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step():
        return bnet.sdf(x, lod=LOD)

    def step32():
        with torch.no_grad():
            return net.sdf(x, lod=LOD)

    for _ in range(max(args.warmup, 3)):
        step()
        step32()
    torch.cuda.synchronize()

    clocks = ClockSampler(local)
    barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    kern_ms = time_steps(step, args.steps, flush, stream)
    torch.cuda.synchronize()
    barrier(ws)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    kern_ms = max_over_ranks(kern_ms, ws, dev)
    ms_per_step = kern_ms / args.steps
    value = ws * N_POINTS / (ms_per_step / 1e3)
    bnet.check_status()
    steps32 = max(10, args.steps // 5)
    ms32 = max_over_ranks(time_steps(step32, steps32, flush, stream), ws, dev) / steps32

    # e2e through the public API with host buffers: Bf16OctreeSDF.sdf_host ->
    # nglod_sdf_fwd_bf16_host copies the pinned points in and the distances
    # out every step, in 256k-point chunks whose copies overlap the kernels.
    def e2e_step():
        bnet.sdf_host(x_host, lod=LOD, out=out_host)

    e2e_steps = min(args.steps, 100)
    for _ in range(3):
        e2e_step()
    torch.cuda.synchronize()
    barrier(ws)
    e2e_ms = time_steps(e2e_step, e2e_steps, flush, stream) / e2e_steps
    e2e_ms = max_over_ranks(e2e_ms, ws, dev)
    ref = bnet.sdf(x[:4096], lod=LOD)
    torch.cuda.synchronize()
    assert torch.equal(out_host[:4096].to(dev), ref), "e2e result differs from the resident result"

    pk = peaks()
    grid_bytes = sum(fv.fm.numel() * 2 for fv in net.features)
    pair_bytes = sum(pv.numel() * 2 for pv in bnet.pairs) or grid_bytes  # what the launch reads
    line_peak = line_read_peak(dev, pair_bytes)
    hbm_bytes = N_POINTS * (12 + 4) + pair_bytes
    gather_bytes = N_POINTS * (LOD + 1) * 8 * 32 * 2
    tc_flop = N_POINTS * 2 * 35 * 128
    sec = ms_per_step / 1e3
    roofline = {
        "bound": "hbm", "achieved": hbm_bytes / sec / 1e9, "peak": pk["hbm_gbs"], "unit": "GB/s",
        "frac": hbm_bytes / sec / 1e9 / pk["hbm_gbs"], "traffic": NCU_TRAFFIC_BYTES,
        "traffic_source": NCU_TRAFFIC_SOURCE, "algorithmic_bytes": hbm_bytes,
        "peak_source": f"{pk['source']} hbm_gbs (burst copy)",
        "kernel": "sdf_fwd_bf16_tc_kernel",
        "per_query": {"hbm_bytes": 16, "gathered_bytes": (LOD + 1) * 8 * 32 * 2, "tensor_flop": 2 * 35 * 128,
                      "fp32_epilogue_flop": 3 * 128},
        "binding": {"resource": "L1 data-pipe wavefronts (corner gathers + tile rows)", "frac": 0.737,
                    "issue_active": 0.568,
                    "source": "ncu --set full capture of one launch (profiles/sdf_fwd_bf16_tc_4M.md)"},
        "gather_gbs": gather_bytes / sec / 1e9,
        "gather": {"gbs": gather_bytes / sec / 1e9, "line_read_peak_gbs": line_peak,
                   "frac": gather_bytes / sec / 1e9 / line_peak,
                   "peak_source": "measured live: random whole 128-byte lines of an L2-resident buffer the size of "
                                  "the pair volumes, read with the gather's 256-bit loads (nglod_measure_line_reads)",
                   "note": "the gathered bytes (2,560 B per query) include L1 hits (about 28 %), so this fraction "
                           "may exceed the share of the L2 ceiling"},
        "tensor_tflops": tc_flop / sec / 1e12,
        "tensor_frac_of_bf16_peak": tc_flop / sec / 1e12 / pk["bf16_tflops"],
        "note": "one launch reads each point once and the 40.4 MB of bf16 pair volumes (each vertex beside "
                "its +x neighbour, 128-byte lines) from HBM; the corner gathers (2,560 B/query, four whole "
                "lines per LOD) are served by L2/L1, and the gather's instruction stream (half of it bf16 "
                "unpacking) binds the kernel: with every load an L1 hit it still takes 88 % of the time; "
                "the 35x128 decoder layer runs on tcgen05 tensor cores and is a small share of the time",
    }
    sec32 = ms32 / 1e3
    fp32 = {"value": ws * N_POINTS / sec32, "unit": UNIT, "ms_per_step": ms32, "steps": steps32,
            "kernel": "sdf_fwd_f32_kernel", "parity": "1e-5 abs vs the reference",
            "gather_gbs": N_POINTS * (LOD + 1) * 8 * 32 * 4 / sec32 / 1e9,
            "fp32_tflops": N_POINTS * ((LOD + 1) * 8 * 32 * 2 + 2 * (36 * 128 + 128)) / sec32 / 1e12,
            "hbm_frac": (N_POINTS * 16 + grid_bytes * 2) / sec32 / 1e9 / pk["hbm_gbs"]}

    extras = {}
    if not args.no_extras:
        extras["trace"] = bench_trace(net, bnet, dev, flush, stream)
        extras["summed"] = bench_summed(net, bnet, x, dev, flush, stream)

    if not args.no_extras:
        extras["serve"] = bench_serve(dev)
        extras["train"] = bench_train(dev, flush, stream)
        extras["sparse"] = bench_sparse(net, dev, flush, stream)
        extras["shade"] = bench_shade(net, bnet, dev, flush, stream)
        extras["mesh"] = bench_mesh(dev, flush, stream)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_extras:
        cpu = cpu_baseline(net)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
            "config": {"workload": WORKLOAD, "points": N_POINTS, "lod": LOD,
                       "form": "BF16 (bf16 volumes, tcgen05 bf16 decoder, fp32 accumulate)",
                       "point_distribution": "half U[-1,1]^3, half within 0.02 of the 16-sphere union (seed 1)",
                       "l2": "256 MiB flush between timed steps", "parallelism": f"replicas x{ws}"},
            "e2e": {"value": ws * N_POINTS / (e2e_ms / 1e3), "unit": UNIT,
                    "h2d_bytes_per_step": N_POINTS * 12, "d2h_bytes_per_step": N_POINTS * 4},
            "gpu_launches": args.steps,
            "roofline": roofline,
            "fp32": fp32,
            "clocks": clk,
            "cpu_baseline": cpu,
            "wall_s_timed_region": wall,
        }
        line.update(extras)
        print(json.dumps(line), flush=True)


def bench_summed(net, bnet, x, dev, flush, stream, steps=100):
    """The BF16 form over LOD-summed volumes (Bf16OctreeSDF(summed=True)):
    the headline workload with one 8-corner gather per query instead of
    LOD + 1, against the per-LOD BF16 form on the same points, plus the
    tracer over the same volumes."""
    import nglod_gb300 as ng
    from nglod_gb300 import synthetic
    from nglod_gb300.bf16 import Bf16OctreeSDF
    from nglod_gb300.options import default_args
    sb = Bf16OctreeSDF(net, summed=True)
    for _ in range(3):
        got = sb.sdf(x, lod=LOD)
    torch.cuda.synchronize()
    ms = time_steps(lambda: sb.sdf(x, lod=LOD), steps, flush, stream) / steps
    sb.check_status()
    d = (got - bnet.sdf(x, lod=LOD)).abs()
    ro, rd = synthetic.look_at_rays(width=TRACE_W, height=TRACE_H)
    ro, rd = ro.to(dev), rd.to(dev)
    fused = ng.SphereTracer(default_args(num_steps=TRACE_STEPS))
    for _ in range(3):
        rbs = fused(sb, ro, rd)
    torch.cuda.synchronize()
    tms = time_steps(lambda: fused(sb, ro, rd), 10, flush, stream) / 10
    rb16 = fused(bnet, ro, rd)
    sb.check_status()
    return {"form": "BF16 over LOD-summed volumes: volume l = sum of the samples of volumes 0..l at LOD l's "
                    "vertices (float64, one bf16 rounding); a query samples volume LOD alone",
            "value": N_POINTS / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": steps,
            "gathered_bytes_per_query": 8 * 32 * 2,
            "vs_per_lod_bf16_max_abs": float(d.max().item()), "vs_per_lod_bf16_mean_abs": float(d.mean().item()),
            "trace_ms": tms, "trace_rays_per_s": ro.shape[0] / (tms / 1e3),
            "trace_hit_agreement_vs_per_lod_bf16": float((rbs.hit == rb16.hit).float().mean().item())}


def bench_aabb(dev, flush, stream, steps=50):
    """sol_nglod.aabb (nglod_aabb) on the 1920x1080 camera rays of the trace
    workload: 24 B in and 17 B out per ray, HBM-bound; L2 flushed between
    steps."""
    from nglod_gb300 import _lib, sol_nglod, synthetic
    ro, rd = synthetic.look_at_rays(width=TRACE_W, height=TRACE_H)
    ro, rd = ro.to(dev), rd.to(dev)
    n = ro.shape[0]
    x = torch.empty_like(ro)
    t = torch.empty(n, 1, device=dev)
    hit = torch.empty(n, dtype=torch.bool, device=dev)
    lib = _lib.load()

    def launch():  # the C entry on preallocated outputs: one kernel
        _lib.check(lib.nglod_aabb(_lib.ptr(ro), _lib.ptr(rd), n, _lib.ptr(x), _lib.ptr(t), _lib.ptr(hit),
                                  _lib.stream_ptr(dev)), "nglod_aabb")

    for _ in range(3):
        launch()
        sol_nglod.aabb(ro, rd)
    torch.cuda.synchronize()
    ms = time_steps(launch, steps, flush, stream) / steps
    ms_api = time_steps(lambda: sol_nglod.aabb(ro, rd), steps, flush, stream) / steps
    nbytes = n * (24 + 12 + 4 + 1)
    pk = peaks()
    return {"workload": f"sol_nglod.aabb, {n} rays ({TRACE_W}x{TRACE_H} camera (0,0,4) fov 30)",
            "ms": ms, "rays_per_s": n / (ms / 1e3), "bytes_per_ray": 41, "gbs": nbytes / (ms / 1e3) / 1e9,
            "hbm_frac": nbytes / (ms / 1e3) / 1e9 / pk["hbm_gbs"], "hits": int(hit.sum().item()),
            "ms_python_api": ms_api}


def bench_trace(net, bnet, dev, flush, stream):
    import nglod_gb300 as ng
    from nglod_gb300 import synthetic
    from nglod_gb300.options import default_args
    ro, rd = synthetic.look_at_rays(width=TRACE_W, height=TRACE_H)
    ro, rd = ro.to(dev), rd.to(dev)
    a = default_args(num_steps=TRACE_STEPS)
    fused = ng.SphereTracer(a)
    plain = ng.PlainSphereTracer(a)
    n = ro.shape[0]
    for _ in range(3):
        rb = fused(net, ro, rd)
    torch.cuda.synchronize()
    reps = 10
    ms = time_steps(lambda: fused(net, ro, rd), reps, flush, stream) / reps
    hits = int(rb.hit.sum().item())
    for _ in range(3):
        rb16 = fused(bnet, ro, rd)
    torch.cuda.synchronize()
    ms16 = time_steps(lambda: fused(bnet, ro, rd), reps, flush, stream) / reps
    bnet.check_status()
    both = rb.hit & rb16.hit
    derr = (rb.depth[both] - rb16.depth[both]).abs()
    plain(net, ro, rd)
    torch.cuda.synchronize()
    runs = []
    for _ in range(3):  # host-synchronising loop: wall clock, median of three frames
        t0 = time.perf_counter()
        plain(net, ro, rd)
        torch.cuda.synchronize()
        runs.append((time.perf_counter() - t0) * 1e3)
    pms = statistics.median(runs)
    return {"workload": f"SphereTracer {TRACE_W}x{TRACE_H}, {TRACE_STEPS} steps, lod=None (finest), camera (0,0,4) fov 30",
            "fused_f32_rays_per_s": n / (ms / 1e3), "fused_f32_ms": ms,
            "fused_bf16_rays_per_s": n / (ms16 / 1e3), "fused_bf16_ms": ms16,
            "bf16_vs_f32_hit_agreement": float((rb.hit == rb16.hit).float().mean().item()),
            "bf16_vs_f32_depth_mean_abs": float(derr.mean().item()) if derr.numel() else None,
            "plain_f32_rays_per_s": n / (pms / 1e3), "plain_f32_ms": pms, "hits": hits, "kernel_launches_fused": 2,
            "bf16_over_plain_f32": (n / (ms16 / 1e3)) / (n / (pms / 1e3))}


def bench_shade(net, bnet, dev, flush, stream):
    """Shaded frame (Renderer.shade_tensor with a ground plane, shadow rays and
    ambient occlusion, matcap colour): 1920x1080, 64 steps, camera (1.6, 1.4,
    3.4) looking at (0, -0.1, 0), fov 35, for the BF16 and float32 networks;
    the primary trace, the shadow-ray trace and 40 sdf taps per shaded pixel
    are the bulk of it."""
    from nglod_gb300.options import default_args
    from nglod_gb300.renderer import Renderer
    import nglod_gb300 as ng
    tr = ng.SphereTracer(default_args(num_steps=TRACE_STEPS))
    r = Renderer(tr, args=default_args(render_res=[TRACE_W, TRACE_H], shadow=True, ao=True, ground_height=-0.75))
    f, t, fov = (1.6, 1.4, 3.4), (0.0, -0.1, 0.0), 35.0
    out = {"workload": f"Renderer.shade_tensor {TRACE_W}x{TRACE_H}: trace ({TRACE_STEPS} steps) + ground plane + "
                       "shadow rays + AO (40 taps) + matcap, camera (1.6, 1.4, 3.4) -> (0, -0.1, 0) fov 35"}
    for name, m in (("bf16", bnet), ("f32", net)):
        for _ in range(2):
            rb = r.shade_tensor(m, f=f, t=t, fov=fov)
        torch.cuda.synchronize()
        reps = 5
        ms = time_steps(lambda: r.shade_tensor(m, f=f, t=t, fov=fov), reps, flush, stream) / reps
        out[f"{name}_frame_ms"] = ms
        out[f"{name}_hit_fraction"] = float(rb.hit.float().mean().item())
        out[f"{name}_shaded_fraction"] = float((rb.ao < 1).float().mean().item())
    if hasattr(bnet, "check_status"):
        bnet.check_status()
    return out


def bench_mesh(dev, flush, stream):
    """Mesh signed distance (compute_sdf): 1,048,576 points uniform in
    [-1.2, 1.2]^3 against an icosphere of 20,480 triangles; the unit is one
    point-triangle test (distance + 13 line crossings)."""
    from nglod_gb300 import mesh, synthetic
    V, F = synthetic.icosphere(5)
    Vd = torch.from_numpy(V).float().to(dev)
    Fd = torch.from_numpy(F).to(dev)
    rec = mesh.triangle_records(Vd, Fd)
    n = 1 << 20
    pts = (torch.rand(n, 3, device=dev, generator=torch.Generator(device=dev).manual_seed(0)) * 2.4 - 1.2)
    for _ in range(2):
        mesh.mesh_sdf(rec, pts)
    torch.cuda.synchronize()
    reps = 3
    ms = time_steps(lambda: mesh.mesh_sdf(rec, pts), reps, flush, stream) / reps
    pairs = n * F.shape[0]
    return {"workload": f"compute_sdf: {n} points x {F.shape[0]} triangles (icosphere, 5 subdivisions)",
            "ms": ms, "points_per_s": n / (ms / 1e3), "point_triangle_tests_per_s": pairs / (ms / 1e3)}


class _TorchOpsOctreeSDF(torch.nn.Module):
    """The reference's OctreeSDF computation written with stock PyTorch
    operators (F.grid_sample on channel-first volumes, nn.Linear, autograd),
    run on the GPU as the plain-FP32 training comparison
    (sdf-net/lib/models/OctreeSDF.py:38-155).  Same initial weights as ours."""

    def __init__(self, net):
        super().__init__()
        self.fms = torch.nn.ParameterList([torch.nn.Parameter(fv.fm.detach().contiguous().clone())
                                           for fv in net.features])
        self.louts = torch.nn.ModuleList()
        for d in net.louts:
            seq = torch.nn.Sequential(torch.nn.Linear(35, 128), torch.nn.ReLU(), torch.nn.Linear(128, 1))
            seq.load_state_dict(d.state_dict())
            self.louts.append(seq)

    def sdf(self, x, lod):
        import torch.nn.functional as F
        n = x.shape[0]
        acc = None
        for i in range(lod + 1):
            smp = F.grid_sample(self.fms[i], x.reshape(1, n, 1, 1, 3), align_corners=True,
                                padding_mode="border")[0, :, :, 0, 0].transpose(0, 1)
            acc = smp if acc is None else smp + acc
            d = self.louts[i](torch.cat([x, acc], dim=-1))
            if i == lod:
                return d


def bench_train(dev, flush, stream, batch=524_288, steps=20, warm=3, train_steps=2000):
    """Training step of Trainer.step_geometry (L2 over all 5 LODs, Adam 1e-3)
    on a 524,288-point batch of the 16-sphere union (seed 1): ours (fused
    forward over every LOD, hand-written backward, FusedAdam) against the
    reference's computation in stock PyTorch operators on the same GPU.
    Then 2,000 training steps from seed 1 and the BF16 form's difference to
    the float32 drop-in per LOD on the trained weights."""
    import nglod_gb300 as ng
    from nglod_gb300 import synthetic, trainer
    from nglod_gb300.bf16 import Bf16OctreeSDF
    from nglod_gb300.options import default_args
    c, r = synthetic.sphere_union(1)
    x, g = synthetic.training_batch(batch, c, r, seed=0)
    x, g = x.to(dev), g.to(dev)
    torch.manual_seed(1)
    net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2)).to(dev).train()
    ref = _TorchOpsOctreeSDF(net).to(dev)
    opt = trainer.FusedAdam(net.parameters(), lr=1e-3)
    ropt = torch.optim.Adam(ref.parameters(), lr=1e-3)

    def ours():
        trainer.step_geometry(net, opt, x, g)

    def theirs():
        ropt.zero_grad()
        loss = 0
        for lod in range(5):
            loss = loss + ((ref.sdf(x, lod) - g) ** 2).sum()
        (loss / batch).backward()
        ropt.step()

    for _ in range(warm):
        ours()
        theirs()
    torch.cuda.synchronize()
    ms_ours = time_steps(ours, steps, flush, stream) / steps
    ms_ref = time_steps(theirs, max(3, steps // 4), flush, stream) / max(3, steps // 4)
    out = {"workload": "Trainer.step_geometry, batch 524,288 (1/3 uniform, 2/3 surface + N(0, 0.01^2)), "
                       "L2 over LOD 0..4, Adam lr 1e-3",
           "ours_ms_per_step": ms_ours, "ours_points_per_s": batch / (ms_ours / 1e3),
           "torch_ops_ms_per_step": ms_ref, "torch_ops_points_per_s": batch / (ms_ref / 1e3),
           "speedup_vs_torch_ops": ms_ref / ms_ours,
           "gradient_check": "tests/test_train_gpu.py: 1e-4 relative vs reference autograd, 1e-3 vs FP64 differences"}
    if train_steps == 0:
        return out
    # 2,000 steps of configuration 2 from seed 1 (fresh batches every step)
    torch.manual_seed(1)
    net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2)).to(dev).train()
    t0 = time.perf_counter()
    pool = [synthetic.training_batch(batch, c, r, seed=100 + k) for k in range(8)]
    pool = [(a.to(dev), b.to(dev)) for a, b in pool]
    _, losses = trainer.fit(net, pool, train_steps, lr=1e-3, seed=5)
    torch.cuda.synchronize()
    out["train_2000_steps_s"] = time.perf_counter() - t0
    out["train_loss_trace"] = losses
    net.eval()
    bnet = Bf16OctreeSDF(net)
    q = synthetic.near_surface_query(4_194_304, c, r, seed=1).to(dev)
    errs = {}
    with torch.no_grad():
        for lod in range(5):
            d = (bnet.sdf(q, lod=lod) - net.sdf(q, lod=lod)).abs()
            errs[lod] = {"max": float(d.max().item()), "mean": float(d.mean().item())}
    out["trained_bf16_vs_f32_per_lod"] = errs
    gt = synthetic.sphere_union_sdf(q[:262144].double(), c, r).float()[:, None]
    with torch.no_grad():
        out["trained_f32_l1_vs_analytic_lod4"] = float((net.sdf(q[:262144], lod=4) - gt).abs().mean().item())
    return out


def bench_sparse(net, dev, flush, stream, level=7, lod=4, steps=64):
    """Sparse path (sol-renderer): SPC octree of level 7 built on the GPU from
    the voxels whose centres lie within one voxel diagonal of the 16-sphere
    surface (seed 1); per frame: ray/octree traversal to level lod+2 = 6,
    first-nugget flags, sparse sphere trace (64 steps) with BF16 corner
    features and the tensor-core BF16 decoder, 1920x1080 (the same frame
    with the float32 decoder beside it).  Depth/normal maps against the
    dense float32 tracer on the same network."""
    import nglod_gb300 as ng
    from nglod_gb300 import spc, synthetic
    from nglod_gb300.options import default_args
    from nglod_gb300.sparse_sdf import SparseSDF
    c, r = synthetic.sphere_union(1)
    res = 2 ** level
    idx = torch.stack(torch.meshgrid(torch.arange(res), torch.arange(res), torch.arange(res), indexing="ij"), -1)
    idx = idx.reshape(-1, 3).to(dev)
    centres = (idx.double() + 0.5) / res * 2 - 1
    keep = synthetic.sphere_union_sdf(centres, c, r).abs() <= (3 ** 0.5) * (2.0 / res)
    vox = idx[keep].int()
    t0 = time.perf_counter()
    s = spc.SPC.from_voxels(vox, level)
    sp = SparseSDF.from_dense(net, s, precision="bf16")  # tensor-core decoder
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    sp32 = SparseSDF.from_dense(net, s, precision="bf16", decoder="f32")
    ro, rd = synthetic.look_at_rays(width=TRACE_W, height=TRACE_H)
    ro, rd = ro.to(dev), rd.to(dev)

    def frame():
        return sp.render(ro, rd, lod=lod, num_steps=steps)

    for _ in range(3):
        (x, t, hit, normal), nug = frame()
    torch.cuda.synchronize()
    reps = 10
    ms = time_steps(frame, reps, flush, stream) / reps
    ms_trav = time_steps(lambda: spc.spc_raytrace(s.GetOctree(), s.GetPoints(), s.GetPyramid(), ro, rd, lod + 2,
                                                   prefix=s.GetPrefix()), reps, flush, stream) / reps
    sp.check_status()
    sp32.render(ro, rd, lod=lod, num_steps=steps)
    ms32 = time_steps(lambda: sp32.render(ro, rd, lod=lod, num_steps=steps), reps, flush, stream) / reps
    # LOD-summed corner features: one voxel's corners per query
    sps = SparseSDF.from_dense(net, s, precision="bf16", summed=True)
    for _ in range(3):
        (_, ts, hits, _), _ = sps.render(ro, rd, lod=lod, num_steps=steps)
    torch.cuda.synchronize()
    ms_sum = time_steps(lambda: sps.render(ro, rd, lod=lod, num_steps=steps), reps, flush, stream) / reps
    sps.check_status()
    net.lod = lod
    rb = ng.SphereTracer(default_args(num_steps=128))(net, ro, rd)
    net.lod = None
    both = hit & rb.hit
    cosang = (normal[both] * rb.normal[both]).sum(-1)
    return {"workload": f"octree level {level} ({int(s.GetPyramid()[0, level])} leaf voxels, {s.GetOSize()} bytes), "
                        f"frame {TRACE_W}x{TRACE_H}: traversal to level {lod + 2}, sparse trace lod {lod}, "
                        f"{steps} steps, bf16 corner features, tcgen05 bf16 decoder",
            "frame_ms": ms, "rays_per_s": TRACE_W * TRACE_H / (ms / 1e3), "traversal_ms": ms_trav,
            "frame_ms_f32_decoder": ms32,
            "frame_ms_summed": ms_sum,
            "summed_hit_agreement": float((hits == hit).float().mean().item()),
            "nuggets": int(nug.shape[0]), "setup_s": setup_s,
            "vs_dense_f32": {"hit_agreement": float((hit == rb.hit).float().mean().item()),
                             "depth_median_abs": float((t[both] - rb.depth[both]).abs().median().item()),
                             "normal_cos_median": float(cosang.median().item())}}


def bench_serve(dev, duration_s=6.0, rate_hz=200.0, num_models=8):
    """Serving: 8 resident BF16 models (the 16-sphere unions of seeds 2..9 held
    through analytic_init), a seeded Poisson stream at 200 req/s of renders
    (256^2, 512^2, 1280x720, 1920x1080, LOD 0-4) and point queries (1e4-1e6
    points), admitted by the native scheduler (nglod_serve_*) under a 16 GiB
    HBM budget on 8 slots."""
    import nglod_gb300 as ng
    from nglod_gb300 import serve, synthetic
    from nglod_gb300.analytic_init import init_from_sdf
    from nglod_gb300.bf16 import Bf16OctreeSDF
    from nglod_gb300.options import default_args
    models = []
    for seed in range(2, 2 + num_models):
        c, r = synthetic.sphere_union(seed)
        torch.manual_seed(seed)
        net = ng.OctreeSDF(default_args(num_lods=5, base_lod=2))
        init_from_sdf(net, lambda p, c=c, r=r: torch.from_numpy(synthetic.sphere_union_sdf(p.numpy(), c, r)),
                      noise=1e-3, seed=seed)
        models.append(Bf16OctreeSDF(net.to(dev).eval()))
    ex = serve.CudaExecutor(models, dev, num_streams=8)
    gen = torch.Generator(device=dev)

    def pts(spec):
        gen.manual_seed(spec["seed"])
        return torch.rand(spec["n"], 3, device=dev, generator=gen) * 2 - 1

    warm = serve.Server(ex, 16 << 30)
    serve.run_workload(warm, serve.poisson_workload(0.5, rate_hz, num_models, seed=99), pts)
    warm.close()
    torch.cuda.synchronize()
    srv = serve.Server(ex, 16 << 30)
    wl = serve.poisson_workload(duration_s, rate_hz, num_models, seed=7)
    st = serve.run_workload(srv, wl, pts)
    srv.close()
    st["workload"] = (f"{len(wl)} requests, Poisson {rate_hz:.0f}/s for {duration_s:.0f} s, 8 resident BF16 models; "
                      "renders 256^2/512^2/1280x720/1920x1080 at LOD 0-4, 64 steps; queries 1e4-1e6 points")
    return st


def cpu_baseline(net):
    """The reference's CPU torch computation (oracle/torch_port.py) on a bounded sample."""
    from nglod_gb300 import synthetic
    from oracle import torch_port
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    ref = torch_port.RefOctreeSDF({k: v.cpu() for k, v in net.state_dict().items()}, 5)
    c, r = synthetic.sphere_union(1)
    x = synthetic.near_surface_query(CPU_SAMPLE, c, r, seed=1)
    with torch.no_grad():
        ref.sdf(x[:4096], lod=LOD)
        times = []
        for _ in range(3):
            t0 = time.perf_counter()
            ref.sdf(x, lod=LOD)
            times.append(time.perf_counter() - t0)
    med = statistics.median(times)
    return {"value": CPU_SAMPLE / med, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{CPU_SAMPLE} points of the same workload, median of 3 passes, torch CPU ops "
                      f"(grid_sample/linear) as in OctreeSDF.sdf"}


def run_reference(args):
    ws, rank, _ = dist_setup()
    if rank != 0:
        return
    from nglod_gb300 import synthetic
    from oracle import torch_port
    threads = os.cpu_count() or 1
    torch.set_num_threads(threads)
    net, (c, r) = build_model(None)
    ref = torch_port.RefOctreeSDF({k: v.cpu() for k, v in net.state_dict().items()}, 5)
    x = synthetic.near_surface_query(CPU_SAMPLE, c, r, seed=1)
    warm = max(1, min(args.warmup, 2))  # bounded: each step is a 262k-point CPU sample
    with torch.no_grad():
        for _ in range(warm):
            ref.sdf(x, lod=LOD)
        steps = max(1, min(args.steps, 5))
        t0 = time.perf_counter()
        for _ in range(steps):
            ref.sdf(x, lod=LOD)
        dt = time.perf_counter() - t0
    value = CPU_SAMPLE * steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0, "steps": steps,
        "warmup": warm, "requested": {"steps": args.steps, "warmup": args.warmup}, "ms_per_step": dt / steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "points": N_POINTS, "lod": LOD,
                   "sample_points_per_step": CPU_SAMPLE, "parallelism": "host cores"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{CPU_SAMPLE} points per step of the same workload; the reference's torch "
                                   f"CPU operators (oracle/torch_port.py)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_only(args):
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    import nglod_gb300 as ng
    from nglod_gb300.bf16 import Bf16OctreeSDF
    ng.load_library()
    net, _ = build_model(dev)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    if args.only == "trace":
        out = bench_trace(net, Bf16OctreeSDF(net), dev, flush, stream)
    elif args.only == "aabb":
        out = bench_aabb(dev, flush, stream)
    elif args.only == "summed":
        from nglod_gb300 import synthetic
        x = synthetic.near_surface_query(N_POINTS, *synthetic.sphere_union(1), seed=1).to(dev)
        bnet = Bf16OctreeSDF(net)
        for _ in range(3):
            bnet.sdf(x, lod=LOD)
        torch.cuda.synchronize()
        k = min(max(args.steps, 1), 100)
        per_lod_ms = time_steps(lambda: bnet.sdf(x, lod=LOD), k, flush, stream) / k
        out = {"per_lod_bf16_ms": per_lod_ms, **bench_summed(net, bnet, x, dev, flush, stream, steps=k)}
    elif args.only == "train":
        out = bench_train(dev, flush, stream, steps=max(args.steps, 1), warm=max(args.warmup, 1), train_steps=0)
    elif args.only == "sparse":
        out = bench_sparse(net, dev, flush, stream)
    elif args.only == "shade":
        out = bench_shade(net, Bf16OctreeSDF(net), dev, flush, stream)
    elif args.only == "mesh":
        out = bench_mesh(dev, flush, stream)
    else:
        out = bench_serve(dev, duration_s=2.0)
    print(json.dumps({"only": args.only, **out}), flush=True)


def main():
    args = parse()
    if args.only:
        run_only(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

#!/usr/bin/env python
"""Benchmark of the BM4D-OF two-step video denoiser on GB300.

Metric: megapixel-frames per second (W*H*F / 1e6 per second) of the plain
two-step method (runNlBayes, both steps) on the headline workload: 1920x1080,
60 frames, grey, sigma = 20, patches 4x4x4, 16 similar patches, 21x21 search
window, +-4 frames along the flow (seeded synthetic video, exact flow).

  value  -- inputs already resident in HBM (CUDA tensors handed to the C ABI),
            device time of the whole call from CUDA events on the library's
            stream;
  e2e    -- the same call with pinned host buffers: the host->device copy of
            noisy + flows and the device->host copy of basic + final are inside
            the timed region.

One step = one full runNlBayes over the workload.  Inputs (2.5 GB) are larger
than the 129 MB L2, so no flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload hd|c2]

--impl reference times the reference algorithm on the host cores (the CPU
oracle restatement of the reference's code, OpenMP over the reference's tiles,
all host threads) on a bounded crop of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(ROOT, "bm4d-of_gb300"), os.path.join(ROOT, "tests"), os.path.join(ROOT, "oracle")]

import numpy as np  # noqa: E402

WORKLOADS = {
    # name: (W, H, F, sigma, seed)
    "hd": (1920, 1080, 60, 20.0, 5),
    "c2": (854, 480, 20, 20.0, 2),
    "small": (480, 272, 12, 20.0, 3),   # profiling case (about 1 GB on the device)
}
CLI = dict(px1=4, px2=4, pt1=4, pt2=4, wx1=21, wx2=21, np1=16, np2=16, b1=3.0)
METRIC = "megapixel-frames/s at 1 GPU, plain vs learned/mixed at ≤0.05 dB PSNR loss"
UNIT = "MPF/s"
# ncu dram__bytes_read + dram__bytes_write of one step-1 search_kernel launch on
# 480x272x12 (one --set full capture of the small workload)
SEARCH_TRAFFIC_SMALL = 12.04e6 + 7.60e6
# CPU sample (crop of the same workload) for the host-core baseline: 12
# frames, so that every reference patch has the full 9-frame search range it
# has in the long video
CPU_SAMPLE = (480, 272, 12)


def resolve(lib, W, H, F, sigma):
    from helpers import resolve_params
    return resolve_params(lib, (W, H, F, 1), sigma, **CLI)


def workload(name):
    import synthetic
    W, H, F, sigma, seed = WORKLOADS[name]
    clean, ff, bf = synthetic.video(W, H, F, seed)
    nz = synthetic.noisy(clean, sigma, seed)
    return clean, nz, ff, bf


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in self.rows:
            for i, n in enumerate(names):
                if len(r) > 5 + i and r[5 + i].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_max_ms(ms, world):
    """The slowest rank's time: every rank is an independent replica of the
    whole workload (no data exchange), so the job takes as long as its slowest
    replica.  The reduction runs on the process group's own device (CUDA
    tensors for NCCL, host tensors for gloo)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def plan_groups(W, H, F, p, nparts):
    """Reference patches (groups) of one step over all tiles of a run, counted
    on the host without the GPU library: the tiles of subDivideTight
    (lib_videot.hpp:853-916, grid from determineFactor, utilities.cpp:137-158)
    and the reference grid of processNlBayes (nldct.cpp:520-553).
    tests/test_bench_baseline.py checks it against bm4dof_plan."""
    if nparts == 1:
        nw, nh = 1, 1
    else:
        nh = 2
        while nparts % nh:
            nh += 1
        nw = nparts // nh
        if nh > nw:
            nw, nh = nh, nparts // nh
    wt = int(np.ceil(np.float32(W) / np.float32(nw)))
    ht = int(np.ceil(np.float32(H) / np.float32(nh)))
    N, px, pt, wx = p.boundary, p.sizePatch, p.sizePatchTime, p.sizeSearchWindow

    def count(ori, end, step, b0, b1):
        return sum(1 for v in range(ori, end)
                   if (v - ori) % step == 0 or (not b1 and v == end - 1) or (not b0 and v == ori))

    nf = count(0, F - (pt - 1), p.offSetTime, False, False)
    total = 0
    for j in range(nh):
        for i in range(nw):
            ox, ex = max(0, i * wt - N), min(W, (i + 1) * wt + N)
            oy, ey = max(0, j * ht - N), min(H, (j + 1) * ht + N)
            bx0, bx1, by0, by1 = ox > 0, ex < W, oy > 0, ey < H
            half = px - 1 + wx // 2
            nx = count(half if bx0 else 0, (ex - ox) - (half if bx1 else px - 1), p.offSet, bx0, bx1)
            ny = count(half if by0 else 0, (ey - oy) - (half if by1 else px - 1), p.offSet, by0, by1)
            total += nx * ny * nf
    return total


def cpu_baseline(nz, ff, bf, sigma, threads=None, sample=CPU_SAMPLE):
    """The reference algorithm on the host cores (oracle restatement, OpenMP over
    the reference's 2*threads tiles) on a crop of the workload, scaled to the
    whole workload by groups.

    The reference's work is proportional to the groups it processes: every
    group searches the same 21x21x9 candidates (12 sample frames give every
    group the full temporal range) and filters and aggregates the same patch
    group, whatever tile it lies in.  The crop's tiles are small, so it
    processes more groups per pixel (tile halos) than the whole video would,
    and its few tiles balance unevenly over the threads.  So the CPU time of
    all threads (user + system) per processed group is measured on the crop
    (about 2 % apart between a 160x136 and a 480x272 crop, where wall-clock
    time per group differed by 11 %), and the whole video's time is that
    per-group cost times the groups the reference processes on it with the
    same thread count (2*threads tiles of the full frame), divided evenly over
    the threads: a perfectly balanced run, which no real run beats."""
    import pyoracle
    pyoracle.build()
    O = pyoracle.Oracle()
    threads = threads or os.cpu_count() or 1
    W, H, F = sample
    crop = lambda v: np.ascontiguousarray(v[:F, :, :H, :W])
    p1, p2 = resolve(O, W, H, F, sigma)
    c0 = os.times()
    t = time.perf_counter()
    O.runNlBayes(crop(nz), crop(ff), crop(bf), p1, p2, nparts=2 * threads, nthreads=threads)
    dt = time.perf_counter() - t
    c1 = os.times()
    cpu_s = (c1.user - c0.user) + (c1.system - c0.system)
    FW, FH, FF = nz.shape[3], nz.shape[2], nz.shape[0]
    g_sample = plan_groups(W, H, F, p1, 2 * threads) + plan_groups(W, H, F, p2, 2 * threads)
    r1, r2 = resolve(O, FW, FH, FF, sigma)
    g_full = plan_groups(FW, FH, FF, r1, 2 * threads) + plan_groups(FW, FH, FF, r2, 2 * threads)
    full_s = cpu_s / g_sample * g_full / threads
    return {"value": FW * FH * FF / 1e6 / full_s, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{W}x{H}x{F} crop of the same workload, both steps, {2 * threads} tiles on {threads} threads: "
                      f"{dt:.1f} s wall, {cpu_s:.0f} CPU-s for {g_sample} groups ({cpu_s / g_sample * 1e6:.0f} "
                      f"CPU-us per group); {FW}x{FH}x{FF} at {2 * threads} tiles has {g_full} groups: "
                      f"{full_s:.0f} s on {threads} threads, perfectly balanced",
            "sample_value": W * H * F / 1e6 / dt, "cpu_us_per_group": cpu_s / g_sample * 1e6,
            "groups_sample": g_sample, "groups_full": g_full}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return 0
    W, H, F, sigma, seed = WORKLOADS[args.workload]
    _, nz, ff, bf = workload(args.workload)
    samples = []
    for _ in range(args.warmup):
        cpu_baseline(nz, ff, bf, sigma)
    for _ in range(args.steps):
        samples.append(cpu_baseline(nz, ff, bf, sigma))
    v = statistics.median(s["value"] for s in samples)
    cb = dict(samples[0])
    cb["value"] = v
    cfg = config(args)
    sw, sh, sf = CPU_SAMPLE
    cfg["workload"] = (f"reference algorithm (oracle restatement) on {cb['cores']} host cores: "
                       f"{sw}x{sh}x{sf} crop of the grey video {W}x{H}x{F} (sigma {sigma:g}, plain two-step FP32), "
                       f"{2 * cb['cores']} tiles, timed; its CPU time per group applied to the {W}x{H}x{F} "
                       f"video's groups at {2 * cb['cores']} tiles, spread evenly over the cores")
    cfg["timed_sample"] = {"W": sw, "H": sh, "frames": sf, "tiles": 2 * cb["cores"]}
    cfg["tiles"] = 2 * cb["cores"]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": cfg, "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


SIGMAS = (5.0, 10.0, 20.0, 30.0, 40.0, 50.0)


def batch_specs(n, seed=4):
    """Uneven batch: widths in [320, 1920], heights in [240, 1080] (multiples of
    8), 5..30 frames, sigma from {5, 10, 20, 30, 40, 50}, each sequence with its
    own seed."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        W = int(rng.integers(40, 241)) * 8
        H = int(rng.integers(30, 136)) * 8
        F = int(rng.integers(5, 31))
        out.append((W, H, F, float(rng.choice(SIGMAS)), 1000 * seed + i))
    return out


def run_batch(args):
    """Many sequences in one CUDA graph (bm4dof_run_batched), tuned by the
    library's autotuner on a sample of the batch."""
    import torch
    import bm4dof
    import synthetic
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    ctx = bm4dof.Context(local)
    specs = batch_specs(args.batch_n)
    items, host = [], []
    for (W, H, F, sigma, seed) in specs:
        clean, ff, bf = synthetic.video(W, H, F, seed)
        nz = synthetic.noisy(clean, sigma, seed)
        p1, p2 = resolve(bm4dof, W, H, F, sigma)
        h = [torch.from_numpy(a).pin_memory() for a in (nz, ff, bf)]
        d = [t.cuda() for t in h]
        items.append({"noisy": d[0], "fflow": d[1], "bflow": d[2], "basic": torch.empty_like(d[0]),
                      "final": torch.empty_like(d[0]), "p1": p1, "p2": p2, "nparts": args.nparts})
        host.append(h + [torch.empty_like(h[0]).pin_memory()])
    mpf = sum(W * H * F for (W, H, F, _, _) in specs) / 1e6
    best, table = ctx.autotune(items, sample=min(8, len(items)))
    for _ in range(max(args.warmup, 3)):
        ctx.run_batched(items, tuning=best)
    tms = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            ctx.run_batched(items, tuning=best)
            tms.append(ctx.timings()[0][4])
    ms_step = statistics.mean(tms)
    launches = ctx.timings()[1]
    # per-sequence agreement with the unbatched plain path (the smallest four)
    order = sorted(range(len(specs)), key=lambda i: specs[i][0] * specs[i][1] * specs[i][2])[:4]
    agree = 0
    for i in order:
        it = items[i]
        _, f, _ = ctx.runNlBayes(it["noisy"], it["fflow"], it["bflow"], it["p1"], it["p2"], nparts=args.nparts)
        agree += bool(torch.equal(f, it["final"]))
    # end to end: host inputs copied in and finals copied out inside the timed region
    e2e = []
    h2d = sum(sum(t.numel() * 4 for t in h[:3]) for h in host)
    d2h = sum(h[3].numel() * 4 for h in host)
    for _ in range(args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for it, h in zip(items, host):
            it["noisy"].copy_(h[0], non_blocking=True)
            it["fflow"].copy_(h[1], non_blocking=True)
            it["bflow"].copy_(h[2], non_blocking=True)
        torch.cuda.synchronize()
        ctx.run_batched(items, tuning=best)
        for it, h in zip(items, host):
            h[3].copy_(it["final"], non_blocking=True)
        torch.cuda.synchronize()
        e2e.append(time.perf_counter() - t0)
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": world * mpf / (ms_step / 1e3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (per-sequence seeded cosine+rectangle texture, motion, exact flow, AWGN)",
        "config": {"workload": f"batch of {len(specs)} grey sequences, W in [320,1920], H in [240,1080], "
                               f"5..30 frames, sigma in {{5..50}}, plain two-step FP32, one CUDA graph",
                   "sequences": len(specs), "megapixel_frames": mpf, "tuning": best,
                   "autotune": [list(r) for r in table], "parallelism": f"replicas x{world}"},
        "roofline": None,
        "e2e": {"value": world * mpf / statistics.mean(e2e), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches, "clocks": clk.summary(),
        "agreement_with_unbatched": f"{agree}/{len(order)} sequences bit-identical",
    }
    print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def config(args):
    W, H, F, sigma, seed = WORKLOADS[args.workload]
    mb = W * H * F * 4 * 5 / 1e6   # noisy + two 2-channel flows
    return {"workload": f"grey video {W}x{H}x{F}, sigma {sigma:g}, plain two-step FP32",
            "W": W, "H": H, "frames": F, "sigma": sigma, "seed": seed, "patch": "4x4x4",
            "n_similar": 16, "search": "21x21, +-4 frames along the flow", "tiles": args.nparts,
            "l2": f"inputs {mb:.0f} MB > 129 MB L2 (no flush)" if mb > 129 else f"inputs {mb:.0f} MB",
            "parallelism": f"replicas x{args.gpus}"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hd", choices=sorted(WORKLOADS) + ["batch"])
    ap.add_argument("--batch-n", type=int, default=64, help="sequences of the batch workload")
    ap.add_argument("--nparts", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true", help="skip the host-core baseline")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)

    import torch
    import bm4dof
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    W, H, F, sigma, seed = WORKLOADS[args.workload]
    clean, nz, ff, bf = workload(args.workload)
    ctx = bm4dof.Context(local)
    p1, p2 = resolve(bm4dof, W, H, F, sigma)

    # device-resident inputs and outputs
    d_nz, d_ff, d_bf = (torch.from_numpy(a).cuda() for a in (nz, ff, bf))
    d_basic, d_final = torch.empty_like(d_nz), torch.empty_like(d_nz)
    # pinned host buffers for the end-to-end measurement
    h_nz, h_ff, h_bf = (torch.from_numpy(a).pin_memory() for a in (nz, ff, bf))
    h_basic, h_final = torch.empty_like(h_nz).pin_memory(), torch.empty_like(h_nz).pin_memory()

    def step_device():
        ctx.runNlBayes(d_nz, d_ff, d_bf, p1, p2, basic=d_basic, final=d_final, nparts=args.nparts)
        return ctx.timings()

    def step_host():
        ctx.runNlBayes(h_nz.numpy(), h_ff.numpy(), h_bf.numpy(), p1, p2, basic=h_basic.numpy(),
                       final=h_final.numpy(), nparts=args.nparts)
        return ctx.timings()

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(max(args.warmup, 3)):
        step_device()
    barrier()
    totals, searches, launches = [], [], 0
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            ms, n = step_device()
            totals.append(ms[4])
            searches.append(ms[0])
            launches += n
        barrier()
        wall = time.perf_counter() - t0
    dev_ms = replica_max_ms(sum(totals), world)
    ms_step = dev_ms / args.steps
    mpf = W * H * F / 1e6
    value = world * mpf / (ms_step / 1e3)
    _, _, ratios = ctx.runNlBayes(d_nz, d_ff, d_bf, p1, p2, basic=d_basic, final=d_final, nparts=args.nparts)
    stage_ms, _ = ctx.timings()

    # end to end through the C ABI with pinned host buffers
    step_host()
    barrier()
    e2e_ms = []
    for _ in range(args.steps):
        ms, _ = step_host()
        e2e_ms.append(ms[4])
    barrier()
    e2e_stage = ms
    e2e_value = world * mpf / (replica_max_ms(statistics.mean(e2e_ms), world) / 1e3)

    if rank != 0:
        return 0
    # roofline of the dominant kernel (patch search): algorithmic FP32
    # operations (one subtract, one multiply, one add per patch element per
    # candidate) over the measured launch duration
    whf = W * H * F
    groups = [round(r * whf / 100.0) for r in ratios]
    ncand = 21 * 21 * 9
    flops_per_launch = statistics.mean(g * 3 * 64 * ncand for g in groups)
    launch_ms = statistics.mean(searches) / 2.0
    achieved = flops_per_launch / (launch_ms / 1e3) / 1e12
    # the search's instruction mix timed alone on this GPU (registers only,
    # packed subtract and multiply, scalar adds): the rate it could reach
    peak, mix_ms = bm4dof.fp32_mix_rate(local)
    nominal = 152 * 128 * 2.07e9 / 1e12
    psnr = lambda a, b: float(10 * np.log10(255.0 ** 2 / np.mean((a.astype(np.float64) - b) ** 2)))
    final_np = d_final.cpu().numpy()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded cosine+rectangle texture, global translation + moving rectangles, exact flow, AWGN)",
        "config": config(args),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak,
                     # DRAM bytes per launch: ncu capture of the 480x272x12 step-1 launch
                     # (12.04 MB read + 7.60 MB written), scaled by the pixel count
                     "traffic": SEARCH_TRAFFIC_SMALL * (W * H * F) / (480 * 272 * 12),
                     "traffic_source": "ncu dram__bytes_read+write of search_kernel on 480x272x12, "
                                       "scaled by pixels (the frames and flows, read about once)",
                     "kernel": "search_kernel",
                     "peak_source": "measured on this GPU by bm4dof_fp32_mix_rate: the exact search's FP32 "
                                    "instruction mix (packed sub/mul.rn.f32x2 + scalar adds) from registers, "
                                    "3 ops per element (MEASURED_PEAKS.json has HBM and bf16 tensor peaks only)",
                     "nominal_fp32_tops": nominal, "frac_of_nominal": achieved / nominal},
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(nz.nbytes + ff.nbytes + bf.nbytes),
                "d2h_bytes_per_step": int(2 * nz.nbytes),
                "stage_ms": {"search": e2e_stage[0], "filter": e2e_stage[1], "aggregation": e2e_stage[2],
                             "other": e2e_stage[3], "total": e2e_stage[4]}},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "stage_ms": {"search": stage_ms[0], "filter": stage_ms[1], "aggregation": stage_ms[2],
                     "other": stage_ms[3], "total": stage_ms[4]},
        "groups": groups,
        "quality_db": {"noisy": psnr(nz, clean), "final": psnr(final_np, clean)},
        "wall_s_timed": wall,
    }
    # the faster forms of the same workload, timed the same way, with their
    # PSNR loss against the plain method
    forms = {}
    import train_gains
    gains = train_gains.load_weights()
    variants = [("mixed", {"mixed": True}), ("mixed_certified", {"mixed": "certified"}),
                ("vbm3d_search", {"vbm3d": True}), ("paste_boost", {})]
    if gains is not None:
        ctx.set_gain_network(gains)
        variants += [("learned", {"learned": True}), ("learned+mixed", {"learned": True, "mixed": True})]
    import copy
    q1, q2 = copy.copy(p1), copy.copy(p2)
    q1.doPasteBoost = q2.doPasteBoost = 1   # the reference's paste trick (nlbParams::doPasteBoost)
    for name, kw in variants:
        v1, v2 = (q1, q2) if name == "paste_boost" else (p1, p2)
        for _ in range(2):
            ctx.runNlBayes(d_nz, d_ff, d_bf, v1, v2, basic=d_basic, final=d_final, nparts=args.nparts, **kw)
        tms = []
        for _ in range(max(2, min(args.steps, 5))):   # a few timed runs per form keep the bench short
            ctx.runNlBayes(d_nz, d_ff, d_bf, v1, v2, basic=d_basic, final=d_final, nparts=args.nparts, **kw)
            ms, _ = ctx.timings()
            tms.append(ms[4])
        fq = psnr(d_final.cpu().numpy(), clean)
        forms[name] = {"value": world * mpf / (statistics.mean(tms) / 1e3), "unit": UNIT,
                       "ms_per_step": statistics.mean(tms), "speedup_vs_plain": ms_step / statistics.mean(tms),
                       "stage_ms": dict(zip(("search", "filter", "aggregation", "other", "total"),
                                            ctx.timings()[0])),
                       "psnr_db": fq, "psnr_loss_vs_plain_db": line["quality_db"]["final"] - fq}
        if kw.get("learned"):
            g, fb = ctx.learned_stats()
            forms[name]["fallback_groups"] = [fb, g]
        if kw.get("mixed"):
            g, ex, unc = ctx.mixed_stats()
            forms[name]["search_groups"] = {"tensor_core_prescreen": g, "exact_search": ex,
                                            "uncertified_rerank": unc}
    line["forms"] = forms
    # the step before the path: TV-L1 flows of the whole video (2(F-1) frame
    # pairs in one batch, tvl1flow-seq.sh parameters), host video in, flows out
    ctx.tvl1_video(nz)
    ctx.tvl1_video(nz)
    fms = ctx.timings()[0][4]
    line["flow"] = {"method": "TV-L1 (lib/tvl1flow), 2(F-1) pairs batched", "pairs": 2 * (F - 1), "ms": fms,
                    "pairs_per_s": 2 * (F - 1) / (fms / 1e3)}
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(nz, ff, bf, sigma)
    print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

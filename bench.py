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
# CPU sample (crop of the same workload) for the host-core baseline
CPU_SAMPLE = (480, 272, 13)


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


def cpu_baseline(nz, ff, bf, sigma, threads=None, sample=CPU_SAMPLE):
    """The reference algorithm on the host cores (oracle restatement, OpenMP over
    the reference's 2*threads tiles) on a crop of the workload."""
    import pyoracle
    pyoracle.build()
    O = pyoracle.Oracle()
    threads = threads or os.cpu_count() or 1
    W, H, F = sample
    crop = lambda v: np.ascontiguousarray(v[:F, :, :H, :W])
    p1, p2 = resolve(O, W, H, F, sigma)
    t = time.perf_counter()
    O.runNlBayes(crop(nz), crop(ff), crop(bf), p1, p2, nparts=2 * threads, nthreads=threads)
    dt = time.perf_counter() - t
    return {"value": W * H * F / 1e6 / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{W}x{H}x{F} crop of the same workload, both steps, {dt:.1f} s, "
                      f"{2 * threads} tiles"}


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
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": config(args), "cpu_baseline": cb,
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def config(args):
    W, H, F, sigma, seed = WORKLOADS[args.workload]
    return {"workload": f"grey video {W}x{H}x{F}, sigma {sigma:g}, plain two-step FP32",
            "W": W, "H": H, "frames": F, "sigma": sigma, "seed": seed, "patch": "4x4x4",
            "n_similar": 16, "search": "21x21, +-4 frames along the flow", "tiles": args.nparts,
            "l2": "inputs 2.5 GB > 129 MB L2 (no flush)", "parallelism": f"replicas x{args.gpus}"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="hd", choices=sorted(WORKLOADS))
    ap.add_argument("--nparts", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true", help="skip the host-core baseline")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

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
    dev_ms = sum(totals)
    if world > 1:
        t = torch.tensor([dev_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        dev_ms = float(t.item())
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
    e2e_value = world * mpf / (statistics.mean(e2e_ms) / 1e3)

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
    peak = 152 * 128 * 2.07e9 / 1e12
    psnr = lambda a, b: float(10 * np.log10(255.0 ** 2 / np.mean((a.astype(np.float64) - b) ** 2)))
    final_np = d_final.cpu().numpy()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded cosine+rectangle texture, global translation + moving rectangles, exact flow, AWGN)",
        "config": config(args),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "search_exact_kernel",
                     "peak_source": "nominal FP32 CUDA-core rate: 152 SMs x 128 lanes x 2.07 GHz "
                                    "(MEASURED_PEAKS.json has HBM and bf16 tensor peaks only)"},
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(nz.nbytes + ff.nbytes + bf.nbytes),
                "d2h_bytes_per_step": int(2 * nz.nbytes)},
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
    for name, kw in (("mixed", {"mixed": True}),):
        for _ in range(2):
            ctx.runNlBayes(d_nz, d_ff, d_bf, p1, p2, basic=d_basic, final=d_final, nparts=args.nparts, **kw)
        tms = []
        for _ in range(args.steps):
            ctx.runNlBayes(d_nz, d_ff, d_bf, p1, p2, basic=d_basic, final=d_final, nparts=args.nparts, **kw)
            ms, _ = ctx.timings()
            tms.append(ms[4])
        fq = psnr(d_final.cpu().numpy(), clean)
        forms[name] = {"value": world * mpf / (statistics.mean(tms) / 1e3), "unit": UNIT,
                       "ms_per_step": statistics.mean(tms), "stage_ms": dict(zip(
                           ("search", "filter", "aggregation", "other", "total"), ctx.timings()[0])),
                       "psnr_db": fq, "psnr_loss_vs_plain_db": line["quality_db"]["final"] - fq}
    line["forms"] = forms
    if not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(nz, ff, bf, sigma)
    print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

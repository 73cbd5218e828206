#!/usr/bin/env python
"""Benchmark: the plain neighbourhood-filter suite on one 1024x1024x256 uint16
stack (seeded blob generator, 20k blobs) and its uint8 mask (> 400).

One step runs every filter of the suite once, each as its own call:
  gaussian_blur sigma (3,3,1.5) -> f32      mean/minimum/maximum r (5,5,2) -> u16
  median_box 3x3x3 -> u16                   median_sphere r=2 -> u16
  sobel_3d -> f32                           erode/dilate_sphere r=1 and r=2 on the mask
value = voxels filtered per second over the whole suite (Gvoxel/s);
per_filter gives each filter's Gvoxel/s and fraction of the measured HBM
peak (algorithmic bytes = sizeof(src) + sizeof(dst) per voxel).

The same line carries the other workloads of the benchmark, each with its
own clocks and roofline fraction (single-GPU runs):
  config1  plain gaussian sigma (2,2,1) on a 256x256x64 uint16 stack to f32,
           beside the reference kernels on the host cores on the same stack;
  batch    the top-hat chain over 512 uneven images: batched (one graph
           launch) against per-image plain calls and per-kernel launches;
  serve    Poisson-arrival requests at 200/1000/5000 req/s, served with
           continuous admission against one slot, p50/p99 latency, plus a
           closed-loop saturation run;
  large    large-halo filters on a 2048x2048x400 float32 stack.

  python bench.py [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference kernels on the host cores (oracle/_ref:
the reference's .cl compiled as C++, else the oracle restatement) on a
bounded sample of the same workload (a full-width 1024x1024x32 slab of the
stack) and on the whole 256x256x64 stack of config1.  Under torchrun each
rank runs an independent replica (the path shards by stack; no collective).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for p in (ROOT, ROOT / "clij-opencl-kernels_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))

SHAPE = (256, 1024, 1024)  # (z, y, x)
N_BLOBS = 20000
SEED = 2
SAMPLE = (32, 1024, 1024)  # CPU-baseline sample: a full-width z-slab of the same stack
METRIC = "Gvoxel/s (plain filter suite, 1024x1024x256)"
CONFIG1_SHAPE, CONFIG1_BLOBS, CONFIG1_SEED = (64, 256, 256), 200, 1
L2_FLUSH_BYTES = 512 << 20  # written between timed calls whose data fits in L2 (129 MB)


# DRAM bytes per voxel (read + write) of each filter's kernel from the ncu
# launch list (dram__bytes_read.sum + dram__bytes_write.sum) of the build
# named in TRAFFIC_SOURCE, on a 1024x1024x128 slab of the same stack (traffic
# scales with the voxels).
TRAFFIC_SOURCE = "ncu launch list of commit 4b4376a, 1024x1024x128 slab, scaled to the stack"
NCU_DRAM_BYTES_PER_VOXEL = {
    "gaussian_blur s(3,3,1.5)": 5.76, "mean_box r(5,5,2)": 3.72, "minimum_box r(5,5,2)": 3.70,
    "maximum_box r(5,5,2)": 3.71, "median_box r1": 3.71, "median_sphere r2": 3.70, "sobel_3d": 5.64,
    "erode_sphere r1": 1.70, "erode_sphere r2": 1.78, "dilate_sphere r1": 1.71, "dilate_sphere r2": 1.78,
}
# The selection networks are bound by the min/max (ALU) pipe, not by DRAM:
# its busy fraction from the one-kernel capture of the same kernel.
NCU_ALU_PIPE_BUSY = {"median_sphere r2": 0.877}
# Packed 16-bit min/max instructions per voxel of the selection networks
# (box: 336 per thread and z pair of two rows, 8 voxels; sphere: 334 per
# thread and z pair of one row, 4 voxels).  Each SM sub-partition issues one
# such warp instruction every two cycles, which sets the networks' floor.
NETWORK_MINMAX_PER_VOXEL = {"median_box r1": 42.0, "median_sphere r2": 83.5}


def alu_roofline(name, voxels, ms, sms, mhz):
    """The min/max-pipe floor of a network median and the measured fraction of it."""
    mm = NETWORK_MINMAX_PER_VOXEL.get(name)
    if mm is None or not ms or not sms or not mhz:
        return {}
    floor_ms = voxels * mm / 32 / (sms * 4 * 0.5 * mhz * 1e6) * 1e3
    return {"minmax_per_voxel": mm, "alu_floor_ms": round(floor_ms, 4), "alu_frac": round(floor_ms / ms, 4),
            "alu_floor_basis": f"{sms} SMs x 4 sub-partitions x 1 warp min/max per 2 cycles at {mhz:.0f} MHz"}


NOMINAL_HBM_GBS = 7900.0  # GB300 HBM3e, nominal (the measured copy peak is the roofline)


def suite_spec():
    """(name, kind, kernel, params, src, dst dtype code, bytes/voxel)."""
    return [
        ("gaussian_blur s(3,3,1.5)", "sep", "gaussian_blur_separable_3d", ((19, 19, 11), (3.0, 3.0, 1.5)), "img", 4, 6),
        ("mean_box r(5,5,2)", "sep", "mean_separable_3d", ((11, 11, 5), (5.0, 5.0, 2.0)), "img", 2, 4),
        ("minimum_box r(5,5,2)", "sep", "minimum_separable_3d", ((11, 11, 5), (5.0, 5.0, 2.0)), "img", 2, 4),
        ("maximum_box r(5,5,2)", "sep", "maximum_separable_3d", ((11, 11, 5), (5.0, 5.0, 2.0)), "img", 2, 4),
        ("median_box r1", "exec", "median_box_3d", {"Nx": 3, "Ny": 3, "Nz": 3}, "img", 2, 4),
        ("median_sphere r2", "exec", "median_sphere_3d", {"Nx": 5, "Ny": 5, "Nz": 5}, "img", 2, 4),
        ("sobel_3d", "exec", "sobel_3d", {}, "img", 4, 6),
        ("erode_sphere r1", "morph", "erode_sphere_3d", 1, "mask", 0, 2),
        ("erode_sphere r2", "morph", "erode_sphere_3d", 2, "mask", 0, 2),
        ("dilate_sphere r1", "morph", "dilate_sphere_3d", 1, "mask", 0, 2),
        ("dilate_sphere r2", "morph", "dilate_sphere_3d", 2, "mask", 0, 2),
    ]


def hbm_peak():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.proc = None
        self.index = index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        self.result = None
        if self.proc is None:
            return
        time.sleep(0.25)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [v.strip() for v in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        if sm:
            self.result = {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                           "reasons": sorted(reasons)}


def dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def gpu_local_cpus(index: int):
    """The CPUs of the GPU's NUMA node (sysfs local_cpulist of its PCI
    device), or None.  Host buffers first touched from them live in the memory
    next to the GPU's host link."""
    try:
        bus = subprocess.run(["nvidia-smi", "-i", str(index), "--query-gpu=pci.bus_id", "--format=csv,noheader"],
                             capture_output=True, text=True, timeout=20).stdout.strip()
        dom, rest = bus.split(":", 1)
        text = Path(f"/sys/bus/pci/devices/{int(dom, 16):04x}:{rest.lower()}/local_cpulist").read_text().strip()
        cpus = set()
        for part in text.split(","):
            lo, _, hi = part.partition("-")
            cpus.update(range(int(lo), int(hi or lo) + 1))
        cpus &= os.sched_getaffinity(0)
        return cpus or None
    except Exception:
        return None


def replicas_value(local_ms: float, voxels_per_step: int, steps: int, ws: int, device=None):
    """Replicas only (the path shards by stack, no exchange step): every
    rank filters its own stack; the job's time is the slowest rank's and its
    throughput all ranks' voxels over that time.  Returns (max_ms, Gvoxel/s)."""
    ms = local_ms
    if ws > 1:
        import torch
        import torch.distributed as tdist
        t = torch.tensor([local_ms], dtype=torch.float64, device=device)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, ws * voxels_per_step * steps / (ms * 1e-3) / 1e9


def config1_stack(device):
    """The 256x256x64 uint16 stack of config1 (200 blobs, seed 1)."""
    import torch

    from clk import synth
    return synth.blobs(CONFIG1_SHAPE, CONFIG1_BLOBS, seed=CONFIG1_SEED, dtype=torch.uint16, device=device)


def reference_config1(a_np, steps: int, nt: int, kind: str):
    """The reference kernels on the whole config1 stack (three launches of
    gaussian_blur_separable_3d with float temporaries), best and mean of
    `steps` runs on `nt` host threads."""
    import numpy as np

    from oracle import oracle
    impl = "ref" if kind == "reference" else "port"
    runs = []
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        oracle.separable("gaussian_blur_separable_3d", a_np, np.float32, (13, 13, 7), (2.0, 2.0, 1.0), impl=impl,
                         nthreads=nt)
        runs.append(time.perf_counter() - t0)
    ms = statistics.mean(runs) * 1e3
    return {"ms": round(ms, 3), "ms_best": round(min(runs) * 1e3, 3), "gvox_s": round(a_np.size / (ms * 1e-3) / 1e9, 4),
            "cores": nt, "kind": kind, "runs": len(runs),
            "what": "reference kernels on the host cores, the whole 256x256x64 stack"}


def run_reference(args):
    """The reference kernels on the host cores, on a bounded sample."""
    ws, rank, _ = dist()
    if rank != 0:  # rank 0 alone times the host cores; the others exit 0 without work
        return 0
    import numpy as np
    import torch

    from clk import synth
    from oracle import oracle

    kind = "reference" if oracle.ref_available() else "port"
    # a full-width slab of the stack's extent with the stack's blob density
    nb = max(1, int(N_BLOBS * SAMPLE[0] / SHAPE[0]))
    img = synth.blobs(SAMPLE, nb, seed=SEED, device="cpu")
    a = img.contiguous().numpy()
    mask = (a > 400).astype(np.uint8)
    nt = os.cpu_count() or 1
    spec = suite_spec()
    NP = {0: np.uint8, 2: np.uint16, 4: np.float32}
    impl = "ref" if kind == "reference" else "port"

    def one_step():
        for name, kindf, kernel, params, srcn, ddt, bpv in spec:
            src = a if srcn == "img" else mask
            if kindf == "sep":
                oracle.separable(kernel, src, NP[ddt], params[0], params[1], impl=impl, nthreads=nt)
            elif kindf == "exec":
                oracle.execute(kernel, src, NP[ddt], list(params.values()), impl=impl, nthreads=nt)
            else:
                cur = src
                for _ in range(params):
                    cur = oracle.execute(kernel, cur, np.uint8, impl=impl, nthreads=nt)

    for _ in range(args.warmup):
        one_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one_step()
    dt = time.perf_counter() - t0
    vox = a.size * len(spec) * args.steps
    v = vox / dt / 1e9
    c1 = reference_config1(config1_stack("cpu").numpy(), max(3, args.steps), nt, kind)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Gvoxel/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16/u8 in; u16/f32/u8 out",
            "data": "synthetic (seeded blob generator)",
            "config": {"workload": "plain filter suite on a 1024x1024x32 slab with the blob density of the "
                                   "1024x1024x256 u16 stack",
                       "filters": [s[0] for s in spec]},
            "cpu_baseline": {"value": v, "unit": "Gvoxel/s", "cores": nt, "kind": kind,
                             "sample": f"{SAMPLE[2]}x{SAMPLE[1]}x{SAMPLE[0]} voxels x {len(spec)} filters"},
            "e2e": {"value": v, "unit": "Gvoxel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "config1": c1}
    print(json.dumps(line))


def batch_images(n=512, seed=3, device="cuda"):
    """The uneven batch: 40% u8 / 40% u16 / 20% f32; half 2-D with X, Y
    log-uniform in [64, 1024], half 3-D with X, Y log-uniform in [64, 512]
    and Z uniform in [16, 128]; blob density of the 1024x1024x256 stack,
    intensities scaled to the pixel type's range."""
    import numpy as np
    import torch

    from clk import synth

    rng = np.random.default_rng(seed)
    density = N_BLOBS / float(SHAPE[0] * SHAPE[1] * SHAPE[2])
    imgs = []
    for k in range(n):
        u = rng.random()
        dt = torch.uint8 if u < 0.4 else (torch.uint16 if u < 0.8 else torch.float32)
        if k % 2 == 0:
            shp = tuple(int(np.exp(rng.uniform(np.log(64), np.log(1024)))) for _ in range(2))
        else:
            xy = [int(np.exp(rng.uniform(np.log(64), np.log(512)))) for _ in range(2)]
            shp = (int(rng.integers(16, 129)), xy[0], xy[1])
        nb = max(1, int(round(density * float(np.prod(shp)))))
        imgs.append(synth.blobs(shp, nb, seed=seed * 100003 + k, dtype=dt, device=device, scale_to_dtype=True))
    return imgs


def event_timer(stream, steps: int, warmup: int):
    """fn -> (mean ms per call over `steps`, per-call ms) with CUDA events on
    `stream` after `warmup` untimed calls."""
    import torch

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        lat = []
        e0.record(stream)
        for _ in range(steps):
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            z.record(stream)
            lat.append((a, z))
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, [a.elapsed_time(z) for a, z in lat]
    return timed


def batch_section(args, peak: float, local: int = 0):
    """Top-hat chain over 512 uneven images, batched (one graph launch)
    against per-image plain calls and per-kernel launches, same results."""
    import torch

    import clk

    imgs = batch_images()
    outs = [torch.empty_like(t) for t in imgs]
    ops = [clk.op_separable("gaussian_blur_separable", (13, 13, 13), (2.0, 2.0, 2.0)),
           clk.op_separable("minimum_separable", (9, 9, 9), (4.0, 4.0, 4.0)),
           clk.op_separable("maximum_separable", (9, 9, 9), (4.0, 4.0, 4.0)),
           clk.op_kernel("median_box", (3, 3, 3))]
    t0 = time.perf_counter()
    b = clk.Batch(ops, imgs, outs)
    plan_s = time.perf_counter() - t0
    vox = sum(t.numel() for t in imgs) * len(ops)
    nbytes = sum(2 * t.numel() * t.element_size() for t in imgs) * len(ops)  # each step reads + writes its image
    stream = torch.cuda.current_stream()
    warm = max(3, args.warmup)
    timed = event_timer(stream, args.steps, warm)
    with Clocks(local) as clocks:
        l0 = clk.launch_count()
        ms_b, lat_b = timed(b.run)
        launches_b = (clk.launch_count() - l0) // (args.steps + warm)
    batched = [t.clone() for t in outs]
    l0 = clk.launch_count()
    ms_p, _ = timed(b.run_plain)
    launches_p = (clk.launch_count() - l0) // (args.steps + warm)
    same = all(torch.equal(x.view(torch.uint8) if x.dtype != torch.uint8 else x,
                           y.view(torch.uint8) if y.dtype != torch.uint8 else y) for x, y in zip(batched, outs))
    l0 = clk.launch_count()
    ms_k, _ = timed(b.run_per_kernel)
    launches_k = (clk.launch_count() - l0) // (args.steps + warm)
    n_u8 = sum(t.dtype == torch.uint8 for t in imgs)
    n_u16 = sum(t.dtype == torch.uint16 for t in imgs)
    gbs = nbytes / (ms_b * 1e-3) / 1e9
    res = {
        "value": round(vox / (ms_b * 1e-3) / 1e9, 3), "unit": "Gvoxel/s", "ms_per_step": round(ms_b, 4),
        "ms_best": round(min(lat_b), 4), "steps": args.steps, "warmup": warm,
        "workload": "batched top-hat: 512 images (half 2-D XY in [64,1024], half 3-D XY in [64,512] x Z in "
                    "[16,128]), gaussian s=2 -> minimum r=4 -> maximum r=4 -> median_box r=1",
        "images": len(imgs), "u8": n_u8, "u16": n_u16, "f32": len(imgs) - n_u8 - n_u16,
        "voxels_per_step": vox, "l2": "working set far larger than L2",
        "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(gbs / peak, 4), "algorithmic_bytes_per_step": nbytes},
        "plain": {"value": round(vox / (ms_p * 1e-3) / 1e9, 3), "ms_per_step": round(ms_p, 4),
                  "launches_per_step": launches_p, "what": "per image, whole-filter calls (clk_separable, "
                                                           "clk_execute), one stream"},
        "per_kernel": {"value": round(vox / (ms_k * 1e-3) / 1e9, 3), "ms_per_step": round(ms_k, 4),
                       "launches_per_step": launches_k, "what": "per image, one clk_execute per kernel and axis "
                                                                "(the reference's launch pattern)"},
        "speedup_vs_plain": round(ms_p / ms_b, 3), "speedup_vs_per_kernel": round(ms_k / ms_b, 3),
        "gpu_launches": launches_b, "graph_kernels": b.launches,
        "identical_to_plain": bool(same), "plan_and_autotune_s": round(plan_s, 2), "clocks": clocks.result,
    }
    b.close()
    return res


def run_batch(args):
    import torch
    torch.cuda.set_device(0)
    peak, _ = hbm_peak()
    r = batch_section(args, peak)
    line = {"metric": "Gvoxel/s (batched pipeline, 512 uneven images)", "value": r["value"], "unit": "Gvoxel/s",
            "n_gpus": 1, "steps": args.steps, "warmup": r["warmup"], "ms_per_step": r["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u8/u16/f32 pixels, same type out",
            "data": "synthetic: seeded blob images, intensities scaled to type",
            "config": {"workload": r["workload"], "images": r["images"], "voxels_per_step": r["voxels_per_step"],
                       "l2": r["l2"]}, **{k: v for k, v in r.items() if k not in ("value", "ms_per_step")}}
    print(json.dumps(line))


def serve_pipeline(clk, rng):
    """1-4 steps sampled uniformly from {gaussian s in [1,4], mean r in [1,5],
    median_box r=1, erode/dilate_sphere r in [1,2], sobel}."""
    import numpy as np
    ops = []
    for _ in range(int(rng.integers(1, 5))):
        k = int(rng.integers(0, 5))
        if k == 0:
            s = float(rng.uniform(1, 4))
            n = 2 * int(np.ceil(3 * s)) + 1
            ops.append(clk.op_separable("gaussian_blur_separable", (n, n, n), (s, s, s)))
        elif k == 1:
            r = int(rng.integers(1, 6))
            ops.append(clk.op_separable("mean_separable", (2 * r + 1,) * 3, (r, r, r)))
        elif k == 2:
            ops.append(clk.op_kernel("median_box", (3, 3, 3)))
        elif k == 3:
            ops.append(clk.op_morphology("erode_sphere" if rng.random() < 0.5 else "dilate_sphere",
                                         int(rng.integers(1, 3))))
        else:
            ops.append(clk.op_kernel("sobel"))
    return ops


def serve_section(args, local: int = 0):
    """Served pipelines: Poisson arrivals at 200 / 1000 / 5000 req/s, each
    request one stack from the batched workload's size and type mix and a
    random 1-4 step pipeline, served with continuous admission (16 slots,
    64 GiB budget) against the same arrivals served one at a time; then a
    closed-loop saturation run (every request queued at once) of both."""
    import numpy as np
    import torch

    import clk

    pool = batch_images(n=96, seed=5)
    duration = 1.5

    def serve(reqs, outs, slots, arrivals):
        srv = clk.Server(slots=slots, hbm_budget_bytes=64 << 30)
        srv.wait(srv.submit(reqs[0][0], reqs[0][1], outs[0]))  # warm-up (not counted)
        srv.close()
        srv = clk.Server(slots=slots, hbm_budget_bytes=64 << 30)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k, ((ops, src), out) in enumerate(zip(reqs, outs)):
            if arrivals is not None:
                while time.perf_counter() - t0 < arrivals[k]:
                    pass
            srv.submit(ops, src, out)
        srv.drain(600000)
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        return {"p50_ms": round(st["p50_ms"], 3), "p99_ms": round(st["p99_ms"], 3),
                "mean_ms": round(st["mean_ms"], 3), "gvox_s": round(st["voxel_steps"] / wall / 1e9, 3),
                "completed": int(st["completed"]), "failed": int(st["failed"]),
                "peak_temporaries_gib": round(st["bytes_peak"] / 2**30, 3), "wall_s": round(wall, 3)}

    results = []
    with Clocks(local) as clocks:
        for rate in (200, 1000, 5000):
            rng = np.random.default_rng(rate)
            n = int(rate * duration)
            arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
            reqs = [(serve_pipeline(clk, rng), pool[int(rng.integers(0, len(pool)))]) for _ in range(n)]
            outs = [torch.empty_like(src) for _, src in reqs]
            row = {"rate_req_s": rate, "requests": n}
            for mode, slots in (("served", 16), ("serial", 1)):
                row[mode] = serve(reqs, outs, slots, arrivals)
            results.append(row)
        # closed loop: every request queued at t = 0, so the server runs at
        # its capacity; served against serial is the throughput gain of
        # continuous batching over one-at-a-time plain calls
        rng = np.random.default_rng(7)
        n = 2000
        reqs = [(serve_pipeline(clk, rng), pool[int(rng.integers(0, len(pool)))]) for _ in range(n)]
        outs = [torch.empty_like(src) for _, src in reqs]
        sat = {"requests": n, "served": serve(reqs, outs, 16, None), "serial": serve(reqs, outs, 1, None)}
        sat["served_over_serial"] = round(sat["served"]["gvox_s"] / max(sat["serial"]["gvox_s"], 1e-12), 3)
    top = results[-1]
    return {"value": top["served"]["p99_ms"], "unit": "ms (p99 at 5000 req/s)",
            "workload": "served pipelines: continuous admission, 16 slots, 64 GiB budget for temporaries; serial = "
                        "the same arrivals through 1 slot", "duration_s_per_rate": duration,
            "rates": results, "saturation": sat, "clocks": clocks.result}


def run_serve(args):
    import torch
    torch.cuda.set_device(0)
    r = serve_section(args)
    line = {
        "metric": "served p99 latency and Gvoxel/s (Poisson arrivals, uneven u8/u16/f32 stacks, 1-4 step pipelines)",
        "value": r["value"], "unit": r["unit"], "n_gpus": 1, "steps": len(r["rates"]),
        "warmup": 1, "ms_per_step": None, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "u8/u16/f32 pixels, same type out", "data": "synthetic: 96 seeded blob stacks, random pipelines",
        "config": {"workload": r["workload"], "duration_s_per_rate": r["duration_s_per_rate"]},
        "rates": r["rates"], "saturation": r["saturation"], "clocks": r["clocks"],
    }
    print(json.dumps(line))


def neighbours_spec():
    """The filters either side of the path, on the suite's stack and mask:
    (name, kernel, params, src, dst dtype code, bytes/voxel)."""
    return [
        ("minimum_sphere r1", "minimum_sphere_3d", {"Nx": 3, "Ny": 3, "Nz": 3}, "img", 2, 4),
        ("maximum_sphere r1", "maximum_sphere_3d", {"Nx": 3, "Ny": 3, "Nz": 3}, "img", 2, 4),
        ("mean_sphere r1", "mean_sphere_3d", {"Nx": 3, "Ny": 3, "Nz": 3}, "img", 2, 4),
        ("minimum_sphere r2", "minimum_sphere_3d", {"Nx": 5, "Ny": 5, "Nz": 5}, "img", 2, 4),
        ("mean_sphere r2", "mean_sphere_3d", {"Nx": 5, "Ny": 5, "Nz": 5}, "img", 2, 4),
        ("minimum_slice_by_slice_sphere r2", "minimum_slice_by_slice_sphere_3d", {"Nx": 5, "Ny": 5}, "img", 2, 4),
        ("median_slice_by_slice_box r1", "median_slice_by_slice_box_3d", {"Nx": 3, "Ny": 3}, "img", 2, 4),
        ("erode_sphere_slice_by_slice", "erode_sphere_slice_by_slice_3d", {}, "mask", 0, 2),
        ("gradient_z", "gradient_z_3d", {}, "img", 4, 6),
        ("laplace_diamond", "laplace_diamond_3d", {}, "img", 4, 6),
        ("laplace_box", "laplace_box_3d", {}, "img", 4, 6),
        ("greater_constant 400", "greater_constant_3d", {"scalar": 400.0}, "img", 0, 3),
        ("copy u16->f32", "copy_3d", {}, "img", 4, 6),
    ]


def run_neighbours(args):
    """The neighbourhood filters either side of the path, each its own
    clk_execute call on the 1024x1024x256 u16 stack (u8 mask for the
    morphology), with the reference kernels timed on a 256x256x32 sample."""
    import torch

    import clk
    from clk import synth

    torch.cuda.set_device(0)
    peak, peak_kind = hbm_peak()
    img = synth.blobs(SHAPE, N_BLOBS, seed=SEED, dtype=torch.uint16)
    mask = synth.mask_of(img, 400.0)
    V = img.numel()
    spec = neighbours_spec()
    if args.filters:
        import re
        spec = [t for t in spec if re.search(args.filters, t[0])]
    srcs = {"img": img, "mask": mask}
    outs = {t[0]: torch.empty(SHAPE, dtype=clk.torch_dtype(t[4]), device="cuda") for t in spec}
    stream = torch.cuda.current_stream()

    def call(t):
        name, kernel, params, srcn, ddt, bpv = t
        p = {("src1" if kernel.startswith("greater_constant") else "src"): srcs[srcn], "dst": outs[name]}
        p.update(params)
        clk.execute(kernel, p, stream=stream)

    for _ in range(max(3, args.warmup)):
        for t in spec:
            call(t)
    torch.cuda.synchronize()
    ev = {t[0]: [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                 for _ in range(args.steps)] for t in spec}
    t_begin, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = clk.launch_count()
    with Clocks(0) as clocks:
        torch.cuda.synchronize()
        t_begin.record(stream)
        for k in range(args.steps):
            for t in spec:
                ev[t[0]][k][0].record(stream)
                call(t)
                ev[t[0]][k][1].record(stream)
        t_end.record(stream)
        torch.cuda.synchronize()
    launches = clk.launch_count() - launches0
    total_ms = t_begin.elapsed_time(t_end)
    per = {}
    for name, kernel, params, srcn, ddt, bpv in spec:
        ms = statistics.mean(a.elapsed_time(b) for a, b in ev[name])
        per[name] = {"ms": round(ms, 4), "gvox_s": round(V / (ms * 1e-3) / 1e9, 2),
                     "hbm_frac": round(V * bpv / (ms * 1e-3) / 1e9 / peak, 4), "bytes_per_voxel": bpv}
    cpu = None
    if not args.no_cpu_baseline:
        import numpy as np

        from oracle import oracle as O
        kind = "reference" if O.ref_available() else "port"
        a = np.ascontiguousarray(img.cpu().numpy()[:SAMPLE[0], :SAMPLE[1], :SAMPLE[2]])
        m = np.ascontiguousarray(mask.cpu().numpy()[:SAMPLE[0], :SAMPLE[1], :SAMPLE[2]])
        nt = os.cpu_count() or 1
        NP = {0: np.uint8, 2: np.uint16, 4: np.float32}
        t0 = time.perf_counter()
        for name, kernel, params, srcn, ddt, bpv in spec:
            ints = [v for n, v in params.items() if n != "scalar"]
            floats = [v for n, v in params.items() if n == "scalar"]
            O.execute(kernel, a if srcn == "img" else m, NP[ddt], ints, floats,
                      impl="ref" if kind == "reference" else "port", nthreads=nt)
        dt = time.perf_counter() - t0
        cpu = {"value": a.size * len(spec) / dt / 1e9, "unit": "Gvoxel/s", "cores": nt, "kind": kind,
               "sample": f"the first {SAMPLE[0]} planes ({SAMPLE[2]}x{SAMPLE[1]}x{SAMPLE[0]}) of the stack x {len(spec)} filters, {dt:.1f} s"}
    line = {
        "metric": "Gvoxel/s (neighbourhood filters either side of the path, 1024x1024x256)",
        "value": round(V * len(spec) * args.steps / (total_ms * 1e-3) / 1e9, 3), "unit": "Gvoxel/s", "n_gpus": 1,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u16 in (u8 mask); u16/u8/f32 out", "data": "synthetic: the suite's seeded blob stack and mask",
        "config": {"workload": "neighbourhood filters either side of the path on 1024x1024x256 uint16, each its "
                               "own call", "voxels": V, "l2": "inputs larger than L2; no flush"},
        "per_filter": per, "gpu_launches": launches, "clocks": clocks.result, "cpu_baseline": cpu,
    }
    print(json.dumps(line))
    return 0


LARGE_SHAPE = (400, 2048, 2048)  # (z, y, x): 6.71 GB of float32


def large_section(args, peak: float, shape=LARGE_SHAPE, filters: str = "", local: int = 0):
    """Large-halo filters on one 2048x2048x400 float32 stack (blobs plus
    N(0, 20) noise): gaussian sigma (10,10,5) (N = 61,61,31), maximum r
    (15,15,7) and median_sphere r=2, each its own call, f32 -> f32."""
    import torch

    import clk
    from clk import synth

    img = synth.blobs(shape, max(1, int(N_BLOBS * shape[0] / LARGE_SHAPE[0])), seed=SEED + 5, dtype=torch.float32,
                      poisson=False, noise_sigma=20.0)
    V = img.numel()
    out = torch.empty_like(img)
    stream = torch.cuda.current_stream()
    spec = [
        ("gaussian_blur s(10,10,5)", lambda: clk.separable("gaussian_blur_separable_3d", img, out, (61, 61, 31),
                                                           (10.0, 10.0, 5.0), stream=stream)),
        ("maximum_box r(15,15,7)", lambda: clk.separable("maximum_separable_3d", img, out, (31, 31, 15),
                                                         (15.0, 15.0, 7.0), stream=stream)),
        ("median_sphere r2", lambda: clk.execute("median_sphere_3d", {"src": img, "dst": out, "Nx": 5, "Ny": 5,
                                                                       "Nz": 5}, stream=stream)),
    ]
    if filters:
        import re
        spec = [t for t in spec if re.search(filters, t[0])]
    for _ in range(max(3, args.warmup)):
        for _, fn in spec:
            fn()
    torch.cuda.synchronize()
    ev = {n: [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)] for n, _ in spec}
    t_begin, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = clk.launch_count()
    with Clocks(local) as clocks:
        torch.cuda.synchronize()
        t_begin.record(stream)
        for k in range(args.steps):
            for n, fn in spec:
                ev[n][k][0].record(stream)
                fn()
                ev[n][k][1].record(stream)
        t_end.record(stream)
        torch.cuda.synchronize()
    launches = clk.launch_count() - launches0
    total_ms = t_begin.elapsed_time(t_end)
    per = {}
    for n, _ in spec:
        runs = [a.elapsed_time(b) for a, b in ev[n]]
        ms = statistics.mean(runs)
        per[n] = {"ms": round(ms, 3), "ms_best": round(min(runs), 3), "gvox_s": round(V / (ms * 1e-3) / 1e9, 2),
                  "hbm_frac": round(V * 8 / (ms * 1e-3) / 1e9 / peak, 4), "bytes_per_voxel": 8}
    dom = max(per, key=lambda n: per[n]["ms"])
    dom_gbs = V * 8 / (per[dom]["ms"] * 1e-3) / 1e9
    return {"value": round(V * len(spec) * args.steps / (total_ms * 1e-3) / 1e9, 3), "unit": "Gvoxel/s",
            "ms_per_step": round(total_ms / args.steps, 3), "steps": args.steps, "warmup": max(3, args.warmup),
            "workload": f"large-halo filters on {shape[2]}x{shape[1]}x{shape[0]} float32, each its own call",
            "voxels": V, "l2": "inputs larger than L2 (6.7 GB); no flush", "per_filter": per,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(dom_gbs, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(dom_gbs / peak, 4), "traffic": None},
            "gpu_launches": launches, "clocks": clocks.result}


def run_large(args):
    import torch
    torch.cuda.set_device(0)
    peak, peak_kind = hbm_peak()
    shape = tuple(int(v) for v in args.shape.split(",")) if args.shape else LARGE_SHAPE
    r = large_section(args, peak, shape, args.filters)
    r["roofline"]["peak_kind"] = peak_kind
    line = {
        "metric": "Gvoxel/s (large-halo filters, 2048x2048x400 f32)", "value": r["value"], "unit": "Gvoxel/s",
        "n_gpus": 1, "steps": args.steps, "warmup": r["warmup"], "ms_per_step": r["ms_per_step"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded blob stack plus N(0,20) noise, float32",
        "config": {"workload": r["workload"], "voxels": r["voxels"], "l2": r["l2"]},
        "per_filter": r["per_filter"], "roofline": r["roofline"], "gpu_launches": r["gpu_launches"],
        "clocks": r["clocks"],
    }
    print(json.dumps(line))
    return 0


def config1_section(args, peak: float, local: int = 0, cpu: bool = True):
    """Plain gaussian_blur_separable_3d sigma (2,2,1), N = (13,13,7), on the
    256x256x64 uint16 stack (200 blobs) to float32.  Its 24 MiB of data fit
    in L2, so a 512 MiB buffer is written between timed calls and each call
    is timed alone with CUDA events.  Beside it: the reference kernels on
    the host cores on the same stack."""
    import torch

    import clk

    img = config1_stack("cuda")
    out = torch.empty(img.shape, dtype=torch.float32, device="cuda")
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def call():
        clk.separable("gaussian_blur_separable_3d", img, out, (13, 13, 7), (2.0, 2.0, 1.0), stream=stream)

    for _ in range(max(3, args.warmup)):
        call()
    torch.cuda.synchronize()
    runs = []
    l0 = clk.launch_count()
    with Clocks(local) as clocks:
        for _ in range(max(10, args.steps)):
            flush.fill_(1.0)
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            call()
            z.record(stream)
            runs.append((a, z))
        torch.cuda.synchronize()
    launches = clk.launch_count() - l0
    ms_runs = [a.elapsed_time(z) for a, z in runs]
    ms = statistics.mean(ms_runs)
    V = img.numel()
    gbs = V * 6 / (ms * 1e-3) / 1e9
    res = {"ms": round(ms, 4), "ms_best": round(min(ms_runs), 4), "gvox_s": round(V / (ms * 1e-3) / 1e9, 2),
           "runs": len(ms_runs), "voxels": V,
           "workload": "plain gaussian_blur_separable_3d s(2,2,1) N(13,13,7), 256x256x64 uint16 -> float32",
           "l2": "512 MiB written between timed calls (the stack fits in L2)",
           "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(gbs / peak, 4), "bytes_per_voxel": 6},
           "gpu_launches": launches, "clocks": clocks.result}
    if cpu:
        try:
            from oracle import oracle
            kind = "reference" if oracle.ref_available() else "port"
            ref = reference_config1(img.cpu().numpy(), 3, os.cpu_count() or 1, kind)
            res["cpu_reference"] = ref
            res["gpu_over_cpu_reference"] = round(ref["ms"] / ms, 1)
        except Exception as e:  # the oracle is optional infrastructure on the box
            res["cpu_reference"] = {"kind": "unavailable", "why": str(e)}
    return res


def host_link(h_img, img, h_out, outs, stream, push_kernel, zero_copy, h2d_bytes, d2h_bytes, e2e_ms):
    """The host link's own rates, measured the way the e2e run moves its
    bytes: host->device by copy_3d kernels reading the pinned stack (or a
    copy engine), device->host by a copy_3d kernel storing into a pinned
    host image (or a copy engine).  bound_ms_per_step = the step's bytes at
    those rates with the two directions overlapped (the link is full
    duplex); frac = bound / measured."""
    import torch

    import clk
    name = max(outs, key=lambda n: outs[n].numel() * outs[n].element_size())
    dev_out, hst_out = outs[name], h_out[name]
    d_img = torch.empty_like(img)

    def h2d():
        if push_kernel:
            clk.execute("copy_3d", {"src": h_img, "dst": d_img}, stream=stream)
        else:
            with torch.cuda.stream(stream):
                d_img.copy_(h_img, non_blocking=True)

    def d2h():
        if zero_copy:
            clk.execute("copy_3d", {"src": dev_out, "dst": hst_out}, stream=stream)
        else:
            with torch.cuda.stream(stream):
                hst_out.copy_(dev_out, non_blocking=True)

    res = {}
    for key, fn, nbytes in (("h2d_gbs", h2d, h_img.numel() * h_img.element_size()),
                            ("d2h_gbs", d2h, dev_out.numel() * dev_out.element_size())):
        fn()
        torch.cuda.synchronize()
        runs = []
        for _ in range(5):
            a, z = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            z.record(stream)
            torch.cuda.synchronize()
            runs.append(a.elapsed_time(z))
        res[key] = round(nbytes / (min(runs) * 1e-3) / 1e9, 1)
    del d_img
    bound = max(h2d_bytes / (res["h2d_gbs"] * 1e9), d2h_bytes / (res["d2h_gbs"] * 1e9)) * 1e3
    res["bound_ms_per_step"] = round(bound, 2)
    res["frac"] = round(bound / e2e_ms, 4)
    res["how"] = ("best of 5 single transfers of the stack (h2d) and the largest output (d2h) through the same "
                  "mechanism the e2e step uses")
    return res


def cpu_baseline(a_np, mask_np):
    """Reference CPU kernels on a bounded sample (first SAMPLE voxels)."""
    import numpy as np

    from oracle import oracle

    kind = "reference" if oracle.ref_available() else "port"
    impl = "ref" if kind == "reference" else "port"
    a = np.ascontiguousarray(a_np[:SAMPLE[0], :SAMPLE[1], :SAMPLE[2]])
    m = np.ascontiguousarray(mask_np[:SAMPLE[0], :SAMPLE[1], :SAMPLE[2]])
    nt = os.cpu_count() or 1
    NP = {0: np.uint8, 2: np.uint16, 4: np.float32}
    t0 = time.perf_counter()
    for name, kindf, kernel, params, srcn, ddt, bpv in suite_spec():
        src = a if srcn == "img" else m
        if kindf == "sep":
            oracle.separable(kernel, src, NP[ddt], params[0], params[1], impl=impl, nthreads=nt)
        elif kindf == "exec":
            oracle.execute(kernel, src, NP[ddt], list(params.values()), impl=impl, nthreads=nt)
        else:
            cur = src
            for _ in range(params):
                cur = oracle.execute(kernel, cur, np.uint8, impl=impl, nthreads=nt)
    dt = time.perf_counter() - t0
    return {"value": a.size * len(suite_spec()) / dt / 1e9, "unit": "Gvoxel/s", "cores": nt, "kind": kind,
            "sample": f"the first {SAMPLE[0]} planes ({SAMPLE[2]}x{SAMPLE[1]}x{SAMPLE[0]}) of the stack x "
                      f"{len(suite_spec())} filters, "
                      f"{dt:.1f} s"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--full-sample", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="suite only: skip the config1 / batch / serve / large sections of the line")
    ap.add_argument("--e2e-pull", default="zero-copy", choices=["zero-copy", "copy"],
                    help="how results reach host memory in the e2e run: the filters store into pinned host "
                         "images (zero-copy) or write device images that copy engines then pull")
    ap.add_argument("--e2e-push", default="kernel", choices=["kernel", "copy"],
                    help="how the input stack and mask reach the device in the e2e run: copy_3d kernels reading "
                         "the pinned host images (kernel) or copy-engine copies")
    ap.add_argument("--shape", default="", help="suite stack as z,y,x (default 256,1024,1024)")
    ap.add_argument("--filters", default="", help="regex selecting suite filters by name")
    ap.add_argument("--workload", default="suite",
                    choices=["suite", "batch", "serve", "large", "neighbours", "config1"],
                    help="suite: plain filter suite on 1024x1024x256 u16 (default); batch: top-hat chain over 512 uneven "
                         "images; serve: Poisson-arrival requests; large: large-halo f32 "
                         "filters on 2048x2048x400; neighbours: the filters either side of the path")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "batch":
        return run_batch(args)
    if args.workload == "large":
        return run_large(args)
    if args.workload == "neighbours":
        return run_neighbours(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "config1":
        import torch
        torch.cuda.set_device(0)
        print(json.dumps(config1_section(args, hbm_peak()[0])))
        return 0

    import torch

    import clk
    from clk import synth

    ws, rank, local = dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    peak, peak_kind = hbm_peak()

    shape = SHAPE
    if args.shape:  # a smaller stack of the same data density (profiling captures)
        shape = tuple(int(v) for v in args.shape.split(","))
    n_blobs = max(1, int(N_BLOBS * shape[0] * shape[1] * shape[2] / (SHAPE[0] * SHAPE[1] * SHAPE[2])))
    img = synth.blobs(shape, n_blobs, seed=SEED + rank, dtype=torch.uint16, device=dev)
    mask = synth.mask_of(img, 400.0)
    V = img.numel()
    spec = suite_spec()
    if args.filters:
        import re
        spec = [s for s in spec if re.search(args.filters, s[0])]
    outs = {}
    for name, kind, kernel, params, srcn, ddt, bpv in spec:
        outs[name] = torch.empty(shape, dtype=clk.torch_dtype(ddt), device=dev)
    tmp_mask = torch.empty_like(mask)
    stream = torch.cuda.current_stream()

    def run(name, kind, kernel, params, srcn, src_t, out_t, st=None):
        st = stream if st is None else st
        if kind == "sep":
            clk.separable(kernel, src_t, out_t, params[0], params[1], stream=st)
        elif kind == "exec":
            p = {"src": src_t, "dst": out_t}
            p.update(params)
            clk.execute(kernel, p, stream=st)
        elif params == 1:  # r=1: one launch of the reference kernel
            clk.execute(kernel, {"src": src_t, "dst": out_t}, stream=st)
        else:  # radius r: r successive launches, fused in pairs
            clk.morphology(kernel, src_t, out_t, params, stream=st)

    def step(srcs):
        for name, kind, kernel, params, srcn, ddt, bpv in spec:
            run(name, kind, kernel, params, srcn, srcs[srcn], outs[name])

    srcs = {"img": img, "mask": mask}
    for _ in range(max(3, args.warmup)):
        step(srcs)
    torch.cuda.synchronize()
    if ws > 1:
        tdist.barrier()

    ev = {s[0]: [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                 for _ in range(args.steps)] for s in spec}
    t_begin, t_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = clk.launch_count()
    with Clocks(local) as clocks:
        torch.cuda.synchronize()
        t_begin.record(stream)
        for k in range(args.steps):
            for name, kind, kernel, params, srcn, ddt, bpv in spec:
                ev[name][k][0].record(stream)
                run(name, kind, kernel, params, srcn, srcs[srcn], outs[name])
                ev[name][k][1].record(stream)
        t_end.record(stream)
        torch.cuda.synchronize()
    launches = clk.launch_count() - launches0
    total_ms = t_begin.elapsed_time(t_end)
    total_ms, value = replicas_value(total_ms, V * len(spec), args.steps, ws, device=dev)
    per = {}
    for name, kind, kernel, params, srcn, ddt, bpv in spec:
        runs = [a.elapsed_time(b) for a, b in ev[name]]
        ms = statistics.mean(runs)
        gbs = V * bpv / (ms * 1e-3) / 1e9
        per[name] = {"ms": round(ms, 4), "ms_median": round(statistics.median(runs), 4),
                     "ms_best": round(min(runs), 4), "gvox_s": round(V / (ms * 1e-3) / 1e9, 2),
                     "hbm_frac": round(gbs / peak, 4), "bytes_per_voxel": bpv}
    try:  # the networks' ALU floor at the sampled SM clock (the maximum clock if none was sampled)
        sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
        mhz = (clocks.result or {}).get("sm_mhz") or 2070.0
        for name in per:
            per[name].update(alu_roofline(name, V, per[name]["ms"], sms, mhz))
    except Exception:  # informational only
        pass
    dom = max(per, key=lambda n: per[n]["ms"])
    dom_gbs = V * per[dom]["bytes_per_voxel"] / (per[dom]["ms"] * 1e-3) / 1e9

    e2e = None
    if not args.no_e2e:
        # The same suite from pinned host buffers, pipelined the way a caller
        # would: the host->device copy of step k+1's stack and mask (copy
        # engine, two device input sets) overlaps the filters of step k.  The
        # results reach host memory either by the filters storing straight
        # into pinned host images over the host link (zero-copy, the
        # default: clk_host_image_pointer) or by device outputs that a third
        # stream pulls with copy engines.  Every byte crosses the link inside
        # the timed region either way.
        saved_aff = os.sched_getaffinity(0)
        local_cpus = gpu_local_cpus(local)
        if local_cpus:  # pinned pages first-touched next to the GPU
            os.sched_setaffinity(0, local_cpus)
        zero_copy = args.e2e_pull == "zero-copy"
        push_kernel = args.e2e_push == "kernel"
        h_img = img.cpu().pin_memory()
        h_mask = mask.cpu().pin_memory()
        h_out = {n: torch.empty(shape, dtype=o.dtype).pin_memory() for n, o in outs.items()}
        for t in h_out.values():
            t.zero_()
        d_in = [{"img": torch.empty_like(img), "mask": torch.empty_like(mask)} for _ in range(2)]
        d_out = None if zero_copy else [{n: torch.empty_like(o) for n, o in outs.items()} for _ in range(2)]
        # the filters of a step are independent (each reads the step's input,
        # writes its own output): three compute streams keep the host link
        # busy across kernel boundaries
        css = [torch.cuda.Stream() for _ in range(3)]
        cs, hs, ds = css[0], torch.cuda.Stream(), torch.cuda.Stream()
        ev_in = [torch.cuda.Event() for _ in range(2)]
        ev_in_free = [[torch.cuda.Event() for _ in css] for _ in range(2)]
        ev_out = [{n: torch.cuda.Event() for n in outs} for _ in range(2)]
        ev_out_free = [{n: torch.cuda.Event() for n in outs} for _ in range(2)]
        used = [False, False]

        def e2e_step(k):
            b = k % 2
            with torch.cuda.stream(hs):
                if used[b]:
                    for e in ev_in_free[b]:
                        hs.wait_event(e)
                if push_kernel:
                    clk.execute("copy_3d", {"src": h_img, "dst": d_in[b]["img"]}, stream=hs)
                    clk.execute("copy_3d", {"src": h_mask, "dst": d_in[b]["mask"]}, stream=hs)
                else:
                    d_in[b]["img"].copy_(h_img, non_blocking=True)
                    d_in[b]["mask"].copy_(h_mask, non_blocking=True)
                ev_in[b].record(hs)
            for c in css:
                c.wait_event(ev_in[b])
            for f, (name, kind, kernel, params, srcn, ddt, bpv) in enumerate(spec):
                c = css[f % len(css)]
                if zero_copy:
                    run(name, kind, kernel, params, srcn, d_in[b][srcn], h_out[name], st=c)
                    continue
                if used[b]:
                    c.wait_event(ev_out_free[b][name])
                run(name, kind, kernel, params, srcn, d_in[b][srcn], d_out[b][name], st=c)
                ev_out[b][name].record(c)
            for e, c in zip(ev_in_free[b], css):
                e.record(c)
            if not zero_copy:
                with torch.cuda.stream(ds):
                    for name in outs:
                        ds.wait_event(ev_out[b][name])
                        h_out[name].copy_(d_out[b][name], non_blocking=True)
                        ev_out_free[b][name].record(ds)
            used[b] = True

        e2e_step(0)
        e2e_step(1)
        torch.cuda.synchronize()
        l0 = clk.launch_count()
        t0 = time.perf_counter()
        for k in range(args.steps):
            e2e_step(k)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        os.sched_setaffinity(0, saved_aff)
        e2e = {"value": round(V * len(spec) * args.steps / dt / 1e9, 3), "unit": "Gvoxel/s",
               "h2d_bytes_per_step": img.numel() * 2 + mask.numel(),
               "d2h_bytes_per_step": sum(o.numel() * o.element_size() for o in outs.values()),
               "ms_per_step": round(dt * 1e3 / args.steps, 2),
               "gpu_launches": clk.launch_count() - l0,
               "push": args.e2e_push, "pull": args.e2e_pull,
               "path": ("pinned host stack + mask -> device (" + ("copy_3d kernels" if push_kernel else "copy engine")
                        + "), clk C-ABI calls " + ("storing every output straight into pinned host images (zero-copy "
                                                   "over the host link)" if zero_copy else
                                                   "writing device outputs that copy engines pull to pinned host")
                        + "; the filters of a step spread over three streams; the next step's input copy overlaps "
                        "them")}
        if zero_copy:  # the host images hold the filters' results
            ok = all(torch.equal(h_out[n], outs[n].cpu()) for n in outs) if args.steps > 0 else True
            e2e["host_results_match_device"] = bool(ok)
        e2e["link"] = host_link(h_img, img, h_out, outs, cs, push_kernel, zero_copy,
                                e2e["h2d_bytes_per_step"], e2e["d2h_bytes_per_step"], e2e["ms_per_step"])

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(img.cpu().numpy(), mask.cpu().numpy())
        except Exception as e:  # the oracle is optional infrastructure on the box
            cpu = {"value": None, "unit": "Gvoxel/s", "cores": os.cpu_count(), "kind": "unavailable",
                   "sample": f"oracle could not run: {e}"}

    extras = {}
    if ws == 1 and not args.no_extras and not args.shape and not args.filters:
        del outs, tmp_mask
        if not args.no_e2e:
            del h_out, h_img, h_mask, d_in, d_out
        torch.cuda.empty_cache()
        extras["config1"] = config1_section(args, peak, local, cpu=not args.no_cpu_baseline)
        extras["batch"] = batch_section(args, peak, local)
        torch.cuda.empty_cache()
        extras["serve"] = serve_section(args, local)
        torch.cuda.empty_cache()
        extras["large"] = large_section(args, peak, local=local)
        torch.cuda.empty_cache()

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Gvoxel/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": round(total_ms / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u16 in (u8 mask); u16/f32/u8 out; f32 arithmetic",
            "data": "synthetic: seeded blob stack (background 100, 20k Gaussian blobs, Poisson), mask = img > 400",
            "config": {"workload": f"plain filter suite, {shape[2]}x{shape[1]}x{shape[0]} uint16 stack + uint8 "
                                   "mask, each filter run separately", "voxels": V, "filters": [s[0] for s in spec],
                       "l2": "inputs larger than L2 (512 MiB stack, 256 MiB mask); no flush"},
            "per_filter": per,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(dom_gbs, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(dom_gbs / peak, 4), "peak_kind": peak_kind,
                         "frac_of_nominal": round(dom_gbs / NOMINAL_HBM_GBS, 4),
                         "traffic": (round(NCU_DRAM_BYTES_PER_VOXEL[dom] * V) if dom in NCU_DRAM_BYTES_PER_VOXEL
                                     else None),
                         "traffic_source": TRAFFIC_SOURCE,
                         "algorithmic_bytes": int(V * per[dom]["bytes_per_voxel"]),
                         **({"alu_pipe_busy": NCU_ALU_PIPE_BUSY[dom],
                             "note": "selection network: bound by the min/max (ALU) pipe, not HBM",
                             **{k: per[dom][k] for k in ("minmax_per_voxel", "alu_floor_ms", "alu_frac")
                                if k in per[dom]}}
                            if dom in NCU_ALU_PIPE_BUSY else {})},
            "gpu_launches": launches,
            "clocks": clocks.result,
            "e2e": e2e,
            "cpu_baseline": cpu,
            **extras,
        }
        print(json.dumps(line))
    if ws > 1:
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()

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

  python bench.py [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference kernels on the host cores (oracle/_ref:
the reference's .cl compiled as C++, else the oracle restatement) on a
bounded sample of the same workload.  Under torchrun each rank runs an
independent replica (the path shards by stack; no collective).
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
SAMPLE = (32, 256, 256)  # CPU-baseline sample: a sub-stack of the same data
METRIC = "Gvoxel/s (plain filter suite, 1024x1024x256)"


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


def run_reference(args):
    """The reference kernels on the host cores, on a bounded sample."""
    ws, rank, _ = dist()
    if rank != 0:
        return
    import numpy as np
    import torch

    from clk import synth
    from oracle import oracle

    kind = "reference" if oracle.ref_available() else "port"
    img = synth.blobs(SHAPE, N_BLOBS, seed=SEED, device="cpu") if args.full_sample else None
    if img is None:  # same generator, restricted to the sample's extent and blob density
        vol = SAMPLE[0] * SAMPLE[1] * SAMPLE[2]
        nb = max(1, int(N_BLOBS * vol / (SHAPE[0] * SHAPE[1] * SHAPE[2])))
        img = synth.blobs(SAMPLE, nb, seed=SEED, device="cpu")
    a = img[:SAMPLE[0], :SAMPLE[1], :SAMPLE[2]].contiguous().numpy()
    mask = (a > 400).astype(np.uint8)
    nt = os.cpu_count() or 1
    spec = suite_spec()
    NP = {0: np.uint8, 2: np.uint16, 4: np.float32}

    def one_step():
        for name, kindf, kernel, params, srcn, ddt, bpv in spec:
            src = a if srcn == "img" else mask
            if kindf == "sep":
                oracle.separable(kernel, src, NP[ddt], params[0], params[1], impl="ref" if kind == "reference"
                                 else "port", nthreads=nt)
            elif kindf == "exec":
                oracle.execute(kernel, src, NP[ddt], list(params.values()), impl="ref" if kind == "reference"
                               else "port", nthreads=nt)
            else:
                cur = src
                for _ in range(params):
                    cur = oracle.execute(kernel, cur, np.uint8, impl="ref" if kind == "reference" else "port",
                                         nthreads=nt)

    for _ in range(args.warmup):
        one_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one_step()
    dt = time.perf_counter() - t0
    vox = a.size * len(spec) * args.steps
    v = vox / dt / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Gvoxel/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u16/u8 in; u16/f32/u8 out",
            "data": "synthetic (seeded blob generator)",
            "config": {"workload": "plain filter suite on a 256x256x32 sample of the 1024x1024x256 u16 stack",
                       "filters": [s[0] for s in spec]},
            "cpu_baseline": {"value": v, "unit": "Gvoxel/s", "cores": nt, "kind": kind,
                             "sample": f"{SAMPLE[2]}x{SAMPLE[1]}x{SAMPLE[0]} voxels x {len(spec)} filters"},
            "e2e": {"value": v, "unit": "Gvoxel/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


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
            "sample": f"{SAMPLE[2]}x{SAMPLE[1]}x{SAMPLE[0]} corner of the stack x {len(suite_spec())} filters, "
                      f"{dt:.1f} s"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--full-sample", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

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

    img = synth.blobs(SHAPE, N_BLOBS, seed=SEED + rank, dtype=torch.uint16, device=dev)
    mask = synth.mask_of(img, 400.0)
    V = img.numel()
    spec = suite_spec()
    outs = {}
    for name, kind, kernel, params, srcn, ddt, bpv in spec:
        outs[name] = torch.empty(SHAPE, dtype=clk.torch_dtype(ddt), device=dev)
    tmp_mask = torch.empty_like(mask)
    stream = torch.cuda.current_stream()

    def run(name, kind, kernel, params, srcn, src_t, out_t):
        if kind == "sep":
            clk.separable(kernel, src_t, out_t, params[0], params[1], stream=stream)
        elif kind == "exec":
            p = {"src": src_t, "dst": out_t}
            p.update(params)
            clk.execute(kernel, p, stream=stream)
        elif params == 1:  # r=1: one launch of the reference kernel
            clk.execute(kernel, {"src": src_t, "dst": out_t}, stream=stream)
        else:  # radius r: r successive launches, fused in pairs
            clk.morphology(kernel, src_t, out_t, params, stream=stream)

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
    if ws > 1:
        t = torch.tensor([total_ms], device=dev)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        total_ms = float(t.item())
    per = {}
    for name, kind, kernel, params, srcn, ddt, bpv in spec:
        ms = statistics.mean(a.elapsed_time(b) for a, b in ev[name])
        gbs = V * bpv / (ms * 1e-3) / 1e9
        per[name] = {"ms": round(ms, 4), "gvox_s": round(V / (ms * 1e-3) / 1e9, 2),
                     "hbm_frac": round(gbs / peak, 4), "bytes_per_voxel": bpv}
    dom = max(per, key=lambda n: per[n]["ms"])
    dom_gbs = V * per[dom]["bytes_per_voxel"] / (per[dom]["ms"] * 1e-3) / 1e9
    value = ws * V * len(spec) * args.steps / (total_ms * 1e-3) / 1e9

    e2e = None
    if not args.no_e2e:
        h_img = img.cpu().pin_memory()
        h_mask = mask.cpu().pin_memory()
        h_out = {n: torch.empty(SHAPE, dtype=o.dtype).pin_memory() for n, o in outs.items()}
        d_img, d_mask = torch.empty_like(img), torch.empty_like(mask)

        def e2e_step():
            d_img.copy_(h_img, non_blocking=True)
            d_mask.copy_(h_mask, non_blocking=True)
            step({"img": d_img, "mask": d_mask})
            for n, o in outs.items():
                h_out[n].copy_(o, non_blocking=True)

        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        e2e = {"value": round(V * len(spec) * args.steps / dt / 1e9, 3), "unit": "Gvoxel/s",
               "h2d_bytes_per_step": img.numel() * 2 + mask.numel(),
               "d2h_bytes_per_step": sum(o.numel() * o.element_size() for o in outs.values()),
               "path": "pinned host stack + mask -> device, clk C-ABI calls, all outputs -> pinned host"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(img.cpu().numpy(), mask.cpu().numpy())
        except Exception as e:  # the oracle is optional infrastructure on the box
            cpu = {"value": None, "unit": "Gvoxel/s", "cores": os.cpu_count(), "kind": "unavailable",
                   "sample": f"oracle could not run: {e}"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Gvoxel/s", "n_gpus": ws, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": round(total_ms / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u16 in (u8 mask); u16/f32/u8 out; f32 arithmetic",
            "data": "synthetic: seeded blob stack (background 100, 20k Gaussian blobs, Poisson), mask = img > 400",
            "config": {"workload": "plain filter suite, 1024x1024x256 uint16 stack + uint8 mask, each filter "
                                   "run separately", "voxels": V, "filters": [s[0] for s in spec],
                       "l2": "inputs larger than L2 (512 MiB stack, 256 MiB mask); no flush"},
            "per_filter": per,
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(dom_gbs, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(dom_gbs / peak, 4), "peak_kind": peak_kind,
                         "traffic": None},
            "gpu_launches": launches,
            "clocks": clocks.result,
            "e2e": e2e,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line))
    if ws > 1:
        tdist.destroy_process_group()


if __name__ == "__main__":
    main()

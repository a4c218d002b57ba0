"""Benchmark: primary Mrays/s per traversal on one GB300.

Workload (the reference's CT-scan benchmark shape): a 512x361x512 RGBA8
CT-like volume (synthetic, seed 1, standing in for the Stanford bunny CT),
converted on the GPU to a rope octree (`convert --rope`, lossless), rendered
at 1920x1080 with all five traversals (dda on the grid; svo-naive, esvo,
svo-df, svo-rope on the octree) along a 450-frame camera path (orbit at 2x the
extent, dolly to 0.3x, rotation about an interior point).

One step = one frame of the path rendered by all five traversals.  `value`
is the rays of all K steps divided by the device time of the K steps (CUDA
events on the launch stream; volumes resident in HBM); `e2e` is the same
metric through the C ABI's host-buffer entry point (xn_render), with the
camera upload and the image read-back inside the timed region.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --impl reference the reference's algorithm runs on the host cores (the
oracle's FP32 restatement of the shaders; the reference's own Vulkan shaders
need a graphics stack that this machine does not have) over a sample of rows
of the same frames.
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

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

TRAVERSALS = ("dda", "svo-naive", "esvo", "svo-df", "svo-rope")
WIDTH, HEIGHT = 1920, 1080
DIMS = (512, 361, 512)  # x, y, z
EMISSION = 10.0
PATH_FRAMES = 450
METRIC = "primary Mrays/s per traversal on 1 GB300"
WORKLOAD = "CT-scan 512x361x512 RGBA8 grid + rope octree, 5 traversals at 1920x1080, 450-frame path"


def frame_indices(k: int, offset: int = 0) -> list[int]:
    return [(offset + (j * PATH_FRAMES) // max(1, k)) % PATH_FRAMES for j in range(k)]


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def load_traffic() -> dict:
    """DRAM bytes per launch from the committed ncu summary, if present."""
    p = ROOT / "profiles" / "traffic_ct_1080p.txt"
    out = {}
    if p.exists():
        for line in p.read_text().splitlines():
            f = line.split()
            if len(f) == 2 and not line.startswith("#"):
                out[f[0]] = float(f[1])
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        time.sleep(0.15)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.out = self.proc.communicate(timeout=5)[0]
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out = ""

    def summary(self):
        if not self.proc or not getattr(self, "out", ""):
            return None
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in self.out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm), "reasons": sorted(reasons)}


def setup_dist(n_gpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("XN_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return world, rank, local, dist


def make_scene(device: int):
    import torch
    from xenodon_gb300 import cameras, volumes
    t0 = time.time()
    grid = volumes.ct_shell(*DIMS, seed=1, device=f"cuda:{device}")
    gen_s = time.time() - t0
    path = cameras.ct_path(DIMS)
    torch.cuda.synchronize()
    return grid, path, gen_s


def cpu_sample(oracle, grid, nodes, path, frames, row_step, threads):
    """FP32 oracle over every `row_step`-th row of the given frames; returns
    (rays, seconds, per-traversal Mrays/s)."""
    rays, secs = 0, 0.0
    per = {t: [0, 0.0] for t in TRAVERSALS}
    for fi in frames:
        f, u, p = path[fi]
        cam = oracle.make_camera(f, u, p)
        for t in TRAVERSALS:
            for y in range(row_step // 2, HEIGHT, row_step):
                view = oracle.make_view(WIDTH, HEIGHT, EMISSION, output_offset=(0, y), output_extent=(WIDTH, 1))
                t0 = time.perf_counter()
                oracle.render(t, grid=grid if t == "dda" else None, nodes=None if t == "dda" else nodes, camera=cam,
                              view=view, threads=threads, want_loads=False)
                dt = time.perf_counter() - t0
                rays += WIDTH
                secs += dt
                per[t][0] += WIDTH
                per[t][1] += dt
    return rays, secs, {t: (v[0] / v[1] / 1e6 if v[1] else None) for t, v in per.items()}


def run_reference(args):
    world, rank, local, dist = setup_dist(args.gpus)
    if rank != 0:
        return 0
    import oracle
    from xenodon_gb300 import cameras, volumes
    oracle.build()
    grid = volumes.ct_shell(*DIMS, seed=1, device="cpu")
    nodes, st = oracle.build_svo(grid, "rope")
    path = cameras.ct_path(DIMS)
    threads = os.cpu_count() or 1
    row_step = args.ref_row_step
    for fi in frame_indices(args.warmup, offset=7):
        cpu_sample(oracle, grid, nodes, path, [fi], row_step * 4, threads)
    rays, secs, per = 0, 0.0, {}
    times = []
    for fi in frame_indices(args.steps):
        r, s, per = cpu_sample(oracle, grid, nodes, path, [fi], row_step, threads)
        rays += r
        secs += s
        times.append(s)
    value = rays / secs / 1e6
    sample = (f"every {row_step}th row of {args.steps} frames x 5 traversals "
              f"({rays // (5 * args.steps)} rays per traversal per frame)")
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 4), "unit": "Mrays/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1000 * secs / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "resolution": [WIDTH, HEIGHT], "volume": list(DIMS),
                   "traversals": list(TRAVERSALS), "octree_nodes": st["n_nodes"]},
        "per_traversal": {t: (round(v, 4) if v else None) for t, v in per.items()},
        "cpu_baseline": {"value": round(value, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 4), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference's Vulkan shaders need a graphics stack (unavailable on this box); "
                "its algorithm runs as the oracle's FP32 C restatement on all host cores",
    }
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    import xenodon_gb300 as xg
    from xenodon_gb300 import build as native
    world, rank, local, dist = setup_dist(args.gpus)
    torch.cuda.set_device(local)
    native.build()
    grid, path, gen_s = make_scene(local)
    ctx = xg.Context(local)
    t0 = time.time()
    nodes, st = ctx.build_svo(grid, "rope", "chan-diff", 0)
    build_s = time.time() - t0
    vol_grid = ctx.upload_grid(grid)
    vol_svo = ctx.upload_svo(nodes, st["side"])
    vols = {t: (vol_grid if t == "dda" else vol_svo) for t in TRAVERSALS}
    params = xg.make_params(WIDTH, HEIGHT, EMISSION)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    out = torch.empty((HEIGHT, WIDTH), dtype=torch.int32, device="cuda")
    cams = [xg.make_camera(*c) for c in path]

    def step(fi, events=None):
        for ti, t in enumerate(TRAVERSALS):
            if events is not None:
                events[ti][0].record(stream)
            ctx.render_device(vols[t], t, cams[fi], params, out.data_ptr(), None, None, sptr)
            if events is not None:
                events[ti][1].record(stream)

    for fi in frame_indices(args.warmup, offset=3):
        step(fi)
    torch.cuda.synchronize()
    frames = frame_indices(args.steps)
    ev = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)] for _ in TRAVERSALS]
          for _ in frames]
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record(stream)
        for j, fi in enumerate(frames):
            step(fi, ev[j])
        end.record(stream)
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    total_ms = start.elapsed_time(end)
    kern_ms = {t: sum(ev[j][ti][0].elapsed_time(ev[j][ti][1]) for j in range(len(frames)))
               for ti, t in enumerate(TRAVERSALS)}
    if ctx.ray_errors():
        print("warning: rays hit an iteration cap", file=sys.stderr)
    if dist:
        tt = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
    rays_per_frame = WIDTH * HEIGHT
    total_rays = rays_per_frame * len(TRAVERSALS) * len(frames) * world
    value = total_rays / (total_ms * 1e3)
    per = {t: rays_per_frame * len(frames) / (kern_ms[t] * 1e3) for t in TRAVERSALS}

    # algorithmic bytes: 4 B per reference word read + 4 B per pixel store
    loads = torch.empty((HEIGHT, WIDTH), dtype=torch.int32, device="cuda")
    alg_bytes = {}
    for t in TRAVERSALS:
        words = 0
        for fi in frames:
            ctx.render_device(vols[t], t, cams[fi], params, out.data_ptr(), None, loads.data_ptr(), sptr)
            words += int(loads.to(torch.int64).sum().item())
        alg_bytes[t] = 4.0 * words / len(frames) + 4.0 * rays_per_frame
    torch.cuda.synchronize()
    dominant = max(TRAVERSALS, key=lambda t: kern_ms[t])
    peaks = load_peaks()
    avg_ms = kern_ms[dominant] / len(frames)
    achieved = alg_bytes[dominant] / (avg_ms * 1e-3) / 1e9
    traffic = load_traffic().get(dominant)
    per_kernel_roofline = {
        t: {"gbs": round(alg_bytes[t] / (kern_ms[t] / len(frames) * 1e-3) / 1e9, 1),
            "frac": round(alg_bytes[t] / (kern_ms[t] / len(frames) * 1e-3) / 1e9 / peaks["hbm_gbs"], 4),
            "bytes_per_launch": int(alg_bytes[t]), "ms_per_launch": round(kern_ms[t] / len(frames), 4)}
        for t in TRAVERSALS}

    # end to end through the public host-buffer entry point
    host = torch.empty((HEIGHT, WIDTH, 4), dtype=torch.uint8, pin_memory=True).numpy()
    for fi in frame_indices(min(args.warmup, 3), offset=5):
        for t in TRAVERSALS:
            ctx.render(vols[t], t, cams[fi], params, out=host)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for fi in frames:
        for t in TRAVERSALS:
            ctx.render(vols[t], t, cams[fi], params, out=host)
    e2e_s = time.perf_counter() - t0
    if dist:
        tt = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_s = float(tt.item())
    e2e = total_rays / e2e_s / 1e6
    cam_bytes = 36 + 48  # xn_camera + xn_params per launch
    d2h = len(TRAVERSALS) * (rays_per_frame * 4 + 4)

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world, "steps": len(frames),
        "warmup": args.warmup, "ms_per_step": round(total_ms / len(frames), 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "resolution": [WIDTH, HEIGHT], "volume": list(DIMS),
                   "traversals": list(TRAVERSALS), "frames": f"{len(frames)} of {PATH_FRAMES} path frames",
                   "emission_coeff": EMISSION, "octree_nodes": st["n_nodes"],
                   "l2": f"no flush: inputs larger than L2 (grid {grid.nbytes >> 20} MiB, "
                         f"octree {st['n_nodes'] * 40 >> 20} MiB)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "per_traversal": {t: round(v, 2) for t, v in per.items()},
        "roofline": {"bound": "hbm", "kernel": dominant, "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"],
                     "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4),
                     "traffic": traffic, "peak_source": peaks["source"],
                     "algorithmic_bytes_per_launch": int(alg_bytes[dominant])},
        "roofline_per_kernel": per_kernel_roofline,
        "e2e": {"value": round(e2e, 2), "unit": "Mrays/s", "h2d_bytes_per_step": len(TRAVERSALS) * cam_bytes,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": len(frames) * len(TRAVERSALS),
        "clocks": clk.summary(),
        "build": {"svo_build_s": round(build_s, 3), "volume_gen_s": round(gen_s, 2)},
    }
    if rank == 0 and not args.no_cpu_baseline:
        import oracle
        oracle.build()
        threads = os.cpu_count() or 1
        rays, secs, cper = cpu_sample(oracle, grid, nodes, path, frames[:1], args.cpu_row_step, threads)
        line["cpu_baseline"] = {"value": round(rays / secs / 1e6, 4), "unit": "Mrays/s", "cores": threads,
                                "kind": "port",
                                "sample": f"every {args.cpu_row_step}th row of frame {frames[0]}, all 5 traversals "
                                          f"({rays // 5} rays each), FP32 oracle restatement"}
    if rank == 0:
        print(json.dumps(line))
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--cpu-row-step", type=int, default=20)
    ap.add_argument("--ref-row-step", type=int, default=60)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

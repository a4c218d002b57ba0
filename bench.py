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


def load_issue() -> dict:
    """Issue-slot and ALU-pipe use per traversal (fractions of peak) from the
    committed ncu summary, if present: the second bound of the octree
    traversals, which reread their node words from L1."""
    p = ROOT / "profiles" / "issue_ct_1080p.txt"
    out = {}
    if p.exists():
        for line in p.read_text().splitlines():
            f = line.split()
            if len(f) == 3 and not line.startswith("#"):
                out[f[0]] = {"issue_active_frac": round(float(f[1]) / 100, 4),
                             "alu_pipe_frac": round(float(f[2]) / 100, 4)}
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


def aggregate_replicas(total_ms: float, rays_local: int, world: int, dist, device: str = "cpu"):
    """Replicas (one per GPU, no exchange): the timed region of the job is the
    slowest rank's; every rank renders rays_local rays.  Returns (max ms,
    whole-job Mrays/s)."""
    if dist:
        import torch
        t = torch.tensor([total_ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, rays_local * world / (total_ms * 1e3)


def make_scene(device: int):
    import torch
    from xenodon_gb300 import cameras, volumes
    t0 = time.time()
    grid = volumes.ct_shell(*DIMS, seed=1, device=f"cuda:{device}")
    gen_s = time.time() - t0
    path = cameras.ct_path(DIMS)
    torch.cuda.synchronize()
    return grid, path, gen_s


def band_offsets(bands: int, rows: int) -> list[int]:
    """Top rows of `bands` bands of `rows` rows spread evenly over the frame."""
    bands = max(1, min(bands, HEIGHT // rows))
    return [((2 * i + 1) * HEIGHT // (2 * bands) - rows // 2) for i in range(bands)]


def cpu_sample(oracle, grid, nodes, path, frames, bands, rows, threads):
    """FP32 oracle over `bands` bands of `rows` full-width rows per frame and
    traversal, one oracle call (one pool of `threads` threads) per band, so
    the per-call set-up is small next to the band's work.  Returns (rays,
    seconds, per-traversal Mrays/s)."""
    rays, secs = 0, 0.0
    per = {t: [0, 0.0] for t in TRAVERSALS}
    for fi in frames:
        f, u, p = path[fi]
        cam = oracle.make_camera(f, u, p)
        for t in TRAVERSALS:
            for y in band_offsets(bands, rows):
                view = oracle.make_view(WIDTH, HEIGHT, EMISSION, output_offset=(0, y), output_extent=(WIDTH, rows))
                t0 = time.perf_counter()
                oracle.render(t, grid=grid if t == "dda" else None, nodes=None if t == "dda" else nodes, camera=cam,
                              view=view, threads=threads, want_loads=False)
                dt = time.perf_counter() - t0
                rays += WIDTH * rows
                secs += dt
                per[t][0] += WIDTH * rows
                per[t][1] += dt
    return rays, secs, {t: (v[0] / v[1] / 1e6 if v[1] else None) for t, v in per.items()}


def cpu_baseline_line(oracle, grid, nodes, path, frames, bands, rows, single_rows):
    """All host cores on `bands` bands of `rows` rows per frame, and one core
    on one band of `single_rows` rows of the first frame, per traversal."""
    threads = os.cpu_count() or 1
    rays, secs, per = cpu_sample(oracle, grid, nodes, path, frames, bands, rows, threads)
    r1, s1, per1 = cpu_sample(oracle, grid, nodes, path, frames[:1], 1, single_rows, 1)
    return {"value": round(rays / secs / 1e6, 4), "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{min(bands, HEIGHT // rows)} bands of {rows} rows x {WIDTH} px per frame and traversal, "
                      f"{len(frames)} frame(s) ({rays // (5 * len(frames))} rays per traversal per frame), "
                      f"FP32 oracle restatement, one call per band",
            "seconds": round(secs, 2),
            "per_traversal": {t: (round(v, 4) if v else None) for t, v in per.items()},
            "single_core": {"value": round(r1 / s1 / 1e6, 4), "cores": 1, "seconds": round(s1, 2),
                            "sample": f"one band of {single_rows} rows of frame {frames[0]} per traversal",
                            "per_traversal": {t: (round(v, 4) if v else None) for t, v in per1.items()}}}


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
    for fi in frame_indices(args.warmup, offset=7):
        cpu_sample(oracle, grid, nodes, path, [fi], 1, 16, threads)
    rays, secs, per = 0, 0.0, {}
    times = []
    acc = {t: [0, 0.0] for t in TRAVERSALS}
    for fi in frame_indices(args.steps):
        r, s, p = cpu_sample(oracle, grid, nodes, path, [fi], args.ref_bands, args.band_rows, threads)
        rays += r
        secs += s
        times.append(s)
        for t in TRAVERSALS:
            if p[t]:
                acc[t][0] += r // len(TRAVERSALS)
                acc[t][1] += (r // len(TRAVERSALS)) / (p[t] * 1e6)
    per = {t: (v[0] / v[1] / 1e6 if v[1] else None) for t, v in acc.items()}
    value = rays / secs / 1e6
    sample = (f"{args.ref_bands} bands of {args.band_rows} rows x {WIDTH} px of each of {args.steps} frames x 5 "
              f"traversals ({rays // (5 * args.steps)} rays per traversal per frame), one oracle call per band")
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


def measure_batched(ctx, xg, args):
    """Many cameras in one persistent launch vs one launch per frame.

    The 1024^3 gas-field workload: a log-normal density field (P(k) ~ k^-2.5,
    seed 2) built into a rope octree on the device, rendered with esvo and
    svo-rope from 64 cameras on a Fibonacci sphere at 1.8x the extent, 45 deg
    vertical field of view, 1920x1080."""
    import torch
    from xenodon_gb300 import cameras, volumes
    n = args.batched_size
    t0 = time.time()
    g = volumes.gas_field(n, seed=2, device="cuda", as_tensor=True)
    vol, st = ctx.build_svo_volume(g.data_ptr(), (n, n, n), "rope")
    build_s = time.time() - t0
    grid_vol = ctx.upload_grid_device(g.data_ptr(), (n, n, n))
    dda4k = measure_dda_4k(ctx, xg, None, n, vol=grid_vol)
    del g
    torch.cuda.empty_cache()
    w, h = 1920, 1080
    cams = cameras.fibonacci_sphere(args.batched_cameras, np.array([0.5, 0.5, 0.5]), 1.8,
                                    cameras.forward_length_for_vfov(45.0, w, h))
    params = xg.make_params(w, h, EMISSION)
    trav = ("esvo", "svo-rope")
    specs = [(vol, t, xg.make_camera(*c), params) for t in trav for c in cams]
    bufs = [torch.empty((h, w), dtype=torch.int32, device="cuda") for _ in specs]
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    rays = w * h * len(specs)

    def plain():
        for (v, t, c, p), b in zip(specs, bufs):
            ctx.render_device(v, t, c, p, b.data_ptr(), None, None, sptr)

    def timed(fn, reps=2):
        fn()
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        return best

    plain_ms = timed(plain)
    plain_out = [b.clone() for b in bufs[:: max(1, len(bufs) // 8)]]
    jobs = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(specs, bufs))
    # the autotuner samples the whole batch, then times its finalists on all of it
    best, _ = ctx.autotune_batch(jobs, len(specs), sptr)
    for b in bufs:
        b.fill_(-1)
    if best.tile_width:  # a persistent-kernel shape: replayed as a CUDA graph
        graph = ctx.batch_graph(len(specs), best, sptr)
        batched_ms = timed(lambda: graph.launch(jobs, len(specs)))
        graph.close()
    else:  # the plain form won
        batched_ms = timed(lambda: ctx.render_batch(jobs, len(specs), best, sptr))
    same = all(torch.equal(a, b) for a, b in zip(plain_out, bufs[:: max(1, len(bufs) // 8)]))
    small = batched_small_frames(ctx, xg, vol, timed, args)
    args.residents.append({"grid": grid_vol, "svo": vol, "dims": (n, n, n), "rope": True})
    return {
        "workload": f"{n}^3 gas field, rope octree, esvo+svo-rope, {len(cams)} Fibonacci-sphere cameras at 1.8x, "
                    f"45 deg VFOV, {w}x{h}",
        "octree_nodes": st["n_nodes"], "volume_build_s": round(build_s, 2), "frames": len(specs),
        "plain_ms": round(plain_ms, 3), "batched_ms": round(batched_ms, 3),
        "plain_mrays_s": round(rays / (plain_ms * 1e3), 1), "batched_mrays_s": round(rays / (batched_ms * 1e3), 1),
        "speedup": round(plain_ms / batched_ms, 3), "identical_images": bool(same), "launch_shape": best.as_dict(),
        "small_frames": small,
        "dda_4k": dda4k,
    }


def batched_small_frames(ctx, xg, vol, timed, args):
    """The same octree and traversals at 256x256 from 256 cameras: frames too
    small to fill the GPU one launch at a time, the case batching is for."""
    import torch
    from xenodon_gb300 import cameras
    w = h = 256
    cams = cameras.fibonacci_sphere(4 * args.batched_cameras, np.array([0.5, 0.5, 0.5]), 1.8,
                                    cameras.forward_length_for_vfov(45.0, w, h))
    params = xg.make_params(w, h, EMISSION)
    specs = [(vol, t, xg.make_camera(*c), params) for t in ("esvo", "svo-rope") for c in cams]
    bufs = [torch.empty((h, w), dtype=torch.int32, device="cuda") for _ in specs]
    sptr = torch.cuda.current_stream().cuda_stream

    def plain():
        for (v, t, c, p), b in zip(specs, bufs):
            ctx.render_device(v, t, c, p, b.data_ptr(), None, None, sptr)

    plain_ms = timed(plain)
    keep = [b.clone() for b in bufs[::16]]
    jobs = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(specs, bufs))
    best, _ = ctx.autotune_batch(jobs, len(specs), sptr)
    for b in bufs:
        b.fill_(-1)
    batched_ms = timed(lambda: ctx.render_batch(jobs, len(specs), best, sptr))
    same = all(torch.equal(a, b) for a, b in zip(keep, bufs[::16]))
    rays = w * h * len(specs)
    return {"frames": len(specs), "resolution": [w, h], "plain_mrays_s": round(rays / (plain_ms * 1e3), 1),
            "batched_mrays_s": round(rays / (batched_ms * 1e3), 1), "speedup": round(plain_ms / batched_ms, 3),
            "identical_images": bool(same), "launch_shape": best.as_dict()}


def measure_dda_4k(ctx, xg, g, n, vol=None):
    """Plain DDA on the n^3 gas-field grid at 3840x2160 from 8 orbit cameras at
    2x the extent: Mrays/s and the fraction of the HBM roofline (4 B per texel
    the reference reads + 4 B per pixel, over the measured HBM copy bandwidth).
    `vol`: an already resident grid volume (kept), else one is made from g."""
    import torch
    from xenodon_gb300 import cameras
    own = vol is None
    if own:
        vol = ctx.upload_grid_device(g.data_ptr(), (n, n, n))
    w, h = 3840, 2160
    params = xg.make_params(w, h, EMISSION)
    cams = [xg.make_camera(*c) for c in cameras.orbit(np.array([0.5, 0.5, 0.5]), 2.0, 8)]
    out = torch.empty((h, w), dtype=torch.int32, device="cuda")
    loads = torch.empty((h, w), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    for c in cams[:3]:
        ctx.render_device(vol, "dda", c, params, out.data_ptr(), None, None, sptr)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in cams]
    for c, (a, b) in zip(cams, evs):
        a.record(stream)
        ctx.render_device(vol, "dda", c, params, out.data_ptr(), None, None, sptr)
        b.record(stream)
    torch.cuda.synchronize()
    ms = [a.elapsed_time(b) for a, b in evs]
    words = 0
    for c in cams:
        ctx.render_device(vol, "dda", c, params, out.data_ptr(), None, loads.data_ptr(), sptr)
        words += int(loads.to(torch.int64).sum().item())
    torch.cuda.synchronize()
    if own:
        vol.release()
    total_ms = sum(ms)
    alg = 4.0 * words + 4.0 * w * h * len(cams)
    gbs = alg / (total_ms * 1e-3) / 1e9
    peak = load_peaks()["hbm_gbs"]
    return {"workload": f"dda, {n}^3 gas-field grid, {w}x{h}, 8 orbit cameras at 2x the extent",
            "ms_per_frame": round(total_ms / len(cams), 4), "mrays_s": round(w * h * len(cams) / (total_ms * 1e3), 1),
            "algorithmic_gbs": round(gbs, 1), "hbm_frac": round(gbs / peak, 4),
            "texels_per_ray": round(words / (w * h * len(cams)), 1)}


def measure_c3(ctx, xg, args):
    """The 2048^3 workload: a 32 GiB gas-field grid (seed 3, the 1024^3
    recipe) and its octree, DDA and esvo at 3840x2160 along a 150-frame orbit
    at 2x the extent; one launch per frame vs the autotuned persistent batch.

    The octree has about 0.93 nodes per voxel (8e9 here), beyond the 32-bit
    indices of the reference's node array and beyond HBM at 40 bytes a node,
    so it is built lean: straight into the device layout (36 bytes per
    internal node, leaf colours inline), which esvo reads."""
    import torch
    from xenodon_gb300 import cameras, volumes
    n = args.c3_size
    free, _ = torch.cuda.mem_get_info()
    need = 5.5 * n ** 3 * 4  # grid + texture + build scratch + octree at the build's peak
    if free < need:
        return {"skipped": f"{free / 2**30:.0f} GiB free, {need / 2**30:.0f} GiB wanted"}
    t0 = time.time()
    g = volumes.gas_field(n, seed=3, device="cuda", as_tensor=True)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    gen_s = time.time() - t0
    t0 = time.time()
    grid_vol = ctx.upload_grid_device(g.data_ptr(), (n, n, n))
    upload_s = time.time() - t0
    t0 = time.time()
    svo_vol, st = ctx.build_svo_volume(g.data_ptr(), (n, n, n), "sparse", lean=True)
    build_s = time.time() - t0
    del g
    torch.cuda.empty_cache()
    w, h = 3840, 2160
    params = xg.make_params(w, h, EMISSION)
    path = cameras.orbit(np.array([0.5, 0.5, 0.5]), 2.0, 150)
    frames = path[:: max(1, len(path) // args.c3_frames)][: args.c3_frames]
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    result = {"workload": f"{n}^3 gas field (seed 3) grid + lean sparse octree, dda and esvo at {w}x{h}, "
                          f"{len(frames)} frames of a 150-frame orbit at 2x the extent",
              "field_gen_s": round(gen_s, 2), "texture_upload_s": round(upload_s, 2),
              "octree_build_s": round(build_s, 2), "octree_nodes": st["n_nodes"],
              "octree_device_bytes": svo_vol.info()["device_bytes"], "octree_depth": st["depth"]}
    result["dda_4k"] = measure_dda_4k(ctx, xg, None, n, vol=grid_vol)

    def timed(fn, reps=2):
        fn()
        torch.cuda.synchronize()
        best = None
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        return best

    for trav, vol in (("dda", grid_vol), ("esvo", svo_vol)):
        specs = [(vol, trav, xg.make_camera(*c), params) for c in frames]
        bufs = [torch.empty((h, w), dtype=torch.int32, device="cuda") for _ in specs]

        def plain():
            for (v, t, c, p), b in zip(specs, bufs):
                ctx.render_device(v, t, c, p, b.data_ptr(), None, None, sptr)

        plain_ms = timed(plain)
        keep = [b.clone() for b in bufs[::4]]
        jobs = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(specs, bufs))
        untuned_ms = timed(lambda: ctx.render_batch(jobs, len(specs), xg.BatchConfig(8, 128, 0, 1), sptr), reps=1)
        best, _ = ctx.autotune_batch(jobs, len(specs), sptr)
        for b in bufs:
            b.fill_(-1)
        tuned_ms = timed(lambda: ctx.render_batch(jobs, len(specs), best, sptr))
        same = all(torch.equal(a, b) for a, b in zip(keep, bufs[::4]))
        rays = w * h * len(specs)
        result[trav] = {"plain_mrays_s": round(rays / (plain_ms * 1e3), 1),
                        "batch_untuned_mrays_s": round(rays / (untuned_ms * 1e3), 1),
                        "batch_autotuned_mrays_s": round(rays / (tuned_ms * 1e3), 1),
                        "autotuned_vs_plain": round(plain_ms / tuned_ms, 3), "launch_shape": best.as_dict(),
                        "identical_images": bool(same)}
        del bufs, keep
    torch.cuda.empty_cache()
    args.residents.append({"grid": grid_vol, "svo": svo_vol, "dims": (n, n, n), "rope": False})
    return result


def measure_small_dda(ctx, xg, args):
    """The reference's CPU-runnable case: plain DDA on the 128^3 blob grid
    (16 Gaussian blobs, seed 0), one 512x512 frame from the camera line
    `0 0 -0.8660254 0 1 0 0.5 0.5 2.5` (2x the extent on +z, 60 deg vertical
    field of view); the GPU kernel beside the FP32 oracle on all host cores."""
    import torch
    import oracle
    from xenodon_gb300 import volumes
    g = volumes.blobs(128, seed=0)
    vol = ctx.upload_grid(g)
    cam_t = ((0.0, 0.0, -0.8660254), (0.0, 1.0, 0.0), (0.5, 0.5, 2.5))
    cam = xg.make_camera(*cam_t)
    p = xg.make_params(512, 512, EMISSION)
    out = torch.empty((512, 512), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    for _ in range(3):
        ctx.render_device(vol, "dda", cam, p, out.data_ptr(), None, None, stream.cuda_stream)
    torch.cuda.synchronize()
    reps = 200
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        ctx.render_device(vol, "dda", cam, p, out.data_ptr(), None, None, stream.cuda_stream)
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / reps
    rgba, _, _ = ctx.render(vol, "dda", cam, p)
    vol.release()
    oracle.build()
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    ref = oracle.render("dda", grid=g, camera=oracle.make_camera(*cam_t), view=oracle.make_view(512, 512, EMISSION),
                        threads=threads, want_loads=False)
    cpu_s = time.perf_counter() - t0
    diff = int(np.abs(rgba.astype(np.int32) - ref["rgba"].astype(np.int32)).max())
    return {"workload": "dda, 128^3 blob grid (seed 0), 512x512, camera 2x the extent on +z, 60 deg VFOV",
            "gpu_ms_per_frame": round(ms, 4), "gpu_mrays_s": round(512 * 512 / ms / 1e3, 1),
            "cpu_oracle_mrays_s": round(512 * 512 / cpu_s / 1e6, 3), "cpu_threads": threads,
            "max_rgba_diff_vs_oracle": diff}


def measure_headless(xg, nodes, side, path):
    """The `xenodon render --headless` loop on the CT rope octree, esvo at
    1920x1080, 24 frames of the path written as PNG files: frames per second
    with the two output sets (frame n+1 renders while frame n is composited
    and encoded) against XN_HEADLESS_SERIAL=1 (render, wait, save, in turn, as
    the reference does), and with --discard-output."""
    import re
    import tempfile
    from xenodon_gb300 import cameras
    result = {"workload": "xenodon render --headless, CT rope octree, esvo, 1920x1080, 24 path frames, PNG output"}
    with tempfile.TemporaryDirectory() as d:
        xg.svo_save(Path(d) / "ct.svo", nodes, side)
        cameras.write_script(Path(d) / "cam.txt", [path[i] for i in range(0, PATH_FRAMES, PATH_FRAMES // 24)][:24])
        (Path(d) / "h.conf").write_text("device {\n vkindex = 0\n offset = (0, 0)\n extent = (1920, 1080)\n}\n")
        for mode, extra, env_serial in (("pipelined", ["--output", "f-{}.png"], False),
                                        ("serial", ["--output", "g-{}.png"], True),
                                        ("discard", ["--discard-output"], False)):
            env = dict(os.environ)
            env.pop("XN_HEADLESS_SERIAL", None)
            if env_serial:
                env["XN_HEADLESS_SERIAL"] = "1"
            p = subprocess.run([str(xg.CLI_PATH), "render", "--headless", "h.conf", "ct.svo", "-s", "esvo", "-e",
                                str(EMISSION), "--camera", "cam.txt", *extra], cwd=d, env=env, capture_output=True,
                               text=True, timeout=600)
            m = re.search(r"frames: (\d+), fps: ([0-9.eE+-]+)", p.stdout)
            result[mode + "_fps"] = float(m.group(2)) if (p.returncode == 0 and m) else None
        sizes = [f.stat().st_size for f in Path(d).glob("f-*.png")]
        result["png_mb_per_frame"] = round(sum(sizes) / max(1, len(sizes)) / 2**20, 2)
    return result


def measure_serving(ctx, xg, args, scene, residents, server_kw=None):
    """Continuous batching of the serving mix vs one frame per launch.

    Volumes: the 128^3 blob grid and its octree, the CT grid and octree (both
    registered as host data, evictable), and when present the 1024^3 and
    2048^3 gas-field grids and octrees, resident on the device (never
    evicted); a 150 GB HBM budget.  Each request draws a volume uniformly, a
    traversal uniformly from those valid for it (dda on the grid, the octree
    variants on the octree; no svo-rope on the lean 2048^3 tree), a
    resolution from {256^2, 512^2, 1280x720, 1920x1080, 3840x2160} and a
    camera on a sphere at 1.2-3x the extent; arrivals are Poisson at each
    swept rate (seed 4).  Plain latency: the same arrivals served one frame
    per launch in arrival order, from the measured plain render times."""
    from xenodon_gb300 import cameras, volumes
    rng = np.random.default_rng(4)
    blobs = volumes.blobs(128, seed=0)
    bnodes, bst = ctx.build_svo(blobs, "rope", "chan-diff", 0)
    ct_grid, ct_nodes, ct_side = scene
    host = {1: ("grid", blobs), 2: ("svo", (bnodes, bst["side"])), 3: ("grid", ct_grid), 4: ("svo", (ct_nodes, ct_side))}
    configs = [{"grid": 1, "svo": 2, "dims": blobs.shape[2::-1], "rope": True},
               {"grid": 3, "svo": 4, "dims": ct_grid.shape[2::-1], "rope": True}]
    resident = {}
    vid = 5
    for r in residents:
        resident[vid], resident[vid + 1] = r["grid"], r["svo"]
        configs.append({"grid": vid, "svo": vid + 1, "dims": r["dims"], "rope": r["rope"]})
        vid += 2
    res = [(256, 256), (512, 512), (1280, 720), (1920, 1080), (3840, 2160)]

    def draw():
        cfg = configs[int(rng.integers(0, len(configs)))]
        travs = ["dda", "svo-naive", "esvo", "svo-df"] + (["svo-rope"] if cfg["rope"] else [])
        trav = travs[int(rng.integers(0, len(travs)))]
        v = cfg["grid"] if trav == "dda" else cfg["svo"]
        w, h = res[int(rng.integers(0, len(res)))]
        centre = cameras.volume_centre(cfg["dims"]) if trav == "dda" else np.array([0.5, 0.5, 0.5])
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        cam = cameras.look_at(centre + d * rng.uniform(1.2, 3.0), centre)
        return v, trav, cam, xg.make_params(w, h, EMISSION)

    n_req = args.serve_requests
    reqs = [draw() for _ in range(n_req)]
    # plain: one frame per launch, back to back, into the callers' buffers
    handles = dict(resident)
    for v, (kind, d) in host.items():
        handles[v] = ctx.upload_grid(d) if kind == "grid" else ctx.upload_svo(d[0], d[1])
    outs = [np.empty((p.output_region.height, p.output_region.width, 4), np.uint8) for _, _, _, p in reqs]
    for v, t, c, p in reqs[:5]:
        ctx.render(handles[v], t, xg.make_camera(*c), p)
    durations = []
    t0 = time.perf_counter()
    for (v, t, c, p), o in zip(reqs, outs):
        a = time.perf_counter()
        ctx.render(handles[v], t, xg.make_camera(*c), p, out=o)
        durations.append(time.perf_counter() - a)
    plain_s = time.perf_counter() - t0
    rays = sum(p.output_region.width * p.output_region.height for _, _, _, p in reqs)
    for v in host:
        handles[v].release()
    result = {"workload": "request mix over the 128^3 blob, CT, 1024^3 and 2048^3 gas-field grids and octrees "
                          f"({len(configs)} volumes); resolutions 256^2..3840x2160; cameras at 1.2-3x the extent; "
                          "150 GB HBM budget",
              "requests": n_req, "plain_mrays_s": round(rays / plain_s / 1e6, 1), "rates": []}
    for rate in args.serve_rates:
        gaps = rng.exponential(1.0 / rate, n_req) if rate > 0 else np.zeros(n_req)
        arrivals = np.cumsum(gaps)
        # the same arrivals served plainly: one frame at a time, in order
        finish, lat = 0.0, []
        for arr, dur in zip(arrivals, durations):
            finish = max(finish, arr) + dur
            lat.append((finish - arr) * 1e3)
        with xg.Server(ctx, hbm_budget=150 << 30, **(server_kw or {})) as srv:
            for v, (kind, d) in host.items():
                if kind == "grid":
                    srv.add_grid(v, d)
                else:
                    srv.add_svo(v, d[0], d[1])
            for v, h in resident.items():
                srv.add_volume(v, h)
            tickets = []
            start = time.perf_counter()
            for (v, t, c, p), arr in zip(reqs, arrivals):
                while time.perf_counter() < start + arr:
                    pass
                tickets.append(srv.submit(v, t, xg.make_camera(*c), p))
            same = True
            for i, tk in enumerate(tickets):
                img, _ = srv.wait(tk, timeout=300)
                if i % 17 == 0:
                    same &= bool(np.array_equal(img, outs[i]))
            st = srv.stats()
        result["rates"].append({"offered_req_s": rate if rate > 0 else "closed", "p50_ms": round(st["p50_ms"], 3),
                                "p99_ms": round(st["p99_ms"], 3), "mrays_s": round(st["mrays_per_s"], 1),
                                "mean_batch": round(st["mean_batch"], 2), "folded": st["folded"],
                                "fold_launches": st["fold_launches"], "republished": st["republished"],
                                "identical_images": same,
                                "plain_p50_ms": round(float(np.percentile(lat, 50)), 3),
                                "plain_p99_ms": round(float(np.percentile(lat, 99)), 3)})
    sat = max(r["mrays_s"] for r in result["rates"])
    result["served_vs_plain"] = round(sat / result["plain_mrays_s"], 3)
    return result


def measure_svo_4k(ctx, xg, vol, n, trav, frames=4):
    """One octree traversal at 3840x2160 on a resident n^3 gas-field octree
    from `frames` orbit cameras at 2x the extent: Mrays/s, node words the
    reference would read per ray, and those words' bytes per second."""
    import torch
    from xenodon_gb300 import cameras
    w, h = 3840, 2160
    params = xg.make_params(w, h, EMISSION)
    cams = [xg.make_camera(*c) for c in cameras.orbit(np.array([0.5, 0.5, 0.5]), 2.0, frames)]
    out = torch.empty((h, w), dtype=torch.int32, device="cuda")
    loads = torch.empty((h, w), dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    ctx.render_device(vol, trav, cams[0], params, out.data_ptr(), None, None, sptr)
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in cams]
    for c, (a, b) in zip(cams, evs):
        a.record(stream)
        ctx.render_device(vol, trav, c, params, out.data_ptr(), None, None, sptr)
        b.record(stream)
    torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in evs)
    words = 0
    for c in cams:
        ctx.render_device(vol, trav, c, params, out.data_ptr(), None, loads.data_ptr(), sptr)
        words += int(loads.to(torch.int64).sum().item())
    torch.cuda.synchronize()
    rays = w * h * len(cams)
    alg = 4.0 * words + 4.0 * rays
    return {"workload": f"{trav}, {n}^3 gas-field octree, {w}x{h}, {len(cams)} orbit cameras at 2x the extent",
            "ms_per_frame": round(ms / len(cams), 3), "mrays_s": round(rays / (ms * 1e3), 1),
            "words_per_ray": round(words / rays, 1), "algorithmic_gbs": round(alg / (ms * 1e-3) / 1e9, 1)}


def run_svo_4k_only(args):
    """--svo-4k N: the lean sparse octree of the N^3 gas field (the seed-3
    recipe), octree traversals at 3840x2160 (profiling the large-tree
    traversals on a stand-in of the 2048^3 tree)."""
    import torch
    import xenodon_gb300 as xg
    from xenodon_gb300 import build as native, volumes
    native.build()
    ctx = xg.Context(0)
    n = args.svo_4k
    g = volumes.gas_field(n, seed=3, device="cuda", as_tensor=True)
    vol, st = ctx.build_svo_volume(g.data_ptr(), (n, n, n), "sparse", lean=True)
    del g
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    line = {"octree_nodes": st["n_nodes"], "device_bytes": vol.info()["device_bytes"]}
    for trav in args.svo_4k_traversals:
        line[trav] = measure_svo_4k(ctx, xg, vol, n, trav)
    print(json.dumps(line))
    vol.release()
    ctx.close()
    return 0


def run_serve_only(args):
    """--serve-only: the serving mix alone, once per --serve-variants entry
    (server settings as key=value pairs, e.g. band_pixels=524288,streams=3;
    an empty entry is the defaults).  Volumes: the CT scene, and with
    --c3-size the 1024^3 gas field (seed 2, rope octree) and the 2048^3 one
    (seed 3, lean sparse octree) with their grids, resident on the device."""
    import torch
    import xenodon_gb300 as xg
    from xenodon_gb300 import build as native, volumes
    native.build()
    ctx = xg.Context(0)
    grid, _, _ = make_scene(0)
    nodes, st = ctx.build_svo(grid, "rope", "chan-diff", 0)
    residents = []
    if args.c3_size:
        for n, seed, lean in ((args.batched_size, 2, False), (args.c3_size, 3, True)):
            g = volumes.gas_field(n, seed=seed, device="cuda", as_tensor=True)
            torch.cuda.synchronize()
            torch.cuda.empty_cache()  # the generator's temporaries, before the build's scratch
            grid_vol = ctx.upload_grid_device(g.data_ptr(), (n, n, n))
            svo_vol, _ = (ctx.build_svo_volume(g.data_ptr(), (n, n, n), "sparse", lean=True) if lean
                          else ctx.build_svo_volume(g.data_ptr(), (n, n, n), "rope"))
            del g
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
            residents.append({"grid": grid_vol, "svo": svo_vol, "dims": (n, n, n), "rope": not lean})
    out = {}
    for v in args.serve_variants:
        kw = {k: int(x) for k, x in (p.split("=") for p in v.split(",") if p)}
        out[v or "default"] = measure_serving(ctx, xg, args, (grid, nodes, st["side"]), residents, kw)
    print(json.dumps(out))
    for r in residents:
        r["grid"].release()
        r["svo"].release()
    ctx.close()
    return 0


def run_batch_only(args):
    """--batch-only: 512 frames of 256x256 (256 Fibonacci cameras, esvo and
    svo-rope) of the CT volume's rope octree in one persistent launch per
    traversal form (profiling the batch kernel on a small case)."""
    import torch
    import xenodon_gb300 as xg
    from xenodon_gb300 import build as native, cameras, volumes
    native.build()
    ctx = xg.Context(0)
    grid = volumes.ct_shell(*DIMS, seed=1, device="cuda")
    nodes, st = ctx.build_svo(grid, "rope", "chan-diff", 0)
    vol = ctx.upload_svo(nodes, st["side"])
    w = h = 256
    cams = cameras.fibonacci_sphere(256, cameras.volume_centre(DIMS), 1.8, cameras.forward_length_for_vfov(45.0, w, h))
    params = xg.make_params(w, h, EMISSION)
    specs = [(vol, t, xg.make_camera(*c), params) for t in ("esvo", "svo-rope") for c in cams]
    bufs = [torch.empty((h, w), dtype=torch.int32, device="cuda") for _ in specs]
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    jobs = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(specs, bufs))
    cfg = xg.BatchConfig(8, 256, 0, 1)
    for _ in range(2):
        ctx.render_batch(jobs, len(specs), cfg, sptr)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    ctx.render_batch(jobs, len(specs), cfg, sptr)
    b.record(stream)
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    print(json.dumps({"workload": "CT rope octree, esvo + svo-rope, 512 frames of 256x256, batch 8x4 tiles, "
                                  "blocks of 256, queue chunk 1",
                      "ms": round(ms, 3), "mrays_s": round(w * h * len(specs) / (ms * 1e3), 1)}))
    vol.release()
    ctx.close()
    return 0


def run_dda_4k_only(args):
    import torch
    import xenodon_gb300 as xg
    from xenodon_gb300 import build as native, volumes
    native.build()
    ctx = xg.Context(0)
    g = volumes.gas_field(args.dda_4k, seed=2, device="cuda", as_tensor=True)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    line = {}
    for form in args.dda_4k_forms:  # the grid's form on the device is chosen at upload
        os.environ.pop("XN_GRID_LAYOUT", None)
        os.environ.pop("XN_DDA_WARP_TILE", None)
        os.environ.pop("XN_DDA_LSU_SHARE", None)
        os.environ.pop("XN_TEX_READ", None)
        if form in ("bricked", "linear"):
            os.environ["XN_GRID_LAYOUT"] = form
        elif form.startswith("hybrid"):  # hybridK: one warp in K reads the x-fastest copy
            os.environ["XN_GRID_LAYOUT"] = "hybrid"
            os.environ["XN_DDA_LSU_SHARE"] = form[len("hybrid"):] or "4"
        elif form.startswith("texture-w"):
            os.environ["XN_DDA_WARP_TILE"] = form[len("texture-w"):]
        elif form in ("raw", "packed"):  # texel bytes converted in the kernel
            os.environ["XN_TEX_READ"] = form
        line[form] = measure_dda_4k(ctx, xg, g, args.dda_4k)
    for k in ("XN_GRID_LAYOUT", "XN_DDA_WARP_TILE", "XN_DDA_LSU_SHARE", "XN_TEX_READ"):
        os.environ.pop(k, None)
    print(json.dumps(line))
    ctx.close()
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
    # the same build from a device copy of the grid, kept on the device (no
    # host copies): best of 3
    g_dev = torch.from_numpy(grid).to(f"cuda:{local}")
    dev_build_s = None
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        v, _ = ctx.build_svo_volume(g_dev.data_ptr(), (grid.shape[2], grid.shape[1], grid.shape[0]), "rope")
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        v.release()
        dev_build_s = dt if dev_build_s is None else min(dev_build_s, dt)
    del g_dev
    torch.cuda.empty_cache()
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
    rays_per_frame = WIDTH * HEIGHT
    total_rays = rays_per_frame * len(TRAVERSALS) * len(frames) * world
    total_ms, value = aggregate_replicas(total_ms, rays_per_frame * len(TRAVERSALS) * len(frames), world, dist,
                                         "cuda")
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
    for t, r in per_kernel_roofline.items():
        if r["frac"] > 1.0:
            r["note"] = ("above 1: the algorithmic bytes are the reference's reads, most of which this kernel "
                         "skips or takes from L1; DRAM traffic per launch is in `traffic`, the bound in `issue`")
        r["traffic"] = load_traffic().get(t)

    # end to end through the public host-buffer entry points, every frame in
    # the caller's host buffer: xn_output (the asynchronous read-back of the
    # headless outputs; two outputs in turn, so each frame's copy and the
    # host's take of it overlap the next render) and xn_render (synchronous)
    host = torch.empty((HEIGHT, WIDTH, 4), dtype=torch.uint8, pin_memory=True).numpy()
    outs = [xg.Output(ctx, WIDTH * HEIGHT) for _ in range(2)]

    def pipelined(frame_list):
        pending = None
        for i, (fi, t) in enumerate((fi, t) for fi in frame_list for t in TRAVERSALS):
            o = outs[i % 2]
            o.render(vols[t], t, cams[fi], params)
            if pending is not None:
                pending.wait(out=host)
            pending = o
        pending.wait(out=host)

    def synchronous(frame_list):
        for fi in frame_list:
            for t in TRAVERSALS:
                ctx.render(vols[t], t, cams[fi], params, out=host)

    def timed_e2e(fn):
        fn(frame_indices(min(args.warmup, 3), offset=5))
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        fn(frames)
        secs = time.perf_counter() - t0
        if dist:
            tt = torch.tensor([secs], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            secs = float(tt.item())
        return total_rays / secs / 1e6

    e2e = timed_e2e(pipelined)
    e2e_sync = timed_e2e(synchronous)
    for o in outs:
        o.close()
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
        # algorithmic bytes count every reference word a ray reads; the
        # octree walks reread their words from L1, so their fractions are
        # not DRAM use (svo-naive, restarting from the root, is above 1) and
        # issue slots bound them: the figures of the ncu capture
        "issue": {"source": "ncu, profiles/issue_ct_1080p.txt", "per_kernel": load_issue()},
        "e2e": {"value": round(e2e, 2), "unit": "Mrays/s", "h2d_bytes_per_step": len(TRAVERSALS) * cam_bytes,
                "d2h_bytes_per_step": d2h, "api": "xn_output_render / xn_output_wait, two outputs in turn",
                "synchronous_xn_render": round(e2e_sync, 2)},
        "gpu_launches": len(frames) * len(TRAVERSALS),
        "clocks": clk.summary(),
        "build": {"svo_build_s": round(build_s, 3), "volume_gen_s": round(gen_s, 2),
                  # 4 B per voxel read + 40 B per node written, over the whole call (host grid in,
                  # host nodes out, copies included)
                  "algorithmic_gbs": round((4.0 * grid.size / 4 + 40.0 * st["n_nodes"]) / build_s / 1e9, 2),
                  "voxels_per_s": round(grid.size / 4 / build_s, 1),
                  # the device build alone (device grid in, device octree out)
                  "device_build_s": round(dev_build_s, 4),
                  "device_algorithmic_gbs": round((4.0 * grid.size / 4 + 40.0 * st["n_nodes"]) / dev_build_s / 1e9,
                                                  1)},
    }
    if rank == 0 and not args.no_extras:
        # the 1024^3 and 2048^3 volumes stay resident for the serving mix
        args.residents = []
        extras = [("headless", lambda: measure_headless(xg, nodes, st["side"], path)),
                  ("small_dda", lambda: measure_small_dda(ctx, xg, args)),
                  ("batched", lambda: measure_batched(ctx, xg, args))]
        if args.c3_size:
            extras.append(("large", lambda: measure_c3(ctx, xg, args)))
        extras.append(("serving", lambda: measure_serving(ctx, xg, args, (grid, nodes, st["side"]), args.residents)))
        for key, fn in extras:
            try:
                line[key] = fn()
            except Exception as exc:  # the headline line is printed regardless
                line[key] = {"error": f"{type(exc).__name__}: {exc}"}
        for r in args.residents:
            r["grid"].release()
            r["svo"].release()
        torch.cuda.empty_cache()
    if rank == 0 and not args.no_cpu_baseline:
        import oracle
        oracle.build()
        line["cpu_baseline"] = cpu_baseline_line(oracle, grid, nodes, path, frames[:args.cpu_frames], args.cpu_bands,
                                                 args.band_rows, args.single_core_rows)
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
    ap.add_argument("--band-rows", type=int, default=64, help="rows per oracle call of the CPU legs")
    ap.add_argument("--cpu-bands", type=int, default=16, help="bands per frame and traversal of cpu_baseline")
    ap.add_argument("--cpu-frames", type=int, default=6,
                    help="frames of cpu_baseline (with 16 bands: about 10 s on 16 cores)")
    ap.add_argument("--single-core-rows", type=int, default=8, help="rows of the single-core cpu_baseline band")
    ap.add_argument("--ref-bands", type=int, default=3, help="bands per frame and traversal of --impl reference")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and serving measurements")
    ap.add_argument("--batched-size", type=int, default=1024)
    ap.add_argument("--batched-cameras", type=int, default=64)
    ap.add_argument("--c3-size", type=int, default=2048, help="grid size of the large workload (0: skip it)")
    ap.add_argument("--dda-4k", type=int, default=0, metavar="N",
                    help="only the 3840x2160 DDA measurement on an N^3 gas field (for profiling); prints its line")
    ap.add_argument("--dda-4k-forms", nargs="*", default=["texture"],
                    help="grid forms for --dda-4k: texture, texture-w4/-w16/-w32 (warp tile width), bricked, linear, "
                         "hybridK (one warp in K reads an x-fastest copy), raw, packed (texel bytes converted "
                         "in the kernel)")
    ap.add_argument("--svo-4k", type=int, default=0, metavar="N",
                    help="only octree traversals at 3840x2160 on the lean octree of an N^3 gas field (profiling)")
    ap.add_argument("--svo-4k-traversals", nargs="*", default=["esvo"])
    ap.add_argument("--batch-only", action="store_true",
                    help="only the batch kernel on 512 frames of 256x256 of the CT octree (profiling)")
    ap.add_argument("--c3-frames", type=int, default=16)
    ap.add_argument("--serve-requests", type=int, default=200)
    ap.add_argument("--serve-rates", type=float, nargs="*", default=[50.0, 200.0, 1000.0, 2000.0, 0.0])
    ap.add_argument("--serve-only", action="store_true", help="the serving mix alone, per --serve-variants")
    ap.add_argument("--serve-variants", nargs="*", default=[""],
                    help="server settings per run, key=value[,key=value] (Server keyword arguments)")
    args = ap.parse_args(argv)
    if args.impl == "reference":
        return run_reference(args)
    if args.dda_4k:
        return run_dda_4k_only(args)
    if args.svo_4k:
        return run_svo_4k_only(args)
    if args.batch_only:
        return run_batch_only(args)
    if args.serve_only:
        return run_serve_only(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

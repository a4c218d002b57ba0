"""The persistent batch kernel: every job of a mixed batch (volumes, layouts,
traversals, resolutions) must equal its single-frame render bit for bit,
for every launch shape, through graphs and the autotuner."""
from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

CAMS = [((0, 0, -0.8660254), (0, 1, 0), (0.5, 0.5, 2.5)),
        ((0.35, -0.2, -0.91), (0.0, 0.976, -0.215), (0.2, 0.8, 2.0)),
        ((0.6, 0.3, 0.74), (-0.2, 0.95, 0.0), (0.45, 0.55, 0.5))]
SIZES = [(37, 21), (64, 48), (8, 8), (130, 3), (1, 1)]


@pytest.fixture(scope="module")
def scene(ctx):
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.blobs(64, seed=7)
    nodes, st = oracle.build_svo(g, "rope")
    leaf_root, st1 = oracle.build_svo(np.full((4, 4, 4, 4), 99, np.uint8), "rope")
    vols = {"grid": ctx.upload_grid(g), "svo": ctx.upload_svo(nodes, st["side"]),
            "leafroot": ctx.upload_svo(leaf_root, st1["side"])}
    import os
    os.environ["XN_GRID_LAYOUT"] = "linear"
    try:
        vols["grid_linear"] = ctx.upload_grid(g)
    finally:
        del os.environ["XN_GRID_LAYOUT"]
    return xg, vols


def _specs(scene):
    xg, vols = scene
    specs = []
    i = 0
    for vname, travs in (("grid", ["dda"]), ("grid_linear", ["dda"]),
                         ("svo", ["svo-naive", "esvo", "svo-df", "svo-rope"]),
                         ("leafroot", ["svo-naive", "svo-rope"])):
        for t in travs:
            w, h = SIZES[i % len(SIZES)]
            specs.append((vols[vname], t, xg.make_camera(*CAMS[i % len(CAMS)]), xg.make_params(w, h, 10.0)))
            i += 1
    return specs


def _reference_frames(ctx, specs):
    import torch
    outs = []
    for vol, t, cam, p in specs:
        buf = torch.zeros((p.output_region.height, p.output_region.width), dtype=torch.int32, device="cuda")
        ctx.render_device(vol, t, cam, p, buf.data_ptr(), None, None, torch.cuda.current_stream().cuda_stream)
        outs.append(buf)
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in outs]


def _batch_buffers(specs):
    import torch
    return [torch.full((p.output_region.height, p.output_region.width), -1, dtype=torch.int32, device="cuda")
            for _, _, _, p in specs]


@pytest.mark.parametrize("tile,threads,chunk", [(8, 128, 1), (4, 64, 3), (16, 256, 2), (32, 96, 1), (8, 1024, 7),
                                                (8, 128, 0), (4, 256, 0), (32, 1024, 0), (0, 0, 0)])
def test_batch_equals_single_frame_renders(ctx, scene, tile, threads, chunk):
    import torch
    xg, _ = scene
    specs = _specs(scene)
    ref = _reference_frames(ctx, specs)
    bufs = _batch_buffers(specs)
    jobs = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(specs, bufs))
    cfg = xg.BatchConfig(tile, threads, 0, chunk)
    ctx.render_batch(jobs, len(specs), cfg, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for (v, t, c, p), b, r in zip(specs, bufs, ref):
        assert np.array_equal(b.cpu().numpy(), r), (t, p.output_region.width, p.output_region.height)
    assert ctx.ray_errors() == 0


def test_batch_graph_replays_new_tables(ctx, scene):
    import torch
    xg, vols = scene
    specs = _specs(scene)
    ref = _reference_frames(ctx, specs)
    stream = torch.cuda.current_stream().cuda_stream
    g = ctx.batch_graph(64, xg.BatchConfig(8, 128, 0, 2), stream)
    for rnd in range(3):  # alternate slots; each replay reads the table just written
        sub = specs[rnd::2]
        rsub = ref[rnd::2]
        bufs = _batch_buffers(sub)
        jobs = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(sub, bufs))
        g.launch(jobs, len(sub))
        torch.cuda.synchronize()
        for b, r in zip(bufs, rsub):
            assert np.array_equal(b.cpu().numpy(), r)
    g.close()


def test_autotune_picks_a_valid_shape_and_is_used(ctx, scene):
    import torch
    xg, _ = scene
    specs = _specs(scene)[:3]
    bufs = _batch_buffers(specs)
    jobs = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(specs, bufs))
    stream = torch.cuda.current_stream().cuda_stream
    best, ms = ctx.autotune_batch(jobs, len(specs), stream)
    # a persistent-kernel shape, or 0: the plain form (one single-frame launch per job)
    assert best.tile_width in (0, 4, 8, 16, 32) and best.block_threads % 32 == 0 and best.chunk in (0, 1, 2, 4)
    assert ms > 0
    ref = _reference_frames(ctx, specs)
    bufs2 = _batch_buffers(specs)
    jobs2 = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(specs, bufs2))
    ctx.render_batch(jobs2, len(specs), None, stream)  # the tuned shape
    torch.cuda.synchronize()
    for b, r in zip(bufs2, ref):
        assert np.array_equal(b.cpu().numpy(), r)


def test_batch_rejects_bad_shapes_and_jobs(ctx, scene):
    import torch
    xg, vols = scene
    specs = _specs(scene)[:1]
    bufs = _batch_buffers(specs)
    jobs = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(specs, bufs))
    for cfg in (xg.BatchConfig(6, 128, 0, 1), xg.BatchConfig(8, 100, 0, 1), xg.BatchConfig(8, 0, 0, 1)):
        with pytest.raises(xg.XenodonError) as e:
            ctx.render_batch(jobs, 1, cfg)
        assert e.value.code == xg.XN_ERR_ARG
    bad = ctx.make_jobs([(vols["grid"], "esvo", specs[0][2], specs[0][3], bufs[0].data_ptr())])
    with pytest.raises(xg.XenodonError):
        ctx.render_batch(bad, 1)


@pytest.mark.parametrize("vname,trav", [("grid", "dda"), ("svo", "svo-naive"), ("svo", "esvo"), ("svo", "svo-df"),
                                        ("svo", "svo-rope")])
def test_single_traversal_batches_use_the_inlined_form(ctx, scene, monkeypatch, vname, trav):
    # a batch whose jobs share one traversal runs a kernel with that
    # traversal inlined; it must equal the single-frame renders and the
    # generic form (XN_BATCH_GENERIC=1)
    import torch
    xg, vols = scene
    specs = [(vols[vname], trav, xg.make_camera(*CAMS[i % len(CAMS)]), xg.make_params(*SIZES[i % len(SIZES)], 10.0))
             for i in range(6)]
    ref = _reference_frames(ctx, specs)
    stream = torch.cuda.current_stream().cuda_stream
    for generic in ("0", "1"):
        monkeypatch.setenv("XN_BATCH_GENERIC", generic)
        for cfg in (xg.BatchConfig(8, 128, 0, 1), xg.BatchConfig(4, 64, 0, 3), xg.BatchConfig(8, 256, 0, 0)):
            bufs = _batch_buffers(specs)
            jobs = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(specs, bufs))
            ctx.render_batch(jobs, len(specs), cfg, stream)
            torch.cuda.synchronize()
            for b, r in zip(bufs, ref):
                assert np.array_equal(b.cpu().numpy(), r), (trav, generic)


@pytest.mark.parametrize("generic", ["0", "1"])
def test_mixed_batches_split_by_form_or_generic_agree(ctx, scene, monkeypatch, generic):
    # a mixed batch runs one specialised launch per form (default) or one
    # generic launch (XN_BATCH_GENERIC=1); graphs capture the same choice
    import torch
    xg, _ = scene
    monkeypatch.setenv("XN_BATCH_GENERIC", generic)
    specs = _specs(scene)
    ref = _reference_frames(ctx, specs)
    stream = torch.cuda.current_stream().cuda_stream
    bufs = _batch_buffers(specs)
    jobs = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(specs, bufs))
    ctx.render_batch(jobs, len(specs), xg.BatchConfig(4, 256, 0, 0), stream)
    torch.cuda.synchronize()
    for b, r in zip(bufs, ref):
        assert np.array_equal(b.cpu().numpy(), r)
    g = ctx.batch_graph(len(specs), xg.BatchConfig(8, 128, 0, 1), stream)
    for _ in range(2):
        bufs = _batch_buffers(specs)
        jobs = ctx.make_jobs((v, t, c, p, b.data_ptr()) for (v, t, c, p), b in zip(specs, bufs))
        g.launch(jobs, len(specs))
        torch.cuda.synchronize()
        for b, r in zip(bufs, ref):
            assert np.array_equal(b.cpu().numpy(), r)
    g.close()

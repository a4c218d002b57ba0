"""GPU octree build vs the reference's bytes (golden files made by the
reference's own builder) and vs the oracle restatement; bit-exact."""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).with_name("golden") / "svo_golden.npz"


def _golden():
    z = np.load(GOLDEN)
    return z, json.loads(bytes(z["meta"]).decode())


def _types():
    return ("sparse", "rope", "dag")


def test_gpu_build_matches_reference_golden_files(ctx):
    z, meta = _golden()
    done = 0
    for m in meta:
        if m["type"] not in _types():
            continue
        g = z["grid__" + m["grid"]]
        nodes, stats = ctx.build_svo(g, m["type"], m["heuristic"], m["threshold"])
        data = oracle.svo_file_bytes(nodes, stats["side"])
        assert data == bytes(z[m["key"]]), m["key"]
        assert stats == m["stats"], m["key"]
        done += 1
    assert done == len(meta)


@pytest.mark.parametrize("svo_type", ["sparse", "rope", "dag"])
@pytest.mark.parametrize("heuristic,threshold", [("chan-diff", 0), ("chan-diff", 30), ("std-dev", 0.0),
                                                 ("std-dev", 12.5)])
def test_gpu_build_matches_oracle_random_shapes(ctx, svo_type, heuristic, threshold):
    from xenodon_gb300 import volumes
    rng = np.random.default_rng(11)
    shapes = [(1, 1, 1), (1, 7, 1), (2, 2, 2), (5, 3, 9), (17, 33, 8), (40, 23, 31)]
    for i, shape in enumerate(shapes):
        g = volumes.random_grid(*shape, seed=i, density=float(rng.uniform(0.1, 0.7)), levels=4)
        if i % 2:
            g[..., 3] = rng.integers(200, 256, shape)  # vary alpha too
        ref, rstats = oracle.build_svo(g, svo_type, heuristic, threshold)
        got, stats = ctx.build_svo(g, svo_type, heuristic, threshold)
        assert stats == rstats, shape
        assert np.array_equal(got, ref), shape


def test_gpu_build_ct_volume_rope(ctx):
    from xenodon_gb300 import volumes
    g = volumes.ct_shell(96, 68, 96, seed=1, device="cpu")
    ref, rstats = oracle.build_svo(g, "rope")
    got, stats = ctx.build_svo(g, "rope")
    assert stats == rstats
    assert np.array_equal(got, ref)


def test_gpu_build_stddev_sequential_mode_agrees(ctx, monkeypatch):
    # every decision taken by the reference's own sequential double loop
    from xenodon_gb300 import volumes
    g = volumes.random_grid(19, 14, 23, seed=4, density=0.5, levels=6)
    fast, fs = ctx.build_svo(g, "sparse", "std-dev", 21.0)
    monkeypatch.setenv("XN_BUILD_STDDEV_SEQUENTIAL", "1")
    slow, ss = ctx.build_svo(g, "sparse", "std-dev", 21.0)
    ref, rs = oracle.build_svo(g, "sparse", "std-dev", 21.0)
    assert fs == ss == rs
    assert np.array_equal(fast, ref) and np.array_equal(slow, ref)


def test_gpu_build_rejects_bad_arguments(ctx):
    import xenodon_gb300 as xg
    g = np.zeros((2, 2, 2, 4), np.uint8)
    for kw in ({"heuristic": "chan-diff", "threshold": 256}, {"heuristic": "chan-diff", "threshold": 1.5},
               {"heuristic": "std-dev", "threshold": -1.0}):
        with pytest.raises(xg.XenodonError) as e:
            ctx.build_svo(g, "sparse", **kw)
        assert e.value.code == xg.XN_ERR_ARG


def test_gpu_built_octree_renders_like_oracle_built(ctx):
    from xenodon_gb300 import volumes
    import xenodon_gb300 as xg
    g = volumes.blobs(64, seed=2)
    nodes, st = ctx.build_svo(g, "rope")
    ref, _ = oracle.build_svo(g, "rope")
    assert np.array_equal(nodes, ref)
    vol = ctx.upload_svo(nodes, st["side"])
    cam = xg.make_camera((0, 0, -0.8660254), (0, 1, 0), (0.5, 0.5, 2.5))
    rgba, _, _ = ctx.render(vol, "svo-rope", cam, xg.make_params(64, 64, 10.0))
    o = oracle.render("svo-rope", nodes=ref, camera=oracle.make_camera((0, 0, -0.8660254), (0, 1, 0), (0.5, 0.5, 2.5)),
                      view=oracle.make_view(64, 64, 10.0))
    assert np.abs(rgba.astype(int) - o["rgba"].astype(int)).max() <= 1


def test_device_resident_build_and_upload_match_host_paths(ctx):
    import torch
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.blobs(48, seed=8)
    d = torch.from_numpy(g).cuda().contiguous()
    dims = (g.shape[2], g.shape[1], g.shape[0])
    svo_dev, st = ctx.build_svo_volume(d.data_ptr(), dims, "rope")
    nodes, st_host = ctx.build_svo(g, "rope")
    assert st == st_host
    svo_host = ctx.upload_svo(nodes, st_host["side"])
    grid_dev = ctx.upload_grid_device(d.data_ptr(), dims)
    grid_host = ctx.upload_grid(g)
    assert svo_dev.info()["device_bytes"] == svo_host.info()["device_bytes"]
    cam = xg.make_camera((0.3, -0.1, -0.95), (0, 1, -0.105), (0.2, 0.7, 2.2))
    p = xg.make_params(80, 60, 10.0)
    for t in ("svo-naive", "esvo", "svo-df", "svo-rope"):
        a, _, _ = ctx.render(svo_dev, t, cam, p)
        b, _, _ = ctx.render(svo_host, t, cam, p)
        assert np.array_equal(a, b), t
    a, _, _ = ctx.render(grid_dev, "dda", cam, p)
    b, _, _ = ctx.render(grid_host, "dda", cam, p)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("case", ["blobs", "ct", "random-stddev", "random-chandiff", "leaf-root", "one-voxel"])
def test_lean_build_renders_like_the_full_build(ctx, case):
    # XN_BUILD_LEAN writes the device layout directly; everything but svo-rope
    # must be bit for bit what the full build (node array -> layout) gives
    import torch
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    heur, thr = "chan-diff", 0
    if case == "blobs":
        g = volumes.blobs(64, seed=3)
    elif case == "ct":
        g = volumes.ct_shell(80, 57, 80, seed=2, device="cpu")
    elif case == "random-stddev":
        g = volumes.random_grid(29, 40, 33, seed=5, density=0.4, levels=6)
        heur, thr = "std-dev", 9.0
    elif case == "random-chandiff":
        g = volumes.random_grid(17, 9, 30, seed=6, density=0.6, levels=8)
        heur, thr = "chan-diff", 40
    elif case == "leaf-root":
        g = np.full((8, 8, 8, 4), 77, np.uint8)
    else:
        g = np.full((1, 1, 1, 4), 200, np.uint8)
    d = torch.from_numpy(np.ascontiguousarray(g)).cuda()
    dims = (g.shape[2], g.shape[1], g.shape[0])
    lean, st = ctx.build_svo_volume(d.data_ptr(), dims, "sparse", heur, thr, lean=True)
    full, st_full = ctx.build_svo_volume(d.data_ptr(), dims, "sparse", heur, thr)
    assert st == st_full
    ref, rst = oracle.build_svo(g, "sparse", heur, thr)
    assert st == rst
    n_internal = int(np.sum(ref[:, 9] < 0x80000000))
    if n_internal:
        assert lean.info()["device_bytes"] == n_internal * 36
    cams = [((0.3, -0.1, -0.95), (0, 1, -0.105), (0.2, 0.7, 2.2)), ((0.6, 0.3, 0.74), (-0.2, 0.95, 0.0), (0.45, 0.55, 0.5))]
    p = xg.make_params(67, 45, 10.0)
    for cam in cams:
        c = xg.make_camera(*cam)
        for t in ("svo-naive", "esvo", "svo-df"):
            a, ea, _ = ctx.render(lean, t, c, p, emission=True)
            b, eb, _ = ctx.render(full, t, c, p, emission=True)
            assert np.array_equal(a, b) and np.array_equal(ea, eb), (case, t)
    if n_internal:
        with pytest.raises(xg.XenodonError) as e:
            ctx.render(lean, "svo-rope", xg.make_camera(*cams[0]), p)
        assert e.value.code == xg.XN_ERR_ARG


def test_lean_build_rejects_non_sparse_types(ctx):
    import torch
    import xenodon_gb300 as xg
    d = torch.zeros((4, 4, 4, 4), dtype=torch.uint8, device="cuda")
    for t in ("rope", "dag"):
        with pytest.raises(xg.XenodonError) as e:
            ctx.build_svo_volume(d.data_ptr(), (4, 4, 4), t, lean=True)
        assert e.value.code == xg.XN_ERR_ARG

"""Parity of the CUDA traversal kernels with the oracle, through the C ABI.

Tolerances (written here, checked per traversal):
  * RGBA8 image vs the FP32 oracle: identical on >= 99.99% of pixels and
    within 1 LSB per channel on all of them;
  * per-ray emission vs the FP32 oracle: >= 99.9% of rays bit-identical and
    every ray within 1e-5 relative (+1e-7 absolute);
  * per-ray emission vs the FP64 re-trace: 1e-5 relative is met by at least as
    many rays as the reference algorithm in FP32 (the FP32 oracle) meets it,
    less 0.1%; the shaders' own FP32 stepping error keeps a few per cent of
    rays above 1e-5, so 1e-5 cannot be required of every ray;
  * words read per ray (the roofline's algorithmic bytes): equal to the
    oracle's count on every ray.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

TRAV = ("dda", "svo-naive", "esvo", "svo-df", "svo-rope")


def _params_pair(xg, w, h, e=10.0, ratio=(1.0, 1.0, 1.0), out_off=(0, 0), out_ext=None, disp_off=(0, 0),
                 disp_ext=None):
    p = xg.make_params(w, h, e, ratio, out_off, out_ext, disp_off, disp_ext)
    v = oracle.make_view(w, h, e, ratio, out_off, out_ext, disp_off, disp_ext)
    return p, v


def _gpu_counts(ctx, vol, trav, cam, params):
    import torch
    w, h = params.output_region.width, params.output_region.height
    rgba = torch.empty((h, w), dtype=torch.int32, device="cuda")
    loads = torch.empty((h, w), dtype=torch.int32, device="cuda")
    em = torch.empty((h, w, 3), dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream()
    ctx.render_device(vol, trav, cam, params, rgba.data_ptr(), em.data_ptr(), loads.data_ptr(), s.cuda_stream)
    torch.cuda.synchronize()
    return rgba, em.cpu().numpy(), loads.cpu().numpy().view(np.uint32)


def check_parity(ctx, trav, cam_tuple, params, view, grid=None, nodes=None, side=None, vol=None, label=""):
    import xenodon_gb300 as xg
    if vol is None:
        vol = ctx.upload_grid(grid) if trav == "dda" else ctx.upload_svo(nodes, side)
    cam = xg.make_camera(*cam_tuple)
    ocam = oracle.make_camera(*cam_tuple)
    rgba, em, ms = ctx.render(vol, trav, cam, params, emission=True)
    ref = oracle.render(trav, grid=grid, nodes=nodes, camera=ocam, view=view)
    ref64 = oracle.render(trav, grid=grid, nodes=nodes, camera=ocam, view=view, f64=True, want_loads=False)
    assert ref["errors"] == 0, label
    d = np.abs(rgba.astype(np.int32) - ref["rgba"].astype(np.int32))
    assert d.max() <= 1, f"{label} {trav}: RGBA off by {d.max()}"
    same_px = np.all(d == 0, axis=2).mean()
    assert same_px >= 0.9999, f"{label} {trav}: only {same_px:.6f} of pixels identical"
    e32 = ref["emission"]
    exact = (em == e32).all(axis=2).mean()
    assert exact >= 0.999, f"{label} {trav}: only {exact:.5f} of rays bit-identical"
    assert np.all(np.abs(em - e32) <= 1e-5 * np.abs(e32) + 1e-7), f"{label} {trav}: emission beyond 1e-5"
    e64 = ref64["emission"]
    sig = np.abs(e64) > 1e-3 * max(1e-30, np.abs(e64).max())
    if sig.any():
        rel_gpu = (np.abs(em.astype(np.float64) - e64) / np.abs(e64).clip(1e-30))[sig]
        rel_ref = (np.abs(e32.astype(np.float64) - e64) / np.abs(e64).clip(1e-30))[sig]
        assert (rel_gpu <= 1e-5).mean() >= (rel_ref <= 1e-5).mean() - 1e-3, f"{label} {trav}: worse than FP32 reference"
    _, em2, loads = _gpu_counts(ctx, vol, trav, cam, params)
    assert np.array_equal(loads, ref["loads"]), f"{label} {trav}: load counts differ"
    assert np.array_equal(em2, em), f"{label} {trav}: counting variant changed the result"
    return rgba, ms


@pytest.fixture(scope="module")
def blob_volumes():
    from xenodon_gb300 import volumes
    g = volumes.blobs(64, seed=0)
    nodes, st = oracle.build_svo(g, "rope")
    return g, nodes, st["side"]


CAMS = {
    "front": ((0, 0, -0.8660254), (0, 1, 0), (0.5, 0.5, 2.5)),
    "oblique": ((0.35, -0.2, -0.91), (0.0, 0.976, -0.215), (0.2, 0.8, 2.0)),
    "inside": ((0.6, 0.3, 0.74), (-0.2, 0.95, 0.0), (0.45, 0.55, 0.5)),
    "grazing": ((1.0, 0.0, 0.0), (0, 1, 0), (-1.0, 0.5, 0.5)),
}


@pytest.mark.parametrize("cam", list(CAMS))
@pytest.mark.parametrize("trav", TRAV)
def test_parity_blobs(ctx, blob_volumes, trav, cam):
    import xenodon_gb300 as xg
    g, nodes, side = blob_volumes
    p, v = _params_pair(xg, 96, 64)
    check_parity(ctx, trav, CAMS[cam], p, v, grid=g, nodes=nodes, side=side, label=f"blobs/{cam}")


@pytest.mark.parametrize("trav", TRAV)
def test_parity_ct_shell_non_cubic(ctx, trav):
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.ct_shell(64, 45, 64, seed=1, device="cpu")
    nodes, st = oracle.build_svo(g, "rope")
    cam = ((0.3, -0.1, 0.95), (0, 1, 0.1), (0.3, 0.45, -1.2))
    p, v = _params_pair(xg, 80, 60, e=10.0)
    check_parity(ctx, trav, cam, p, v, grid=g, nodes=nodes, side=st["side"], label="ct")


@pytest.mark.parametrize("trav", ("svo-naive", "esvo", "svo-df"))
def test_parity_dag_tree(ctx, trav):
    # DAG trees share subtrees; naive / df / esvo traverse them unchanged
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.random_grid(32, 32, 32, seed=9, density=0.4, levels=3)
    nodes, st = oracle.build_svo(g, "dag")
    p, v = _params_pair(xg, 64, 64, e=5.0)
    check_parity(ctx, trav, CAMS["oblique"], p, v, nodes=nodes, side=st["side"], label="dag")


@pytest.mark.parametrize("trav", TRAV)
def test_parity_subregion_and_voxel_ratio(ctx, blob_volumes, trav):
    # an output region inside a larger display region (one device block of a
    # multi-device headless.conf) with an anisotropic --voxel-ratio
    import xenodon_gb300 as xg
    g, nodes, side = blob_volumes
    p, v = _params_pair(xg, 0, 0, e=7.0, ratio=(1.0, 1.5, 0.75), out_off=(40, 16), out_ext=(50, 37),
                        disp_off=(0, 0), disp_ext=(128, 72))
    check_parity(ctx, trav, CAMS["front"], p, v, grid=g, nodes=nodes, side=side, label="subregion")


@pytest.mark.parametrize("trav", ("svo-naive", "esvo", "svo-df", "svo-rope"))
def test_parity_leaf_root_and_depth_one(ctx, trav):
    import xenodon_gb300 as xg
    g = np.zeros((2, 2, 2, 4), np.uint8)
    g[..., 3] = 255
    g[0, 1, 1, :3] = (250, 10, 10)
    for grid in (np.full((4, 4, 4, 4), 77, np.uint8), g):
        nodes, st = oracle.build_svo(grid, "rope")
        p, v = _params_pair(xg, 32, 32, e=3.0)
        check_parity(ctx, trav, CAMS["oblique"], p, v, nodes=nodes, side=st["side"], label="tiny")


def test_svo_rope_on_a_tree_without_ropes_matches_reference(ctx, blob_volumes):
    # without ropes every leaf's neighbour word is 0 (the root): the reference
    # shader stops after the first leaf, and so do we
    import xenodon_gb300 as xg
    g, _, _ = blob_volumes
    nodes, st = oracle.build_svo(g, "sparse")
    p, v = _params_pair(xg, 48, 48)
    check_parity(ctx, "svo-rope", CAMS["front"], p, v, nodes=nodes, side=st["side"], label="no-ropes")


def test_volume_kind_mismatch_is_rejected(ctx, blob_volumes):
    import xenodon_gb300 as xg
    g, nodes, side = blob_volumes
    vg = ctx.upload_grid(g)
    vs = ctx.upload_svo(nodes, side)
    cam = xg.make_camera(*CAMS["front"])
    p = xg.make_params(8, 8)
    for vol, trav in ((vg, "esvo"), (vs, "dda")):
        with pytest.raises(xg.XenodonError) as e:
            ctx.render(vol, trav, cam, p)
        assert e.value.code == xg.XN_ERR_ARG
    assert vs.info()["has_ropes"] and vs.info()["n_nodes"] == nodes.shape[0]


def test_malformed_octree_upload_is_rejected(ctx, blob_volumes):
    import xenodon_gb300 as xg
    _, nodes, side = blob_volumes
    bad = nodes.copy()
    bad[3, 2] = nodes.shape[0]  # child index out of range
    with pytest.raises(xg.XenodonError) as e:
        ctx.upload_svo(bad, side)
    assert e.value.code == xg.XN_ERR_FORMAT


def test_hbm_budget_refuses_uploads(built_library, blob_volumes):
    import torch
    import xenodon_gb300 as xg
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    g, _, _ = blob_volumes
    with xg.Context(0, hbm_budget=g.nbytes // 2) as c:
        with pytest.raises(xg.XenodonError) as e:
            c.upload_grid(g)
        assert e.value.code == xg.XN_ERR_BUDGET
        assert c.memory()[0] < g.nbytes // 2


@pytest.mark.parametrize("cam", ["front", "inside", "grazing", "oblique"])
def test_parity_dda_bricked_grid_layout(ctx, blob_volumes, monkeypatch, cam):
    # XN_GRID_LAYOUT=bricked: 8^3 bricks of 2x2x1 16-byte groups, zero padding
    import xenodon_gb300 as xg
    g, _, _ = blob_volumes
    monkeypatch.setenv("XN_GRID_LAYOUT", "bricked")
    vol = ctx.upload_grid(g)
    p, v = _params_pair(xg, 96, 64)
    check_parity(ctx, "dda", CAMS[cam], p, v, grid=g, vol=vol, label=f"bricked/{cam}")


def test_parity_dda_bricked_non_cubic_and_batched(ctx, monkeypatch):
    # a grid whose sides are not multiples of the brick; single-frame and
    # batch renders of the bricked form equal the texture form's
    import torch
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.ct_shell(37, 21, 50, seed=1, device="cpu")
    monkeypatch.setenv("XN_GRID_LAYOUT", "bricked")
    vb = ctx.upload_grid(g)
    monkeypatch.delenv("XN_GRID_LAYOUT")
    vt = ctx.upload_grid(g)
    for cam in ("front", "oblique", "inside", "grazing"):
        p, v = _params_pair(xg, 61, 47)
        a, _ = check_parity(ctx, "dda", CAMS[cam], p, v, grid=g, vol=vb, label=f"bricked-ct/{cam}")
        b, _, _ = ctx.render(vt, "dda", xg.make_camera(*CAMS[cam]), p)
        assert np.array_equal(a, b)
    p = xg.make_params(61, 47, 10.0)
    bufs = [torch.full((47, 61), -1, dtype=torch.int32, device="cuda") for _ in range(2)]
    jobs = ctx.make_jobs([(vb, "dda", xg.make_camera(*CAMS["oblique"]), p, bufs[0].data_ptr()),
                          (vt, "dda", xg.make_camera(*CAMS["oblique"]), p, bufs[1].data_ptr())])
    ctx.render_batch(jobs, 2, xg.BatchConfig(8, 128, 0, 1), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert torch.equal(bufs[0], bufs[1])


@pytest.mark.parametrize("share", ["1", "2", "4"])
def test_parity_dda_hybrid_texture_and_lsu_reads(ctx, blob_volumes, monkeypatch, share):
    # XN_GRID_LAYOUT=hybrid: one warp in XN_DDA_LSU_SHARE reads the x-fastest
    # copy, the others the texture; every pixel is the reference's either way
    import xenodon_gb300 as xg
    g, _, _ = blob_volumes
    monkeypatch.setenv("XN_GRID_LAYOUT", "hybrid")
    monkeypatch.setenv("XN_DDA_LSU_SHARE", share)
    vol = ctx.upload_grid(g)
    for cam in ("oblique", "grazing"):
        p, v = _params_pair(xg, 97, 61)
        check_parity(ctx, "dda", CAMS[cam], p, v, grid=g, vol=vol, label=f"hybrid{share}/{cam}")


@pytest.mark.parametrize("ww", ["4", "16", "32"])
def test_dda_texture_warp_tile_shapes_agree(ctx, blob_volumes, monkeypatch, ww):
    # XN_DDA_WARP_TILE: warps of 4x8, 16x2 or 32x1 pixels; per-pixel results
    # and word counts do not depend on the tile shape
    import xenodon_gb300 as xg
    g, _, _ = blob_volumes
    vol = ctx.upload_grid(g)
    p, v = _params_pair(xg, 93, 58)
    monkeypatch.setenv("XN_DDA_WARP_TILE", ww)
    check_parity(ctx, "dda", CAMS["oblique"], p, v, grid=g, vol=vol, label=f"dda-ww{ww}")


@pytest.mark.parametrize("cam", ["front", "inside", "grazing"])
def test_parity_dda_linear_grid_layout(ctx, blob_volumes, monkeypatch, cam):
    # the linear (x-fastest global memory) form of the grid, beside the default texture form
    import xenodon_gb300 as xg
    g, _, _ = blob_volumes
    monkeypatch.setenv("XN_GRID_LAYOUT", "linear")
    vol = ctx.upload_grid(g)
    assert vol.info()["device_bytes"] == g.nbytes
    p, v = _params_pair(xg, 96, 64)
    check_parity(ctx, "dda", CAMS[cam], p, v, grid=g, vol=vol, label=f"linear/{cam}")


def test_octree_device_layout_is_compact(ctx, blob_volumes):
    # the reference's 40-byte nodes are replaced on the device by 32-byte
    # internal nodes plus 32-byte rope records per leaf (68 B per internal node)
    _, nodes, side = blob_volumes
    vol = ctx.upload_svo(nodes, side)
    n_internal = int(np.sum(nodes[:, 9] < 0x80000000))
    n_leaves = nodes.shape[0] - n_internal
    assert vol.info()["device_bytes"] == n_internal * 68 + n_leaves * 32


@pytest.mark.parametrize("trav", ("svo-df", "svo-naive", "esvo", "svo-rope"))
def test_parity_tree_with_inconsistent_depth_fields(ctx, blob_volumes, trav):
    # svo-df reads a node's depth field when it pops back to it; where the
    # fields disagree with the tree the literal traversal (not the masked
    # one) must run, and give the reference's (different) picture
    import xenodon_gb300 as xg
    _, nodes, side = blob_volumes
    bad = nodes.copy()
    internal = np.nonzero(bad[:, 9] < 0x80000000)[0]
    bad[internal[bad[internal, 9] == 2][:3], 9] = 3
    p, v = _params_pair(xg, 96, 64)
    check_parity(ctx, trav, CAMS["oblique"], p, v, nodes=bad, side=side, label="inconsistent-depth")


def test_full_size_ct_frame_matches_oracle_on_sampled_rows(ctx):
    # the benchmark shape: 512x361x512 CT volume, 1920x1080, all five traversals;
    # the oracle renders every 60th row of the same frame
    import torch
    import xenodon_gb300 as xg
    from xenodon_gb300 import cameras, volumes
    g = volumes.ct_shell(512, 361, 512, seed=1, device="cuda")
    nodes, st = ctx.build_svo(g, "rope")
    vg, vs_ = ctx.upload_grid(g), ctx.upload_svo(nodes, st["side"])
    cam_t = cameras.ct_path()[37]
    cam = xg.make_camera(*cam_t)
    p = xg.make_params(1920, 1080, 10.0)
    for trav in TRAV:
        rgba, em, _ = ctx.render(vg if trav == "dda" else vs_, trav, cam, p, emission=True)
        for y in range(7, 1080, 60):
            v = oracle.make_view(1920, 1080, 10.0, output_offset=(0, y), output_extent=(1920, 1))
            ref = oracle.render(trav, grid=g, nodes=nodes, camera=oracle.make_camera(*cam_t), view=v,
                                want_loads=False)
            assert np.abs(rgba[y].astype(int) - ref["rgba"][0].astype(int)).max() <= 1, (trav, y)
            assert np.mean(em[y] == ref["emission"][0]) >= 0.999, (trav, y)
    del torch


@pytest.mark.parametrize("trav", TRAV)
def test_emission_is_exactly_linear_in_the_coefficient(ctx, blob_volumes, trav):
    # colour = trace * e * sqrt(...): doubling e doubles every emission bit for bit
    import xenodon_gb300 as xg
    g, nodes, side = blob_volumes
    vol = ctx.upload_grid(g) if trav == "dda" else ctx.upload_svo(nodes, side)
    cam = xg.make_camera(*CAMS["oblique"])
    _, e1, _ = ctx.render(vol, trav, cam, xg.make_params(64, 48, 3.0), emission=True)
    _, e2, _ = ctx.render(vol, trav, cam, xg.make_params(64, 48, 6.0), emission=True)
    assert np.array_equal(e2, 2 * e1)
    black, e0, _ = ctx.render(vol, trav, cam, xg.make_params(64, 48, 0.0), emission=True)
    assert not np.any(e0) and np.all(black[..., :3] == 0) and np.all(black[..., 3] == 255)


@pytest.mark.parametrize("trav", TRAV)
def test_parity_empty_volume_and_degenerate_regions(ctx, trav):
    import xenodon_gb300 as xg
    g = np.zeros((16, 12, 20, 4), np.uint8)
    g[..., 3] = 255
    nodes, st = oracle.build_svo(g, "rope")
    cases = [  # one pixel; a region of a display rectangle with a negative origin
        dict(w=1, h=1, out_off=(0, 0), disp_off=(0, 0), disp_ext=None),
        dict(w=17, h=5, out_off=(3, 9), disp_off=(-4, 2), disp_ext=(40, 30)),
    ]
    for c in cases:
        p, v = _params_pair(xg, c["w"], c["h"], out_off=c["out_off"], out_ext=(c["w"], c["h"]),
                            disp_off=c["disp_off"], disp_ext=c["disp_ext"])
        check_parity(ctx, trav, CAMS["inside"], p, v, grid=g, nodes=nodes, side=st["side"], label="empty")


@pytest.mark.parametrize("trav", ["esvo", "svo-df"])
@pytest.mark.parametrize("cam", ["oblique", "inside", "grazing"])
def test_stacks_in_shared_memory_equal_local(ctx, blob_volumes, monkeypatch, trav, cam):
    # XN_STACKS=shared puts the esvo and masked svo-df stacks in shared
    # memory, XN_STACKS=local in local memory: same bits, same word counts
    import xenodon_gb300 as xg
    _, nodes, side = blob_volumes
    vol = ctx.upload_svo(nodes, side)
    p, v = _params_pair(xg, 83, 61)
    monkeypatch.setenv("XN_STACKS", "shared")
    shared, _ = check_parity(ctx, trav, CAMS[cam], p, v, nodes=nodes, vol=vol, label=f"{trav}-shared/{cam}")
    _, em_s, loads_s = _gpu_counts(ctx, vol, trav, xg.make_camera(*CAMS[cam]), p)
    monkeypatch.setenv("XN_STACKS", "local")
    local, _, _ = ctx.render(vol, trav, xg.make_camera(*CAMS[cam]), p)
    _, em_l, loads_l = _gpu_counts(ctx, vol, trav, xg.make_camera(*CAMS[cam]), p)
    assert np.array_equal(shared, local)
    assert np.array_equal(em_s, em_l) and np.array_equal(loads_s, loads_l)


@pytest.mark.parametrize("cam", ["oblique", "inside", "grazing", "front"])
def test_naive_resumed_find_equals_root_descent(ctx, blob_volumes, monkeypatch, cam):
    # svo-naive resumes each find from the previous path (fixed point);
    # XN_NAIVE_FIND=root descends from the root like the reference: same bits
    import xenodon_gb300 as xg
    _, nodes, side = blob_volumes
    vol = ctx.upload_svo(nodes, side)
    p, v = _params_pair(xg, 91, 47)
    resumed, _ = check_parity(ctx, "svo-naive", CAMS[cam], p, v, nodes=nodes, vol=vol, label=f"naive/{cam}")
    _, em_r, loads_r = _gpu_counts(ctx, vol, "svo-naive", xg.make_camera(*CAMS[cam]), p)
    monkeypatch.setenv("XN_NAIVE_FIND", "root")
    root, _, _ = ctx.render(vol, "svo-naive", xg.make_camera(*CAMS[cam]), p)
    _, em_0, loads_0 = _gpu_counts(ctx, vol, "svo-naive", xg.make_camera(*CAMS[cam]), p)
    assert np.array_equal(resumed, root)
    assert np.array_equal(em_r, em_0) and np.array_equal(loads_r, loads_0)


@pytest.mark.parametrize("size", [(96, 64), (37, 23), (1, 1), (130, 7)])
@pytest.mark.parametrize("cam", ["oblique", "inside", "grazing", "front"])
def test_df_walked_by_the_warp_equals_one_ray_per_thread(ctx, blob_volumes, monkeypatch, size, cam):
    # XN_DF_PACKET=1: the warp walks the union of its lanes' hit children;
    # each ray's bits and word count must be those of its own traversal
    import xenodon_gb300 as xg
    _, nodes, side = blob_volumes
    vol = ctx.upload_svo(nodes, side)
    p, v = _params_pair(xg, *size)
    monkeypatch.setenv("XN_DF_PACKET", "1")
    packet, _ = check_parity(ctx, "svo-df", CAMS[cam], p, v, nodes=nodes, vol=vol, label=f"df-packet/{cam}")
    _, em_p, loads_p = _gpu_counts(ctx, vol, "svo-df", xg.make_camera(*CAMS[cam]), p)
    monkeypatch.setenv("XN_DF_PACKET", "0")
    plain, _, _ = ctx.render(vol, "svo-df", xg.make_camera(*CAMS[cam]), p)
    _, em_0, loads_0 = _gpu_counts(ctx, vol, "svo-df", xg.make_camera(*CAMS[cam]), p)
    assert np.array_equal(packet, plain)
    assert np.array_equal(em_p, em_0) and np.array_equal(loads_p, loads_0)


@pytest.mark.parametrize("n", [2, 4, 16, 64])
@pytest.mark.parametrize("cam", ["oblique", "inside", "grazing"])
def test_df_lane_walk_equals_warp_walk(ctx, monkeypatch, n, cam):
    # the nodes just above the deepest internal nodes are walked by each lane
    # alone, two levels deep (one with XN_DF_LANE_LEVELS=1); XN_DF_LANE_WALK=0
    # keeps the warp walk there: same bits, same word counts, on trees 1 to 6
    # levels deep
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.random_grid(n, n, n, seed=n + 1, density=0.35, levels=4)
    nodes, st = oracle.build_svo(g, "sparse")
    vol = ctx.upload_svo(nodes, st["side"])
    p, v = _params_pair(xg, 61, 45)
    lane, _ = check_parity(ctx, "svo-df", CAMS[cam], p, v, nodes=nodes, vol=vol, label=f"df-lane/{n}/{cam}")
    _, em_l, loads_l = _gpu_counts(ctx, vol, "svo-df", xg.make_camera(*CAMS[cam]), p)
    monkeypatch.setenv("XN_DF_LANE_LEVELS", "1")
    one, _, _ = ctx.render(vol, "svo-df", xg.make_camera(*CAMS[cam]), p)
    _, em_1, loads_1 = _gpu_counts(ctx, vol, "svo-df", xg.make_camera(*CAMS[cam]), p)
    monkeypatch.delenv("XN_DF_LANE_LEVELS")
    monkeypatch.setenv("XN_DF_LANE_WALK", "0")
    warp, _, _ = ctx.render(vol, "svo-df", xg.make_camera(*CAMS[cam]), p)
    _, em_w, loads_w = _gpu_counts(ctx, vol, "svo-df", xg.make_camera(*CAMS[cam]), p)
    assert np.array_equal(lane, warp) and np.array_equal(one, warp)
    assert np.array_equal(em_l, em_w) and np.array_equal(loads_l, loads_w)
    assert np.array_equal(em_1, em_w) and np.array_equal(loads_1, loads_w)


@pytest.mark.parametrize("read", ["raw", "packed"])
@pytest.mark.parametrize("cam", ["front", "inside", "grazing"])
def test_dda_raw_texel_reads_equal_normalized(ctx, blob_volumes, monkeypatch, cam, read):
    # XN_TEX_READ=raw: the texture returns the bytes and the kernel converts
    # them through its shared table; packed: one 32-bit word per fetch,
    # converted in registers; same bits as the texture unit's UNORM read,
    # single-frame and batched
    import xenodon_gb300 as xg
    import torch
    g, _, _ = blob_volumes
    p, v = _params_pair(xg, 77, 53)
    norm_vol = ctx.upload_grid(g)
    a, _ = check_parity(ctx, "dda", CAMS[cam], p, v, grid=g, vol=norm_vol, label=f"dda-norm/{cam}")
    monkeypatch.setenv("XN_TEX_READ", read)
    raw_vol = ctx.upload_grid(g)
    b, _ = check_parity(ctx, "dda", CAMS[cam], p, v, grid=g, vol=raw_vol, label=f"dda-{read}/{cam}")
    assert np.array_equal(a, b)
    out = torch.empty((p.output_region.height, p.output_region.width), dtype=torch.int32, device="cuda")
    jobs = ctx.make_jobs([(raw_vol, "dda", xg.make_camera(*CAMS[cam]), p, out.data_ptr())])
    sptr = torch.cuda.current_stream().cuda_stream
    ctx.render_batch(jobs, 1, xg.BatchConfig(8, 128, 0, 1), sptr)
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy().view(np.uint8).reshape(a.shape), a)
    raw_vol.release()
    norm_vol.release()

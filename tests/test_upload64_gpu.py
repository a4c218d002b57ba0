"""Octrees handed over as 64-bit node arrays (xn_volume_upload_svo_fmt,
XN_NODES_U64): streamed through a chunk buffer into the device layout, they
render exactly what the same tree uploaded as the reference's 32-bit nodes
renders, for every traversal but svo-rope (whose rope words are not
converted), whatever the chunk size."""
from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

CAMS = [((0.35, -0.2, -0.91), (0.0, 0.976, -0.215), (0.2, 0.8, 2.0)),
        ((0.6, 0.3, 0.74), (-0.2, 0.95, 0.0), (0.45, 0.55, 0.5))]


def _frames(ctx, vol, trav):
    import torch
    import xenodon_gb300 as xg
    p = xg.make_params(72, 56, 8.0)
    out = []
    for c in CAMS:
        rgba = torch.empty((56, 72), dtype=torch.int32, device="cuda")
        em = torch.empty((56, 72, 3), dtype=torch.float32, device="cuda")
        loads = torch.empty((56, 72), dtype=torch.int32, device="cuda")
        s = torch.cuda.current_stream().cuda_stream
        ctx.render_device(vol, trav, xg.make_camera(*c), p, rgba.data_ptr(), em.data_ptr(), None, s)
        ctx.render_device(vol, trav, xg.make_camera(*c), p, rgba.data_ptr(), None, loads.data_ptr(), s)
        torch.cuda.synchronize()
        out.append((rgba.cpu().numpy(), em.cpu().numpy(), loads.cpu().numpy()))
    return out


@pytest.mark.parametrize("chunk", ["0", "1000", "4097"])
@pytest.mark.parametrize("svo_type", ["sparse", "dag", "rope"])
def test_u64_upload_renders_like_u32(ctx, monkeypatch, svo_type, chunk):
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.blobs(48, seed=2)
    nodes, st = oracle.build_svo(g, svo_type)
    monkeypatch.setenv("XN_UPLOAD_CHUNK_NODES", chunk)
    v32 = ctx.upload_svo(nodes, st["side"])
    v64 = ctx.upload_svo64(xg.nodes_to_u64(nodes), st["side"])
    assert v64.info()["n_nodes"] == nodes.shape[0]
    assert not v64.info()["has_ropes"]
    for trav in ("svo-naive", "esvo", "svo-df"):
        for a, b in zip(_frames(ctx, v32, trav), _frames(ctx, v64, trav)):
            for x, y in zip(a, b):
                assert np.array_equal(x, y), (svo_type, trav)
    with pytest.raises(xg.XenodonError):
        ctx.render(v64, "svo-rope", xg.make_camera(*CAMS[0]), xg.make_params(8, 8))
    v32.release()
    v64.release()


def test_u64_upload_of_a_leaf_root_and_bad_indices(ctx, monkeypatch):
    import xenodon_gb300 as xg
    g = np.full((4, 4, 4, 4), 90, np.uint8)
    nodes, st = oracle.build_svo(g, "sparse")
    assert nodes.shape[0] == 1
    v = ctx.upload_svo64(xg.nodes_to_u64(nodes), st["side"])
    a, _, _ = ctx.render(v, "esvo", xg.make_camera(*CAMS[0]), xg.make_params(16, 16))
    b, _, _ = ctx.render(ctx.upload_svo(nodes, st["side"]), "esvo", xg.make_camera(*CAMS[0]), xg.make_params(16, 16))
    assert np.array_equal(a, b)
    from xenodon_gb300 import volumes
    nodes, st = oracle.build_svo(volumes.blobs(16, seed=1), "sparse")
    raw = xg.nodes_to_u64(nodes).copy()
    words = raw.view(np.uint64).reshape(-1, 9)
    internal = np.nonzero(nodes[:, 9] < 0x80000000)[0]
    words[internal[-1], 3] = 1 << 33  # a child beyond the node count, past 32 bits
    monkeypatch.setenv("XN_UPLOAD_CHUNK_NODES", "64")
    with pytest.raises(xg.XenodonError) as e:
        ctx.upload_svo64(raw, st["side"])
    assert e.value.code == xg.XN_ERR_FORMAT

"""Device-layout octree files ("XNDN-SVC", xn_volume_save / xn_volume_load):
a volume read back renders exactly like the one written, malformed files are
refused before any traversal can read them."""
from __future__ import annotations

import struct

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

CAMS = [((0.3, -0.1, -0.95), (0, 1, -0.105), (0.2, 0.7, 2.2)),
        ((0.6, 0.3, 0.74), (-0.2, 0.95, 0.0), (0.45, 0.55, 0.5))]


def _same_renders(ctx, a, b, travs):
    import xenodon_gb300 as xg
    p = xg.make_params(71, 40, 10.0)
    for cam in CAMS:
        c = xg.make_camera(*cam)
        for t in travs:
            ra, ea, _ = ctx.render(a, t, c, p, emission=True)
            rb, eb, _ = ctx.render(b, t, c, p, emission=True)
            assert np.array_equal(ra, rb) and np.array_equal(ea, eb), t


@pytest.fixture(scope="module")
def blob_tree():
    from xenodon_gb300 import volumes
    g = volumes.blobs(64, seed=5)
    nodes, st = oracle.build_svo(g, "rope")
    return g, nodes, st


def test_round_trip_of_an_uploaded_rope_tree(ctx, blob_tree, tmp_path):
    _, nodes, st = blob_tree
    vol = ctx.upload_svo(nodes, st["side"])
    vol.save(tmp_path / "t.svc")
    back = ctx.load_volume(tmp_path / "t.svc")
    assert back.info() == vol.info()
    _same_renders(ctx, vol, back, ("svo-naive", "esvo", "svo-df", "svo-rope"))
    n_int = int(np.sum(nodes[:, 9] < 0x80000000))
    assert (tmp_path / "t.svc").stat().st_size == 64 + n_int * 68 + (nodes.shape[0] - n_int) * 32


def test_round_trip_of_a_lean_build(ctx, tmp_path):
    import torch
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.ct_shell(72, 51, 72, seed=4, device="cpu")
    d = torch.from_numpy(g).cuda()
    lean, st = ctx.build_svo_volume(d.data_ptr(), (72, 51, 72), "sparse", lean=True)
    lean.save(tmp_path / "l.svc")
    back = ctx.load_volume(tmp_path / "l.svc")
    assert back.info() == lean.info()
    _same_renders(ctx, lean, back, ("svo-naive", "esvo", "svo-df"))
    with pytest.raises(xg.XenodonError):
        ctx.render(back, "svo-rope", xg.make_camera(*CAMS[0]), xg.make_params(8, 8))


def test_round_trip_of_a_leaf_root(ctx, tmp_path):
    nodes, st = oracle.build_svo(np.full((4, 4, 4, 4), 123, np.uint8), "rope")
    vol = ctx.upload_svo(nodes, st["side"])
    vol.save(tmp_path / "r.svc")
    back = ctx.load_volume(tmp_path / "r.svc")
    _same_renders(ctx, vol, back, ("svo-naive", "esvo", "svo-df", "svo-rope"))


def test_malformed_files_are_refused(ctx, blob_tree, tmp_path):
    import xenodon_gb300 as xg
    _, nodes, st = blob_tree
    vol = ctx.upload_svo(nodes, st["side"])
    vol.save(tmp_path / "ok.svc")
    data = bytearray((tmp_path / "ok.svc").read_bytes())
    n_inner = struct.unpack_from("<Q", data, 32)[0]

    def refused(blob, msg):
        p = tmp_path / "bad.svc"
        p.write_bytes(bytes(blob))
        with pytest.raises(xg.XenodonError) as e:
            ctx.load_volume(p)
        assert e.value.code == xg.XN_ERR_FORMAT and msg in str(e.value), str(e.value)

    refused(b"XNDN-SVO" + bytes(data[8:]), "Invalid format id")
    refused(data[:40], "truncated header")
    refused(data[:-4], "File size does not match")
    bad = bytearray(data)
    struct.pack_into("<I", bad, 8, 2)
    refused(bad, "unsupported version")
    # an internal child index past the end of the inner array
    bad = bytearray(data)
    words = np.frombuffer(bytes(data[64:64 + n_inner * 32]), np.uint32)
    k = int(np.nonzero(words < 0x80000000)[0][0])
    struct.pack_into("<I", bad, 64 + 4 * k, n_inner + 5)
    refused(bad, "out of range")
    # a rope word past the leaf records
    bad = bytearray(data)
    leaves_at = 64 + n_inner * 68
    struct.pack_into("<I", bad, leaves_at + 4, 0x80000000 | 0x7FFFFFF0)
    refused(bad, "out of range")
    # the untouched file still loads
    assert ctx.load_volume(tmp_path / "ok.svc").info()["n_nodes"] == nodes.shape[0]


def test_depth_fields_that_disagree_select_the_literal_svo_df(ctx, blob_tree, tmp_path):
    # depth words are data the traversals read; a file whose depths disagree
    # with the tree must render svo-df like the reference over those words
    import xenodon_gb300 as xg
    _, nodes, st = blob_tree
    bad_nodes = nodes.copy()
    internal = np.nonzero(bad_nodes[:, 9] < 0x80000000)[0]
    bad_nodes[internal[bad_nodes[internal, 9] == 2][:3], 9] = 3
    vol = ctx.upload_svo(bad_nodes, st["side"])
    vol.save(tmp_path / "d.svc")
    back = ctx.load_volume(tmp_path / "d.svc")
    _same_renders(ctx, vol, back, ("svo-df",))
    cam = CAMS[0]
    p = xg.make_params(71, 40, 10.0)
    rgba, _, _ = ctx.render(back, "svo-df", xg.make_camera(*cam), p)
    ref = oracle.render("svo-df", nodes=bad_nodes, camera=oracle.make_camera(*cam), view=oracle.make_view(71, 40, 10.0))
    assert np.abs(rgba.astype(int) - ref["rgba"].astype(int)).max() <= 1

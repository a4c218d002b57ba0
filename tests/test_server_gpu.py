"""The render server: continuous batching with resident volumes, LRU eviction
and HBM-budget admission.  Every result must equal the same request rendered
alone (bit for bit: the arithmetic is identical)."""
from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def volumes_data():
    from xenodon_gb300 import volumes
    g0 = volumes.blobs(64, seed=11)
    g1 = volumes.ct_shell(48, 34, 48, seed=1, device="cpu")
    n0, s0 = oracle.build_svo(g0, "rope")
    n1, s1 = oracle.build_svo(g1, "rope")
    return {1: ("grid", g0), 2: ("svo", (n0, s0["side"])), 3: ("grid", g1), 4: ("svo", (n1, s1["side"]))}


def _requests(xg, rng, k):
    cams = [((0, 0, -0.8660254), (0, 1, 0), (0.5, 0.5, 2.5)),
            ((0.35, -0.2, -0.91), (0.0, 0.976, -0.215), (0.2, 0.8, 2.0)),
            ((0.6, 0.3, 0.74), (-0.2, 0.95, 0.0), (0.45, 0.55, 0.5))]
    sizes = [(64, 64), (31, 17), (120, 40), (8, 8)]
    out = []
    for i in range(k):
        vid = int(rng.integers(1, 5))
        trav = "dda" if vid in (1, 3) else ["svo-naive", "esvo", "svo-df", "svo-rope"][int(rng.integers(0, 4))]
        w, h = sizes[int(rng.integers(0, len(sizes)))]
        out.append((vid, trav, cams[int(rng.integers(0, 3))], xg.make_params(w, h, 10.0)))
    return out


def _alone(ctx, vols, req):
    import xenodon_gb300 as xg
    vid, trav, cam, p = req
    rgba, _, _ = ctx.render(vols[vid], trav, xg.make_camera(*cam), p)
    return rgba


def _register(server, ctx, volumes_data):
    handles = {}
    for vid, (kind, data) in volumes_data.items():
        if kind == "grid":
            server.add_grid(vid, data)
            handles[vid] = ctx.upload_grid(data)
        else:
            server.add_svo(vid, data[0], data[1])
            handles[vid] = ctx.upload_svo(data[0], data[1])
    return handles


def test_results_equal_alone_and_in_the_mix(ctx, volumes_data):
    import xenodon_gb300 as xg
    rng = np.random.default_rng(3)
    with xg.Server(ctx, max_batch_jobs=16, streams=2) as server:
        vols = _register(server, ctx, volumes_data)
        reqs = _requests(xg, rng, 60)
        tickets = [server.submit(vid, trav, xg.make_camera(*cam), p) for vid, trav, cam, p in reqs]
        for t, req in zip(tickets, reqs):
            rgba, lat = server.wait(t, timeout=60)
            assert lat > 0
            assert np.array_equal(rgba, _alone(ctx, vols, req)), req[:2]
        st = server.stats()
        assert st["completed"] == 60 and st["failed"] == 0
        assert st["batches"] < 60  # requests were batched together
        assert 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
        assert st["mrays_per_s"] > 0


def test_lru_eviction_under_a_tight_budget(ctx, volumes_data):
    import xenodon_gb300 as xg
    # room for the largest volume plus frames, not for all four volumes
    alone = {vid: (ctx.upload_grid(d) if k == "grid" else ctx.upload_svo(d[0], d[1]))
             for vid, (k, d) in volumes_data.items()}
    sizes = {vid: v.info()["device_bytes"] for vid, v in alone.items()}
    for v in alone.values():
        v.release()
    budget = max(sizes.values()) + 4 * 120 * 64 * 4 + (64 << 10)
    assert budget < sum(sizes.values()) - min(sizes.values())
    rng = np.random.default_rng(5)
    with xg.Server(ctx, hbm_budget=budget, max_batch_jobs=4, streams=1) as server:
        vols = _register(server, ctx, volumes_data)
        reqs = _requests(xg, rng, 24)
        results = []
        for vid, trav, cam, p in reqs:  # one at a time: every switch of volume forces an upload
            t = server.submit(vid, trav, xg.make_camera(*cam), p)
            results.append(server.wait(t, timeout=60)[0])
        for r, req in zip(results, reqs):
            assert np.array_equal(r, _alone(ctx, vols, req))
        st = server.stats()
        assert st["evictions"] > 0 and st["uploads"] > 4
        assert st["hbm_used"] <= budget


def test_server_rejects_bad_requests(ctx, volumes_data):
    import xenodon_gb300 as xg
    with xg.Server(ctx, hbm_budget=1 << 20) as server:
        kind, g = volumes_data[1]
        server.add_grid(1, g)
        cam = xg.make_camera((0, 0, 1), (0, 1, 0), (0.5, 0.5, -1))
        with pytest.raises(xg.XenodonError):
            server.submit(9, "dda", cam, xg.make_params(8, 8))  # unknown volume
        with pytest.raises(xg.XenodonError):
            server.submit(1, "esvo", cam, xg.make_params(8, 8))  # traversal does not fit the volume
        with pytest.raises(xg.XenodonError) as e:
            server.submit(1, "dda", cam, xg.make_params(1024, 1024))  # frame larger than the budget
        assert e.value.code == xg.XN_ERR_BUDGET
        # the volume (1 MiB budget, 1 MiB grid + frame) can never fit: the request fails, not hangs
        t = server.submit(1, "dda", cam, xg.make_params(8, 8))
        with pytest.raises(xg.XenodonError):
            server.wait(t, timeout=30)


def test_resident_volumes_are_served_and_never_evicted(ctx, volumes_data):
    # xn_server_add_volume: a volume built on the device (no host copy) is
    # served like the others, counted in the budget, and left to its owner
    import torch
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    g = volumes.blobs(48, seed=21)
    d = torch.from_numpy(g).cuda()
    lean, _ = ctx.build_svo_volume(d.data_ptr(), (48, 48, 48), "sparse", lean=True)
    size = lean.info()["device_bytes"]
    cam = xg.make_camera((0.35, -0.2, -0.91), (0.0, 0.976, -0.215), (0.2, 0.8, 2.0))
    p = xg.make_params(40, 30, 10.0)
    alone, _, _ = ctx.render(lean, "esvo", cam, p)
    kind, g0 = volumes_data[1]
    budget = size + g0.nbytes + (1 << 20)
    with xg.Server(ctx, hbm_budget=budget, max_batch_jobs=4) as server:
        server.add_volume(7, lean)
        server.add_grid(1, g0)
        for _ in range(3):  # alternate: the grid is uploaded, the resident volume never leaves
            t = server.submit(7, "esvo", cam, p)
            assert np.array_equal(server.wait(t, timeout=60)[0], alone)
            t = server.submit(1, "dda", cam, p)
            server.wait(t, timeout=60)
        st = server.stats()
        assert st["hbm_used"] <= budget
    with xg.Server(ctx, hbm_budget=size // 2) as small:
        with pytest.raises(xg.XenodonError) as e:
            small.add_volume(7, lean)
        assert e.value.code == xg.XN_ERR_BUDGET
    # the owner's volume is still usable after the server is gone
    again, _, _ = ctx.render(lean, "esvo", cam, p)
    assert np.array_equal(again, alone)


@pytest.mark.parametrize("threads", ["128", "32"])
def test_frames_fold_into_the_running_persistent_kernel(ctx, volumes_data, monkeypatch, threads):
    """Requests that arrive while the persistent kernel runs are appended to
    its ring and rendered by it: with a long idle time one launch takes all of
    them, each result equal to its render alone (blocks of 128 threads or of
    one warp, XN_FOLD_THREADS)."""
    import time
    import xenodon_gb300 as xg
    monkeypatch.setenv("XN_FOLD_THREADS", threads)
    rng = np.random.default_rng(8)
    with xg.Server(ctx, fold_idle_us=200000) as server:
        vols = _register(server, ctx, volumes_data)
        reqs = _requests(xg, rng, 12)
        tickets = []
        for vid, trav, cam, p in reqs:
            tickets.append(server.submit(vid, trav, xg.make_camera(*cam), p))
            time.sleep(0.002)
        for t, req in zip(tickets, reqs):
            rgba, _ = server.wait(t, timeout=60)
            assert np.array_equal(rgba, _alone(ctx, vols, req)), req[:2]
        st = server.stats()
        assert st["folded"] == 12 + st["republished"]
        assert st["fold_launches"] == 1


def test_persistent_kernel_leaves_when_idle_and_is_launched_again(ctx, volumes_data):
    import time
    import xenodon_gb300 as xg
    rng = np.random.default_rng(9)
    with xg.Server(ctx, fold_idle_us=100) as server:
        vols = _register(server, ctx, volumes_data)
        reqs = _requests(xg, rng, 3)
        for vid, trav, cam, p in reqs:
            t = server.submit(vid, trav, xg.make_camera(*cam), p)
            assert np.array_equal(server.wait(t, timeout=60)[0], _alone(ctx, vols, (vid, trav, cam, p)))
            time.sleep(0.05)  # far longer than the idle time: the kernel has left
        assert server.stats()["fold_launches"] == 3


def test_full_rings_close_and_alternate(ctx, volumes_data):
    import xenodon_gb300 as xg
    rng = np.random.default_rng(10)
    with xg.Server(ctx, max_batch_jobs=4) as server:
        vols = _register(server, ctx, volumes_data)
        reqs = _requests(xg, rng, 30)
        tickets = [server.submit(vid, trav, xg.make_camera(*cam), p) for vid, trav, cam, p in reqs]
        for t, req in zip(tickets, reqs):
            assert np.array_equal(server.wait(t, timeout=60)[0], _alone(ctx, vols, req)), req[:2]
        st = server.stats()
        assert st["completed"] == 30 and st["fold_launches"] >= 30 // 4


@pytest.mark.parametrize("band_pixels,streams", [(0, 2), (1 << 16, 2), (100000, 1), (0, 3)])
def test_large_frames_take_the_single_frame_path(ctx, volumes_data, band_pixels, streams):
    """Frames of 2^19 pixels or more run through the single-frame kernels on
    low-priority streams beside the folded small frames, whole or in bands of
    rows (a band of 100000 pixels does not divide the frames' rows evenly);
    every result equals its render alone."""
    import xenodon_gb300 as xg
    rng = np.random.default_rng(12)
    with xg.Server(ctx, band_pixels=band_pixels, streams=streams) as server:
        vols = _register(server, ctx, volumes_data)
        reqs = _requests(xg, rng, 16)
        big = [(1, "dda", ((0, 0, -0.8660254), (0, 1, 0), (0.5, 0.5, 2.5)), xg.make_params(1024, 512, 10.0)),
               (2, "esvo", ((0.35, -0.2, -0.91), (0.0, 0.976, -0.215), (0.2, 0.8, 2.0)),
                xg.make_params(1280, 720, 10.0)),
               (4, "svo-rope", ((0.6, 0.3, 0.74), (-0.2, 0.95, 0.0), (0.45, 0.55, 0.5)),
                xg.make_params(800, 700, 10.0))]
        mix = reqs[:6] + big[:1] + reqs[6:11] + big[1:] + reqs[11:]
        tickets = [server.submit(vid, trav, xg.make_camera(*cam), p) for vid, trav, cam, p in mix]
        for t, req in zip(tickets, mix):
            assert np.array_equal(server.wait(t, timeout=120)[0], _alone(ctx, vols, req)), req[:2]
        st = server.stats()
        assert st["completed"] == len(mix) and st["failed"] == 0
        assert st["folded"] - st["republished"] == len(reqs)  # the three large frames were not folded


def test_server_trace_file(ctx, volumes_data, tmp_path, monkeypatch):
    """XN_SERVER_TRACE names a file that receives one line per request when
    the server is destroyed."""
    import xenodon_gb300 as xg
    rng = np.random.default_rng(13)
    path = tmp_path / "trace.txt"
    monkeypatch.setenv("XN_SERVER_TRACE", str(path))
    with xg.Server(ctx) as server:
        _register(server, ctx, volumes_data)
        reqs = _requests(xg, rng, 5)
        for t in [server.submit(vid, trav, xg.make_camera(*cam), p) for vid, trav, cam, p in reqs]:
            server.wait(t, timeout=60)
    lines = [ln.split() for ln in path.read_text().splitlines() if not ln.startswith("#")]
    assert len(lines) == 5 and all(len(f) == 8 for f in lines)
    assert all(float(x) >= 0 for f in lines for x in f[4:])


def test_arrivals_across_idle_exits_are_all_rendered(ctx, volumes_data):
    """With an idle time shorter than the gaps between arrivals the persistent
    kernel leaves and is launched again many times while frames keep coming;
    a kernel that has decided to leave takes no new tiles, so frames
    published to it meanwhile go to the next launch.  Every frame is
    rendered, equal to its render alone, and none waits for long."""
    import time
    import xenodon_gb300 as xg
    rng = np.random.default_rng(14)
    with xg.Server(ctx, fold_idle_us=50) as server:
        vols = _register(server, ctx, volumes_data)
        reqs = _requests(xg, rng, 60)
        tickets = []
        t0 = time.perf_counter()
        for vid, trav, cam, p in reqs:
            tickets.append(server.submit(vid, trav, xg.make_camera(*cam), p))
            time.sleep(float(rng.uniform(0.0, 0.0005)))
        for t, req in zip(tickets, reqs):
            rgba, lat = server.wait(t, timeout=60)
            assert np.array_equal(rgba, _alone(ctx, vols, req)), req[:2]
            assert lat < 5000.0
        assert time.perf_counter() - t0 < 60.0
        st = server.stats()
        assert st["completed"] == 60 and st["failed"] == 0
        assert st["folded"] == 60 + st["republished"]
        assert st["fold_launches"] >= 2

"""xn_build_svo_static, the octree build for callers that cannot allocate
device memory (for example code running inside another framework's memory
pool or under a fixed HBM budget).  It must produce exactly the nodes of the
allocating entry point xn_build_svo, call after call, although every call
reuses the same fixed scratch array.  This file is collected last."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _static_build(grid, svo_type, heuristic, threshold, capacity):
    import torch
    import xenodon_gb300 as xg
    lib = xg.load_library()
    g = np.ascontiguousarray(grid, dtype=np.uint8)
    d_vox = torch.from_numpy(g.view(np.int32).reshape(-1).copy()).cuda()
    d_nodes = torch.full((max(1, capacity) * 10,), -1, dtype=torch.int32, device="cuda")
    st = xg.BuildStats()
    stream = torch.cuda.current_stream().cuda_stream
    r = lib.xn_build_svo_static(d_vox.data_ptr(), g.shape[2], g.shape[1], g.shape[0], xg.SVO_TYPES[svo_type],
                                xg.HEURISTICS[heuristic], float(threshold), d_nodes.data_ptr(), capacity,
                                ctypes.byref(st), stream)
    torch.cuda.synchronize()
    stats = {f: int(getattr(st, f)) for f, _ in xg.BuildStats._fields_}
    nodes = d_nodes.cpu().numpy().view(np.uint32).reshape(-1, 10)[:stats["n_nodes"]]
    return r, nodes, stats, lib.xn_last_error().decode()


def test_static_build_matches_allocating_build_on_consecutive_calls(ctx):
    from xenodon_gb300 import volumes
    cases = [
        (volumes.random_grid(40, 23, 31, seed=21, density=0.4, levels=4), "rope", "chan-diff", 0),
        (volumes.blobs(32, seed=5), "dag", "std-dev", 6.5),
        (volumes.random_grid(17, 33, 9, seed=22, density=0.6, levels=3), "sparse", "chan-diff", 50),
    ]
    for grid, svo_type, heuristic, threshold in cases:
        ref, ref_stats = ctx.build_svo(grid, svo_type, heuristic, threshold)
        r, nodes, stats, msg = _static_build(grid, svo_type, heuristic, threshold, ref.shape[0])
        assert r == 0, msg
        assert stats == ref_stats
        assert np.array_equal(nodes, ref)


def test_static_build_rejects_oversized_requests(ctx):
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    big = np.zeros((160, 160, 160, 4), np.uint8)
    r, _, _, msg = _static_build(big, "sparse", "chan-diff", 0, 16)
    assert r == xg.XN_ERR_BUDGET and "static scratch" in msg
    grid = volumes.random_grid(12, 12, 12, seed=3, density=0.5)
    ref, ref_stats = ctx.build_svo(grid, "sparse")
    r, _, stats, msg = _static_build(grid, "sparse", "chan-diff", 0, ref.shape[0] - 1)
    assert r == xg.XN_ERR_ARG and stats["n_nodes"] == ref.shape[0] and "node buffer" in msg

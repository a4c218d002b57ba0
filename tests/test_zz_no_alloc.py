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


def test_static_build_single_voxel_grid(ctx):
    """A 1x1x1 grid is a tree of one leaf (the build's depth-0 case), for
    every tree type."""
    grid = np.zeros((1, 1, 1, 4), np.uint8)
    grid[0, 0, 0] = (17, 200, 3, 255)
    for svo_type in ("sparse", "dag", "rope"):
        ref, ref_stats = ctx.build_svo(grid, svo_type)
        for _ in range(2):
            r, nodes, stats, msg = _static_build(grid, svo_type, "chan-diff", 0, 1)
            assert r == 0, msg
            assert stats == ref_stats
            assert np.array_equal(nodes, ref)


def test_static_build_uniform_grid_is_a_leaf_root(ctx):
    """A uniform 8^3 grid collapses to a root leaf through the level passes
    (not the depth-0 case), for every tree type and both heuristics."""
    grid = np.zeros((8, 8, 8, 4), np.uint8)
    grid[...] = (90, 10, 200, 255)
    for svo_type in ("sparse", "dag", "rope"):
        for heuristic in ("chan-diff", "std-dev"):
            ref, ref_stats = ctx.build_svo(grid, svo_type, heuristic, 0)
            assert ref.shape[0] == 1
            r, nodes, stats, msg = _static_build(grid, svo_type, heuristic, 0, 1)
            assert r == 0, msg
            assert stats == ref_stats
            assert np.array_equal(nodes, ref)


def test_static_build_dag_node_buffer_too_small(ctx):
    """A DAG's node count is known only after deduplication; a buffer one
    node short is refused with the count needed."""
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    grid = volumes.blobs(24, seed=9)
    ref, _ = ctx.build_svo(grid, "dag")
    r, _, stats, msg = _static_build(grid, "dag", "chan-diff", 0, ref.shape[0] - 1)
    assert r == xg.XN_ERR_ARG and stats["n_nodes"] == ref.shape[0] and "node buffer" in msg
    r, nodes, stats, msg = _static_build(grid, "dag", "chan-diff", 0, ref.shape[0])
    assert r == 0, msg
    assert np.array_equal(nodes, ref)


_CONTEXT_SCRIPT = r'''
import ctypes, json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
import xenodon_gb300 as xg
from xenodon_gb300 import volumes

cu = ctypes.CDLL("libcuda.so.1")
def ck(r, what):
    if r != 0:
        raise SystemExit(f"{what}: CUresult {r}")
lib = xg.load_library()
grid = np.ascontiguousarray(volumes.random_grid(21, 30, 26, seed=4, density=0.5, levels=5))
vox = grid.view(np.uint32).reshape(-1)
CAP = 40000

def build_here():
    g, n = ctypes.c_uint64(), ctypes.c_uint64()
    ck(cu.cuMemAlloc_v2(ctypes.byref(g), ctypes.c_size_t(vox.nbytes)), "cuMemAlloc")
    ck(cu.cuMemAlloc_v2(ctypes.byref(n), ctypes.c_size_t(CAP * 40)), "cuMemAlloc")
    ck(cu.cuMemcpyHtoD_v2(g, vox.ctypes.data_as(ctypes.c_void_p), ctypes.c_size_t(vox.nbytes)), "HtoD")
    st = xg.BuildStats()
    r = lib.xn_build_svo_static(g.value, 26, 30, 21, 2, 0, 0.0, n.value, CAP, ctypes.byref(st), None)
    if r != 0:
        raise SystemExit("xn_build_svo_static: " + lib.xn_last_error().decode())
    out = np.empty((st.n_nodes, 10), np.uint32)
    ck(cu.cuMemcpyDtoH_v2(out.ctypes.data_as(ctypes.c_void_p), n, ctypes.c_size_t(out.nbytes)), "DtoH")
    cu.cuMemFree_v2(g)
    cu.cuMemFree_v2(n)
    return out

ck(cu.cuInit(0), "cuInit")
dev = ctypes.c_int()
ck(cu.cuDeviceGet(ctypes.byref(dev), 0), "cuDeviceGet")
primary = ctypes.c_void_p()
ck(cu.cuDevicePrimaryCtxRetain(ctypes.byref(primary), dev), "cuDevicePrimaryCtxRetain")
ck(cu.cuCtxSetCurrent(primary), "cuCtxSetCurrent")
a = build_here()
second = ctypes.c_void_p()
ck(cu.cuCtxCreate_v2(ctypes.byref(second), 0, dev), "cuCtxCreate")
b = build_here()
ck(cu.cuCtxPopCurrent_v2(ctypes.byref(ctypes.c_void_p())), "cuCtxPopCurrent")
ck(cu.cuCtxSetCurrent(primary), "cuCtxSetCurrent")
c = build_here()
ck(cu.cuCtxDestroy_v2(second), "cuCtxDestroy")
np.savez(sys.argv[2], a=a, b=b, c=c)
'''


def test_static_build_follows_the_current_context(ctx, tmp_path):
    """The scratch array's address belongs to one context.  A caller that
    switches to another context on the same device (a driver-API context
    beside the primary one) gets the address of that context's array, and
    the primary context's again when it switches back: three builds, one per
    switch, give the allocating build's nodes.  Runs in a child process so
    that its contexts end with it."""
    import subprocess
    import sys
    from pathlib import Path
    from xenodon_gb300 import volumes
    root = Path(__file__).resolve().parents[1]
    script = tmp_path / "ctx_switch.py"
    script.write_text(_CONTEXT_SCRIPT)
    out = tmp_path / "nodes.npz"
    p = subprocess.run([sys.executable, str(script), str(root), str(out)], capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    ref, _ = ctx.build_svo(volumes.random_grid(21, 30, 26, seed=4, density=0.5, levels=5), "rope")
    got = np.load(out)
    for k in ("a", "b", "c"):
        assert np.array_equal(got[k], ref), k

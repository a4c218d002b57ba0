"""The streamed (one top-level cube at a time) octree build: its file must be
byte-identical to the one-shot build of the whole grid, xn_build_svo +
xn_svo_save, whose bytes are pinned against the reference's own builder."""
from __future__ import annotations

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _one_shot_bytes(ctx, g, heuristic, threshold):
    nodes, st = ctx.build_svo(g, "sparse", heuristic, threshold)
    return oracle.svo_file_bytes(nodes, st["side"]), st


def _streamed(ctx, g, heuristic, threshold, path):
    reads = []

    def read_region(x0, y0, z0, nx, ny, nz):
        reads.append((x0, y0, z0, nx, ny, nz))
        return g[z0:z0 + nz, y0:y0 + ny, x0:x0 + nx]

    st = ctx.build_svo_streamed((g.shape[2], g.shape[1], g.shape[0]), read_region, path, heuristic, threshold)
    return path.read_bytes(), st, reads


@pytest.mark.parametrize("heuristic,threshold", [("chan-diff", 0), ("chan-diff", 40), ("std-dev", 0.0),
                                                 ("std-dev", 9.5)])
def test_two_cube_grid_equals_one_shot_build(ctx, tmp_path, heuristic, threshold):
    # 48x20x30 in a 64^3 tree: only the cubes at x = 0 and x = 32 hold voxels,
    # the other six are black leaves
    from xenodon_gb300 import volumes
    g = volumes.random_grid(30, 20, 48, seed=3, density=0.5, levels=4)
    ref, ref_st = _one_shot_bytes(ctx, g, heuristic, threshold)
    got, st, reads = _streamed(ctx, g, heuristic, threshold, tmp_path / "s.svo")
    assert sorted(r[:3] for r in reads) == [(0, 0, 0), (32, 0, 0)]
    assert st == ref_st
    assert got == ref


@pytest.mark.parametrize("shape", [(32, 32, 32), (24, 31, 17), (2, 1, 2), (1, 1, 1), (3, 2, 2), (64, 9, 40)])
def test_cube_builds_equal_one_shot_build_on_shapes(ctx, tmp_path, shape):
    from xenodon_gb300 import volumes
    g = volumes.random_grid(*shape, seed=sum(shape), density=0.45, levels=3)
    for heuristic, threshold in (("chan-diff", 0), ("chan-diff", 90), ("std-dev", 30.0)):
        ref, ref_st = _one_shot_bytes(ctx, g, heuristic, threshold)
        got, st, _ = _streamed(ctx, g, heuristic, threshold, tmp_path / "s.svo")
        assert st == ref_st, (shape, heuristic)
        assert got == ref, (shape, heuristic)


def test_uniform_cube_is_one_leaf(ctx, tmp_path):
    g = np.zeros((16, 16, 16, 4), np.uint8)
    g[...] = (40, 50, 60, 255)
    ref, ref_st = _one_shot_bytes(ctx, g, "chan-diff", 0)
    got, st, _ = _streamed(ctx, g, "chan-diff", 0, tmp_path / "u.svo")
    assert st["n_nodes"] == 1 and st == ref_st
    assert got == ref
    got, st, _ = _streamed(ctx, g, "std-dev", 0.0, tmp_path / "v.svo")
    assert got == _one_shot_bytes(ctx, g, "std-dev", 0.0)[0]


def test_streamed_ct_volume_equals_one_shot_build(ctx, tmp_path):
    # the benchmark's CT volume (512x361x512): eight cubes of 256^3
    from xenodon_gb300 import volumes
    g = volumes.ct_shell(512, 361, 512, seed=1, device="cuda")
    ref, ref_st = _one_shot_bytes(ctx, g, "chan-diff", 0)
    got, st, reads = _streamed(ctx, g, "chan-diff", 0, tmp_path / "ct.svo")
    assert len(reads) == 8
    assert st == ref_st
    assert got == ref


def test_reader_failure_is_reported(ctx, tmp_path):
    import xenodon_gb300 as xg

    def bad(x0, y0, z0, nx, ny, nz):
        raise OSError("disk gone")

    with pytest.raises(OSError):
        ctx.build_svo_streamed((8, 8, 8), bad, tmp_path / "x.svo")
    with pytest.raises(xg.XenodonError) as e:
        ctx.build_svo_streamed((8, 8, 8), lambda *a: np.zeros((8, 8, 8, 4), np.uint8) if a[3] == 4 else None,
                               tmp_path / "y.svo", "std-dev", -1.0)
    assert e.value.code == xg.XN_ERR_ARG

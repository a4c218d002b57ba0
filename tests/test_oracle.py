"""The oracle itself: pinned against the reference's own builder and checked
with known-answer cases (CPU only)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).with_name("golden") / "svo_golden.npz"


def _golden():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta"]).decode())
    return z, meta


def test_oracle_builder_matches_reference_golden_files(oracle_lib):
    z, meta = _golden()
    assert len(meta) == 50
    for m in meta:
        g = z["grid__" + m["grid"]]
        nodes, stats = oracle_lib.build_svo(g, m["type"], m["heuristic"], m["threshold"])
        data = oracle_lib.svo_file_bytes(nodes, stats["side"])
        assert data == bytes(z[m["key"]]), m["key"]
        assert stats == m["stats"], m["key"]


def test_oracle_builder_matches_reference_builder_random(oracle_lib):
    if not oracle_lib.build_ref():
        pytest.skip("reference sources not present")
    rng = np.random.default_rng(7)
    for i in range(12):
        dims = tuple(int(v) for v in rng.integers(1, 24, 3))
        g = np.zeros(dims + (4,), np.uint8)
        m = rng.random(dims) < rng.uniform(0.05, 0.6)
        g[m] = rng.integers(0, 3, (int(m.sum()), 4)) * 100
        for t in ("sparse", "dag", "rope"):
            for h, th in (("chan-diff", 0), ("chan-diff", 100), ("std-dev", 40.0)):
                ref, rstats = oracle_lib.ref_build_svo(g, t, h, th)
                nodes, stats = oracle_lib.build_svo(g, t, h, th)
                assert oracle_lib.svo_file_bytes(nodes, stats["side"]) == ref
                assert stats == rstats


def _uniform_grid(dz, dy, dx, rgb):
    g = np.zeros((dz, dy, dx, 4), np.uint8)
    g[..., :3] = rgb
    g[..., 3] = 255
    return g


def _centre_pixel(res, w, h):
    return res["emission"][h // 2, w // 2]


@pytest.mark.parametrize("f64", [False, True])
def test_dda_axis_aligned_slab_known_answer(oracle_lib, f64):
    # a ray down the z axis through a uniform 8x8x8 slab of colour c covers 8
    # voxels: emission = c/255 * 8 * e / side (side = 8)
    g = _uniform_grid(8, 8, 8, (255, 128, 0))
    w = h = 16
    cam = oracle_lib.make_camera((0, 0, 1), (0, 1, 0), (0.5, 0.5, -1.0))
    view = oracle_lib.make_view(w, h, emission_coeff=3.0)
    r = oracle_lib.render("dda", grid=g, camera=cam, view=view, f64=f64)
    e = _centre_pixel(r, w, h)
    np.testing.assert_allclose(e, [3.0, 3.0 * 128 / 255, 0.0], rtol=1e-5, atol=1e-6)
    assert r["errors"] == 0


@pytest.mark.parametrize("trav", ["svo-naive", "esvo", "svo-df", "svo-rope"])
def test_svo_axis_aligned_known_answer(oracle_lib, trav):
    g = _uniform_grid(8, 8, 8, (255, 128, 0))
    nodes, stats = oracle_lib.build_svo(g, "rope")
    assert stats["n_nodes"] == 1  # a uniform cube collapses to a leaf root
    w = h = 16
    cam = oracle_lib.make_camera((0, 0, 1), (0, 1, 0), (0.5, 0.5, -1.0))
    view = oracle_lib.make_view(w, h, emission_coeff=2.0)
    r = oracle_lib.render(trav, nodes=nodes, camera=cam, view=view, f64=True)
    # unit cube, path length 1: emission = c/255 * 1 * e
    np.testing.assert_allclose(_centre_pixel(r, w, h), [2.0, 2.0 * 128 / 255, 0.0], rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("trav", ["dda", "svo-naive", "esvo", "svo-df", "svo-rope"])
def test_ray_missing_the_volume_is_black(oracle_lib, trav):
    g = _uniform_grid(8, 8, 8, (200, 200, 200))
    nodes, _ = oracle_lib.build_svo(g, "rope")
    cam = oracle_lib.make_camera((0, 0, -1), (0, 1, 0), (0.5, 0.5, -1.0))  # looking away
    view = oracle_lib.make_view(8, 8, emission_coeff=1.0)
    r = oracle_lib.render(trav, grid=g, nodes=nodes, camera=cam, view=view)
    if trav == "svo-rope":
        # svo_rope.comp:78-103 accepts a box behind the ray origin and adds the
        # first leaf with a negative step; the UNORM store clamps it to black
        assert np.all(r["emission"] <= 0)
    else:
        assert np.all(r["emission"] == 0)
    assert np.all(r["rgba"][..., :3] == 0) and np.all(r["rgba"][..., 3] == 255)


def test_camera_inside_volume_dda(oracle_lib):
    # camera at the centre of a uniform slab: the centre ray travels half the depth
    g = _uniform_grid(16, 16, 16, (255, 255, 255))
    cam = oracle_lib.make_camera((0, 0, 1), (0, 1, 0), (0.5, 0.5, 0.5))
    view = oracle_lib.make_view(8, 8, emission_coeff=1.0)
    r = oracle_lib.render("dda", grid=g, camera=cam, view=view, f64=True)
    np.testing.assert_allclose(_centre_pixel(r, 8, 8), [0.5, 0.5, 0.5], rtol=1e-5)


def test_traversals_agree_on_the_same_volume(oracle_lib):
    from xenodon_gb300 import volumes
    g = volumes.blobs(64, seed=3)  # power of two: DDA and octree share coordinates
    nodes, _ = oracle_lib.build_svo(g, "rope")
    cam = oracle_lib.make_camera((0.2, -0.1, -0.97), (0, 1, 0.0), (0.4, 0.6, 2.2))
    view = oracle_lib.make_view(64, 48, emission_coeff=10.0)
    ems = {}
    for t in ("dda", "svo-naive", "esvo", "svo-df", "svo-rope"):
        r = oracle_lib.render(t, grid=g, nodes=nodes, camera=cam, view=view)
        assert r["errors"] == 0
        ems[t] = r["emission"]
    for t, e in ems.items():
        assert np.abs(e - ems["dda"]).max() < 2e-4, t


def test_fp32_and_fp64_oracles_agree_within_one_lsb(oracle_lib):
    from xenodon_gb300 import volumes
    g = volumes.blobs(48, seed=1)
    nodes, _ = oracle_lib.build_svo(g, "rope")
    cam = oracle_lib.make_camera((0, 0, -0.8660254), (0, 1, 0), (0.5, 0.5, 2.5))
    view = oracle_lib.make_view(64, 64, emission_coeff=10.0)
    for t in ("dda", "svo-naive", "esvo", "svo-df", "svo-rope"):
        a = oracle_lib.render(t, grid=g, nodes=nodes, camera=cam, view=view)
        b = oracle_lib.render(t, grid=g, nodes=nodes, camera=cam, view=view, f64=True)
        d = np.abs(a["rgba"].astype(int) - b["rgba"].astype(int))
        assert d.max() <= 1, t


def _find(nodes, side, pos, max_depth):
    """Independent restatement of Octree::find for the rope check."""
    if any(p < 0 or p >= side for p in pos):
        return 0
    idx, off, ext = 0, [0, 0, 0], side
    while True:
        ext //= 2
        if nodes[idx, 9] & 0x80000000 or ext == 0 or max_depth == 0:
            return idx
        ci = 0
        for a, bit in ((0, 4), (1, 2), (2, 1)):
            if pos[a] >= off[a] + ext:
                ci |= bit
                off[a] += ext
        idx = int(nodes[idx, ci])
        max_depth -= 1


def test_rope_links_match_brute_force_neighbours(oracle_lib):
    from xenodon_gb300 import volumes
    g = volumes.random_grid(11, 9, 13, seed=5, density=0.2, levels=3)
    rope, st = oracle_lib.build_svo(g, "rope")
    sparse, _ = oracle_lib.build_svo(g, "sparse")
    side = st["side"]
    # walk the sparse tree (same node indices), collect leaves with positions
    stack = [(0, (0, 0, 0), side, 0)]
    checked = 0
    while stack:
        idx, pos, ext, depth = stack.pop()
        if sparse[idx, 9] & 0x80000000:
            exp = []
            for a in range(3):
                for s in (1, -1):
                    p = list(pos)
                    p[a] += s * ext
                    exp.append(_find(sparse, side, p, depth))
            assert list(rope[idx, :6]) == exp
            checked += 1
            continue
        h = ext // 2
        k = 0
        for xi in (0, 1):
            for yi in (0, 1):
                for zi in (0, 1):
                    stack.append((int(sparse[idx, k]), (pos[0] + xi * h, pos[1] + yi * h, pos[2] + zi * h), h, depth + 1))
                    k += 1
    assert checked > 100


def test_oracle_counts_reference_loads(oracle_lib):
    # DDA reads one texel per loop iteration: a ray down z through 8 voxels
    # (plus the boundary step) reads dz or dz+1 texels
    g = _uniform_grid(8, 8, 8, (10, 10, 10))
    cam = oracle_lib.make_camera((0, 0, 1), (0, 1, 0), (0.5, 0.5, -1.0))
    view = oracle_lib.make_view(16, 16)
    r = oracle_lib.render("dda", grid=g, camera=cam, view=view)
    assert r["loads"][8, 8] in (8, 9)
    # a leaf root: naive reads is_leaf_depth + colour per step
    nodes, _ = oracle_lib.build_svo(g, "sparse")
    r = oracle_lib.render("svo-naive", nodes=nodes, camera=cam, view=view)
    assert r["loads"][8, 8] % 2 == 0 and r["loads"][8, 8] >= 2


def test_oracle_matches_the_reference_shaders(oracle_lib, glsl_golden):
    # tests/golden/glsl_golden.npz holds what the reference's own shaders
    # (resources/*.comp compiled for the CPU by oracle/glsl_ref.py) render for
    # 138 cases: five traversals, six small volumes (blobs, a non-cubic CT
    # shell, a DAG and a sparse tree, a leaf root, a depth-one tree), cameras
    # outside, inside and grazing the volume, one region of a larger display
    # with an anisotropic voxel ratio, every 16th row of the 128^3 blob
    # configuration at 512x512, and two rows of a frame from each leg of the
    # 512x361x512 CT configuration's path at 1920x1080.  The oracle's FP32
    # restatement must give the same RGBA8 pixels, the same float colour and
    # the same count of words read from the model on every ray.
    assert len(glsl_golden.cases) == 138
    for case in glsl_golden.cases:
        v = glsl_golden.view(case)
        dda = case["traversal"] == "dda"
        view = oracle_lib.make_view(v["width"], v["height"], v["emission"], v["ratio"], v["out_off"], v["out_ext"],
                                    v["disp_off"], v["disp_ext"])
        ref = oracle_lib.render(case["traversal"], grid=glsl_golden.grid(case) if dda else None,
                                nodes=None if dda else glsl_golden.nodes(case),
                                camera=oracle_lib.make_camera(*case["camera"]), view=view)
        rgba, colour, words = glsl_golden.expected(case)
        assert np.array_equal(ref["rgba"], rgba), case["id"]
        assert np.array_equal(ref["emission"].view(np.uint32), colour.view(np.uint32)), case["id"]
        assert np.array_equal(ref["loads"], words), case["id"]


def test_reference_shader_recipe_rewrites(tmp_path):
    # the four rewrites oracle/glsl_ref.py makes on the way to the compiler,
    # on a stand-in shader
    import oracle.glsl_ref as glsl
    (tmp_path / "inc.glsl").write_text("struct Node { uint c[8]; };\nlayout(binding = 2) readonly buffer Octree {\n"
                                       "    Node nodes[];\n} model;\n")
    (tmp_path / "s.comp").write_text('#version 450\n#include "inc.glsl"\n#include "inc.glsl"\n'
                                     "uint find(vec3 pos, out vec3 base, out float side) { return 0; }\n"
                                     "// without out-of-bounds reads\n")
    src = glsl.shader_source(tmp_path, "s.comp")
    assert "#version" not in src and "#include" not in src
    assert src.count("struct Node") == 1
    assert "XoBuffer<Node> nodes;" in src
    assert "uint find(vec3 pos, vec3& base, float& side)" in src
    assert "// without out-of-bounds reads" in src


def test_oracle_matches_the_reference_shaders_random(oracle_lib):
    # the reference's shaders themselves (oracle/glsl_ref.py), where the
    # reference checkout is present, against the restatement on random grids
    # (1 to 47 texels a side), all three tree types, random voxel ratios and
    # cameras anywhere around or inside the volume: identical pixels, float
    # colours and word counts on every ray
    import oracle.glsl_ref as glsl
    if glsl.reference_dir() is not None:
        glsl.build()
    if not glsl.available():
        pytest.skip("reference sources not present")
    rng = np.random.default_rng(123)
    for i in range(90):
        dims = tuple(int(v) for v in rng.integers(1, 48, 3))
        g = np.zeros(dims + (4,), np.uint8)
        m = rng.random(dims) < rng.uniform(0.05, 0.7)
        g[m, :3] = rng.integers(0, 256, (int(m.sum()), 3))
        g[m, 3] = 255
        tree = ("sparse", "dag", "rope")[i % 3]
        nodes, _ = oracle_lib.build_svo(g, tree)
        t = rng.uniform(-1.5, 2.5, 3)
        f = rng.uniform(0, 1, 3) - t
        f = f / max(np.linalg.norm(f), 1e-3) * rng.uniform(0.5, 1.5)
        cam = tuple(tuple(float(x) for x in np.float32(v)) for v in (f, rng.normal(size=3), t))
        ratio = (1.0, 1.0, 1.0) if i % 4 else tuple(float(x) for x in rng.uniform(0.5, 2.0, 3))
        view = oracle_lib.make_view(24, 20, 5.0, ratio)
        for trav in glsl.SHADERS:
            if trav == "svo-rope" and tree != "rope":
                continue
            dda = trav == "dda"
            rgba, colour, words = glsl.render(trav, cam, 24, 20, emission=5.0, ratio=ratio, grid=g if dda else None,
                                              nodes=None if dda else nodes)
            ref = oracle_lib.render(trav, grid=g if dda else None, nodes=None if dda else nodes,
                                    camera=oracle_lib.make_camera(*cam), view=view)
            assert np.array_equal(ref["rgba"], rgba), (i, trav)
            assert np.array_equal(ref["emission"].view(np.uint32), colour.view(np.uint32)), (i, trav)
            assert np.array_equal(ref["loads"], words), (i, trav)

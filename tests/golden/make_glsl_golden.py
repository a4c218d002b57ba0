"""Generate tests/golden/glsl_golden.npz: images and per-ray colours from the
reference's own traversal shaders.

The shaders (resources/dda.comp, svo_naive.comp, esvo.comp, svo_df.comp,
svo_rope.comp with common.glsl and octree.glsl) are compiled for the CPU by
``oracle/glsl_ref.py`` and run once per pixel.  Each case stores the RGBA8
image and the float colour the shader hands to imageStore (after the emission
coefficient, before the RGBA8 conversion) and the 32-bit words each ray read
from the model (texels or node words: the roofline's algorithmic bytes / 4).
The volumes come from the
deterministic generators in ``xenodon_gb300.volumes`` and the octrees from the
oracle's builder (itself pinned byte for byte to the reference's builder by
svo_golden.npz); their SHA-256 is stored so that a test notices a generator
that changed.

Run from the repository root with the reference checkout named by
XENODON_REFERENCE:
    XENODON_REFERENCE=<checkout> python tests/golden/make_glsl_golden.py
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
import oracle.glsl_ref as glsl  # noqa: E402
from xenodon_gb300 import volumes  # noqa: E402

OUT = Path(__file__).resolve().parent / "glsl_golden.npz"

CAMS = {
    "front": ((0, 0, -0.8660254), (0, 1, 0), (0.5, 0.5, 2.5)),
    "oblique": ((0.35, -0.2, -0.91), (0.0, 0.976, -0.215), (0.2, 0.8, 2.0)),
    "inside": ((0.6, 0.3, 0.74), (-0.2, 0.95, 0.0), (0.45, 0.55, 0.5)),
    "grazing": ((1.0, 0.0, 0.0), (0, 1, 0), (-1.0, 0.5, 0.5)),
    "ct": ((0.3, -0.1, 0.95), (0, 1, 0.1), (0.3, 0.45, -1.2)),
    # the 128^3 blob configuration's camera line
    "c0": ((0, 0, -0.8660254), (0, 1, 0), (0.5, 0.5, 2.5)),
}
TRAV = ("dda", "svo-naive", "esvo", "svo-df", "svo-rope")

# volume id -> (generator, keyword arguments); every one is regenerated by the tests
VOLUMES = {
    "blobs32": ("blobs", dict(n=32, seed=0)),
    "ct61x45x50": ("ct_shell", dict(dx=61, dy=45, dz=50, seed=1, device="cpu")),
    "random32": ("random_grid", dict(dx=32, dy=32, dz=32, seed=9, density=0.4, levels=3)),
    "blobs128": ("blobs", dict(n=128, seed=0)),
    "ct512": ("ct_shell", dict(dx=512, dy=361, dz=512, seed=1, device="cpu")),
    "leaf1": ("constant", dict(shape=(1, 1, 1), rgba=(200, 100, 50, 255))),
    "two2": ("two_voxels", dict()),
}


def make_volume(vid: str) -> np.ndarray:
    gen, kw = VOLUMES[vid]
    if gen == "constant":
        g = np.zeros(kw["shape"] + (4,), np.uint8)
        g[...] = kw["rgba"]
        return g
    if gen == "two_voxels":
        g = np.zeros((2, 2, 2, 4), np.uint8)
        g[0, 1, 0, :3] = (90, 20, 200)
        g[1, 0, 1, :3] = (10, 250, 30)
        return g
    return getattr(volumes, gen)(**kw)


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def cases():
    """(case id, volume id, tree type, traversal, camera, view keywords)."""
    from xenodon_gb300 import cameras
    out = []
    for cam in ("front", "oblique", "inside", "grazing"):
        for t in TRAV:
            out.append((f"blobs32-{cam}-{t}", "blobs32", "rope", t, CAMS[cam], dict(width=48, height=40)))
    for cam in ("ct", "oblique", "inside"):
        for t in TRAV:
            out.append((f"ct-{cam}-{t}", "ct61x45x50", "rope", t, CAMS[cam], dict(width=40, height=32)))
    # one region of a larger display, with an anisotropic voxel ratio
    for t in TRAV:
        out.append((f"ct-region-{t}", "ct61x45x50", "rope", t, CAMS["ct"],
                    dict(width=0, height=0, ratio=(1.0, 1.5, 0.75), out_off=(40, 16), out_ext=(50, 37),
                         disp_off=(0, 0), disp_ext=(128, 72), emission=7.0)))
    for t in ("svo-naive", "esvo", "svo-df"):
        out.append((f"dag-oblique-{t}", "random32", "dag", t, CAMS["oblique"], dict(width=40, height=32, emission=5.0)))
        out.append((f"sparse-grazing-{t}", "random32", "sparse", t, CAMS["grazing"], dict(width=40, height=32)))
    for vid in ("leaf1", "two2"):
        for cam in ("front", "inside"):
            for t in TRAV:
                out.append((f"{vid}-{cam}-{t}", vid, "rope", t, CAMS[cam], dict(width=24, height=20)))
    # the 128^3 blob configuration at 512x512, every 16th row
    for row in range(0, 512, 16):
        out.append((f"c0-row{row:03d}-dda", "blobs128", None, "dda", CAMS["c0"],
                    dict(width=0, height=0, out_off=(0, row), out_ext=(512, 1), disp_off=(0, 0),
                         disp_ext=(512, 512))))
    # the 512x361x512 CT configuration at 1920x1080: a frame from each leg of
    # its path (orbit 37, dolly 220, rotation about an interior point 330 and
    # 440), two rows each, every traversal
    path = cameras.ct_path()
    for frame in (37, 220, 330, 440):
        cam = tuple(tuple(float(x) for x in v) for v in path[frame])
        for row in (11 + frame % 7, 540 + frame % 13):
            for t in TRAV:
                out.append((f"c1-f{frame}-row{row:04d}-{t}", "ct512", "rope", t, cam,
                            dict(width=0, height=0, out_off=(0, row), out_ext=(1920, 1), disp_off=(0, 0),
                                 disp_ext=(1920, 1080))))
    return out


def view_args(kw):
    return dict(emission=kw.get("emission", 10.0), ratio=kw.get("ratio", (1.0, 1.0, 1.0)),
                out_off=kw.get("out_off", (0, 0)), out_ext=kw.get("out_ext"), disp_off=kw.get("disp_off", (0, 0)),
                disp_ext=kw.get("disp_ext"))


def main() -> None:
    if not glsl.build():
        raise SystemExit("set XENODON_REFERENCE to the reference checkout")
    grids, trees, hashes, meta, arrays = {}, {}, {}, [], {}
    for cid, vid, typ, trav, cam, kw in cases():
        if vid not in grids:
            grids[vid] = make_volume(vid)
            hashes[vid] = sha(grids[vid])
        grid = grids[vid]
        nodes = None
        if trav != "dda":
            if (vid, typ) not in trees:
                trees[(vid, typ)] = oracle.build_svo(grid, typ)[0]
                hashes[(vid, typ)] = sha(trees[(vid, typ)])
            nodes = trees[(vid, typ)]
        rgba, colour, words = glsl.render(trav, cam, kw["width"], kw["height"], grid=grid if trav == "dda" else None,
                                          nodes=nodes, **view_args(kw))
        arrays[f"{cid}/rgba"] = rgba
        arrays[f"{cid}/colour"] = colour
        arrays[f"{cid}/words"] = words
        meta.append(dict(id=cid, volume=vid, tree=typ, traversal=trav, camera=cam, view=kw,
                         grid_sha256=hashes[vid], nodes_sha256=None if nodes is None else hashes[(vid, typ)]))
    arrays["cases"] = np.frombuffer(json.dumps(dict(volumes=VOLUMES, cases=meta)).encode(), np.uint8)
    np.savez_compressed(OUT, **arrays)
    print(f"{len(meta)} cases -> {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()

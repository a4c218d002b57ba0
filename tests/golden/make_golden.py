"""Generate the golden SVO fixtures in tests/golden/svo_golden.npz.

The octree bytes come from the reference's own builder (src/model/Octree.cpp,
src/model/OctreeConstruction.h, src/model/Grid.cpp compiled unmodified from the
reference sources by ``make -C oracle ref``).  The input grids are stored in the
fixture too, so the tests never regenerate them.

Run from the repository root, in a checkout that has the reference sources:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402


def grids():
    rng = np.random.default_rng(12345)
    out = {}
    # non-power-of-two blob with a colour gradient and a uniform core
    dz, dy, dx = 13, 11, 16
    z, y, x = np.mgrid[0:dz, 0:dy, 0:dx]
    g = np.zeros((dz, dy, dx, 4), np.uint8)
    r = np.sqrt((x - 8.0) ** 2 + (y - 5.0) ** 2 + (z - 6.0) ** 2)
    m = r < 5.5
    g[m, 0] = 200
    g[m, 1] = (x[m] * 9) % 256
    g[m, 2] = 40
    g[m, 3] = 255
    g[r < 2.5] = (90, 90, 90, 255)
    out["blob13x11x16"] = g
    # sparse random voxels with a few repeated colours (DAG sharing)
    g = np.zeros((9, 7, 5, 4), np.uint8)
    m = rng.random((9, 7, 5)) < 0.3
    pal = np.array([[255, 0, 0, 255], [0, 255, 0, 255], [20, 20, 200, 255]], np.uint8)
    g[m] = pal[rng.integers(0, 3, m.sum())]
    out["sparse9x7x5"] = g
    # single voxel
    out["one1x1x1"] = np.array([[[[10, 20, 30, 255]]]], np.uint8)
    # 16^3 with repeated 4^3 tiles: the DAG collapses them
    tile = rng.integers(0, 2, (4, 4, 4, 1)).astype(np.uint8) * np.array([250, 120, 10, 255], np.uint8)
    out["tiled16"] = np.tile(tile, (4, 4, 4, 1))
    # smooth noise for the lossy heuristics
    base = rng.random((6, 6, 6))
    big = np.kron(base, np.ones((3, 3, 3)))[:17, :13, :11]
    g = np.zeros(big.shape + (4,), np.uint8)
    g[..., 0] = (big * 255).astype(np.uint8)
    g[..., 1] = (big * 128).astype(np.uint8)
    g[..., 3] = 255
    g[big < 0.3] = 0
    out["smooth17x13x11"] = g
    return out


CASES = [
    ("sparse", "chan-diff", 0), ("dag", "chan-diff", 0), ("rope", "chan-diff", 0),
    ("sparse", "chan-diff", 40), ("rope", "chan-diff", 40), ("dag", "chan-diff", 40),
    ("sparse", "std-dev", 0.0), ("sparse", "std-dev", 25.5), ("rope", "std-dev", 25.5),
    ("dag", "std-dev", 12.0),
]


def main():
    if not oracle.build_ref():
        raise SystemExit("the reference sources are required to make golden fixtures")
    arrays, meta = {}, []
    for gname, g in grids().items():
        arrays[f"grid__{gname}"] = g
        for t, h, th in CASES:
            data, stats = oracle.ref_build_svo(g, t, h, th)
            key = f"svo__{gname}__{t}__{h}__{th}"
            arrays[key] = np.frombuffer(data, np.uint8)
            meta.append({"key": key, "grid": gname, "type": t, "heuristic": h, "threshold": th,
                         "stats": stats})
    arrays["meta"] = np.frombuffer(json.dumps(meta).encode(), np.uint8)
    np.savez_compressed(Path(__file__).with_name("svo_golden.npz"), **arrays)
    print(f"wrote {len(meta)} golden octrees")


if __name__ == "__main__":
    main()

"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def built_library():
    """Build libxenodon.so and the CLI in-tree (incremental)."""
    from xenodon_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def ctx(built_library):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import xenodon_gb300 as xg
    c = xg.Context(0)
    yield c
    c.close()


class VolumeChanged(Exception):
    """A regenerated golden volume's bytes differ from the stored hash."""


class GlslGolden:
    """tests/golden/glsl_golden.npz: images and per-ray colours made by the
    reference's own traversal shaders (tests/golden/make_glsl_golden.py), with
    the volumes regenerated from the same deterministic generators and checked
    against the stored SHA-256."""

    def __init__(self):
        import json
        import numpy as np
        self.z = np.load(ROOT / "tests" / "golden" / "glsl_golden.npz")
        spec = json.loads(bytes(self.z["cases"]).decode())
        self.volumes = spec["volumes"]
        self.cases = spec["cases"]
        self._grids, self._trees = {}, {}

    def grid(self, case):
        import hashlib
        import numpy as np
        from xenodon_gb300 import volumes
        vid = case["volume"]
        if vid not in self._grids:
            gen, kw = self.volumes[vid]
            if gen == "constant":
                g = np.zeros(tuple(kw["shape"]) + (4,), np.uint8)
                g[...] = kw["rgba"]
            elif gen == "two_voxels":
                g = np.zeros((2, 2, 2, 4), np.uint8)
                g[0, 1, 0, :3] = (90, 20, 200)
                g[1, 0, 1, :3] = (10, 250, 30)
            else:
                g = getattr(volumes, gen)(**kw)
            if hashlib.sha256(g.tobytes()).hexdigest() != case["grid_sha256"]:
                raise VolumeChanged(f"generator of {vid} changed")
            self._grids[vid] = g
        return self._grids[vid]

    def tree(self, case):
        """(nodes, side) of the case's octree, built by the oracle's builder."""
        import hashlib
        import oracle
        key = (case["volume"], case["tree"])
        if key not in self._trees:
            nodes, stats = oracle.build_svo(self.grid(case), case["tree"])
            assert hashlib.sha256(nodes.tobytes()).hexdigest() == case["nodes_sha256"], f"octree of {key} changed"
            self._trees[key] = (nodes, stats["side"])
        return self._trees[key]

    def nodes(self, case):
        return self.tree(case)[0]

    def expected(self, case):
        """RGBA8 image, float colour and words read per ray."""
        return self.z[case["id"] + "/rgba"], self.z[case["id"] + "/colour"], self.z[case["id"] + "/words"]

    @staticmethod
    def view(case):
        v = case["view"]
        return dict(width=v["width"], height=v["height"], emission=v.get("emission", 10.0),
                    ratio=tuple(v.get("ratio", (1.0, 1.0, 1.0))), out_off=tuple(v.get("out_off", (0, 0))),
                    out_ext=tuple(v["out_ext"]) if v.get("out_ext") else None,
                    disp_off=tuple(v.get("disp_off", (0, 0))),
                    disp_ext=tuple(v["disp_ext"]) if v.get("disp_ext") else None)


@pytest.fixture(scope="session")
def glsl_golden():
    return GlslGolden()

"""The reference's own traversal shaders, compiled for the CPU -- TEST
INFRASTRUCTURE ONLY.

Recipe: each compute shader of the reference checkout (resources/dda.comp,
svo_naive.comp, esvo.comp, svo_df.comp, svo_rope.comp, with the common.glsl
and octree.glsl they include) is streamed into g++ behind ``glsl/shim.h`` and
followed by ``glsl/entry.inc``, and built into ``oracle/_ref/glsl_<shader>.so``.
Nothing is written into the repository but those libraries (git-ignored).  On
the way the text gets four mechanical rewrites, and no other change:

* the ``#version`` line is dropped (not a C++ directive);
* ``#include "<file>.glsl"`` is replaced by that file, rewritten the same way;
* an ``out T name`` parameter becomes ``T& name`` (GLSL copies an out
  parameter back on return; every such parameter in these shaders is only
  written, immediately before a return, so a reference is the same);
* a buffer block's unsized array ``T name[];`` becomes ``XoBuffer<T> name;``
  (an array view that counts its accesses: the words the shader reads).

The libraries run the shader's ``main`` once per pixel, with the push
constants and uniforms the reference's host code sets.  They make golden
images and per-ray colours for the oracle (``tests/golden/make_glsl_golden.py``);
the reference checkout is needed to build them, so they exist only where it
is.  The checkout: the ``XENODON_REFERENCE`` environment variable.
"""
from __future__ import annotations

import ctypes
import os
import re
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SHADERS = {"dda": "dda.comp", "svo-naive": "svo_naive.comp", "esvo": "esvo.comp", "svo-df": "svo_df.comp",
           "svo-rope": "svo_rope.comp"}
CXXFLAGS = ["-std=c++17", "-O1", "-fno-aggressive-loop-optimizations", "-fno-strict-aliasing",
            "-ffp-contract=off", "-fno-fast-math", "-ftrivial-auto-var-init=zero", "-fPIC", "-shared",
            "-fvisibility=hidden", "-w"]

_INCLUDE = re.compile(r'^\s*#\s*include\s+"([^"]+\.glsl)"\s*$')
_VERSION = re.compile(r"^\s*#\s*version\b")
_OUT_PARAM = re.compile(r"\bout\s+([A-Za-z_][A-Za-z0-9_]*)\s+([A-Za-z_][A-Za-z0-9_]*)")
_UNSIZED = re.compile(r"^(\s*)([A-Za-z_][A-Za-z0-9_]*)\s+([A-Za-z_][A-Za-z0-9_]*)\s*\[\s*\]\s*;")


def reference_dir() -> Path | None:
    ref = os.environ.get("XENODON_REFERENCE", "")
    if ref and (Path(ref) / "resources" / "dda.comp").exists():
        return Path(ref)
    return None


def shader_source(resources: Path, name: str, _seen: set | None = None) -> str:
    """The shader file `name` with the four rewrites applied."""
    seen = set() if _seen is None else _seen
    out = []
    for line in (resources / name).read_text().splitlines():
        if _VERSION.match(line):
            continue
        m = _INCLUDE.match(line)
        if m:
            inc = m.group(1)
            if inc not in seen:
                seen.add(inc)
                out.append(shader_source(resources, inc, seen))
            continue
        line = _OUT_PARAM.sub(r"\1& \2", line)
        line = _UNSIZED.sub(r"\1XoBuffer<\2> \3;", line)
        out.append(line)
    return "\n".join(out)


def library_path(trav: str) -> Path:
    return OUT / f"glsl_{Path(SHADERS[trav]).stem}.so"


def build(ref: Path | None = None, cxx: str = "g++") -> list[Path]:
    """Compile every shader; returns the libraries built (none without a
    reference checkout)."""
    ref = ref or reference_dir()
    if ref is None:
        return []
    OUT.mkdir(exist_ok=True)
    built = []
    for trav, name in SHADERS.items():
        text = ('#include "shim.h"\n' + shader_source(ref / "resources", name) + "\n" +
                (HERE / "glsl" / "entry.inc").read_text())
        dst = library_path(trav)
        subprocess.run([cxx, *CXXFLAGS, "-I", str(HERE / "glsl"), "-x", "c++", "-", "-o", str(dst)],
                       input=text.encode(), check=True)
        built.append(dst)
    return built


def available() -> bool:
    return all(library_path(t).exists() for t in SHADERS)


_libs: dict = {}


def _lib(trav: str):
    if trav not in _libs:
        lib = ctypes.CDLL(str(library_path(trav)))
        fn = lib.xo_glsl_render
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_void_p, ctypes.c_void_p,
                       ctypes.c_void_p]
        _libs[trav] = (lib, fn)
    return _libs[trav][1]


def render(trav: str, camera, width: int, height: int, emission: float = 10.0, ratio=(1.0, 1.0, 1.0),
           out_off=(0, 0), out_ext=None, disp_off=(0, 0), disp_ext=None, grid: np.ndarray | None = None,
           nodes: np.ndarray | None = None):
    """Run the reference shader `trav` over an output region.  camera:
    (forward, up, translation); grid: (dz, dy, dx, 4) uint8 for dda; nodes:
    (n, 10) uint32 for the octree shaders.  Returns (rgba (h, w, 4) uint8,
    colour (h, w, 3) float32: the colour handed to imageStore, words (h, w)
    uint32: the words each invocation read from the model)."""
    out_ext = out_ext or (width, height)
    disp_ext = disp_ext or (width, height)
    w, h = out_ext
    cam = np.ascontiguousarray(np.concatenate([np.asarray(c, np.float32) for c in camera]), np.float32)
    region = np.array([out_off[0], out_off[1], disp_off[0], disp_off[1]], np.int32)
    extent = np.array([w, h, disp_ext[0], disp_ext[1]], np.uint32)
    rat = np.asarray(ratio, np.float32)
    if trav == "dda":
        g = np.ascontiguousarray(grid, np.uint8)
        dims = np.array([g.shape[2], g.shape[1], g.shape[0]], np.uint32)
        gp, npn = g.ctypes.data, None
    else:
        nd = np.ascontiguousarray(nodes, np.uint32)
        dims = np.zeros(3, np.uint32)
        gp, npn = None, nd.ctypes.data
    colour = np.zeros((h, w, 4), np.float32)
    rgba = np.zeros((h, w, 4), np.uint8)
    words = np.zeros((h, w), np.uint32)
    _lib(trav)(gp, dims.ctypes.data, npn, cam.ctypes.data, region.ctypes.data, extent.ctypes.data,
               rat.ctypes.data, float(emission), colour.ctypes.data, rgba.ctypes.data, words.ctypes.data)
    return rgba, colour[..., :3].copy(), words

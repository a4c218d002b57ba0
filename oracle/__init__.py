"""Oracle for the Xenodon volume ray-traversal path -- TEST INFRASTRUCTURE ONLY.

ctypes bindings to ``oracle/_build/liboracle.so``, the C restatement of the
reference shaders (resources/*.comp, common.glsl, octree.glsl) and of its
octree build (src/model/OctreeConstruction.h, Octree.cpp, Grid.cpp).  Only the
tests, ``__graft_entry__.smoke()`` and the benchmark's CPU-baseline leg use it;
the product library never does.  ``oracle.glsl_ref`` compiles the reference's
own shaders for the CPU, which made the golden images that pin the
restatement.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"
REF_BUILDER = HERE / "_ref" / "xn_ref_build"
REF_CONFIG = HERE / "_ref" / "xn_ref_config"
REF_PNG = HERE / "_ref" / "xn_ref_png"
REF_RECT = HERE / "_ref" / "xn_ref_rect"

TRAVERSALS = {"dda": 0, "svo-naive": 1, "esvo": 2, "svo-df": 3, "svo-rope": 4}
TYPES = {"sparse": 0, "dag": 1, "rope": 2}
HEURISTICS = {"chan-diff": 0, "std-dev": 1}
ERR_ITER, ERR_STACK, ERR_INDEX = 1, 2, 4


class Camera(ctypes.Structure):
    _fields_ = [("forward", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("translation", ctypes.c_float * 3)]


class View(ctypes.Structure):
    _fields_ = [("output_offset", ctypes.c_int32 * 2), ("output_extent", ctypes.c_uint32 * 2),
                ("display_offset", ctypes.c_int32 * 2), ("display_extent", ctypes.c_uint32 * 2),
                ("voxel_ratio", ctypes.c_float * 3), ("emission_coeff", ctypes.c_float)]


class Volume(ctypes.Structure):
    _fields_ = [("rgba", ctypes.c_void_p), ("dim", ctypes.c_uint32 * 3),
                ("nodes", ctypes.c_void_p), ("n_nodes", ctypes.c_uint64)]


class BuildStats(ctypes.Structure):
    _fields_ = [("total_leaves", ctypes.c_uint64), ("unique_leaves", ctypes.c_uint64),
                ("total_nodes", ctypes.c_uint64), ("depth", ctypes.c_uint64),
                ("side", ctypes.c_uint64), ("n_nodes", ctypes.c_uint64)]


_lib = None


def build() -> None:
    """Compile the C restatement (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


def build_ref() -> bool:
    """Compile the reference's own builder from the checkout that
    XENODON_REFERENCE names; without one, report whether a builder was
    compiled before."""
    ref = os.environ.get("XENODON_REFERENCE", "")
    if not ref or not (Path(ref) / "src" / "model" / "OctreeConstruction.h").exists():
        return REF_BUILDER.exists()
    subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REFERENCE={ref}"], check=True)
    return True


def build_ref_config() -> bool:
    """Compile the reference's own headless.conf parser (src/core/Parser.cpp,
    Config.h, src/backend/headless/HeadlessConfig.cpp) from the checkout that
    XENODON_REFERENCE names; without one, report whether it was compiled
    before."""
    ref = os.environ.get("XENODON_REFERENCE", "")
    if not ref or not (Path(ref) / "src" / "core" / "Parser.cpp").exists():
        return REF_CONFIG.exists()
    subprocess.run(["make", "-s", "-C", str(HERE), "ref-config", f"REFERENCE={ref}"], check=True)
    return True


def build_ref_png() -> bool:
    """Compile a decoder from the reference's PNG library (subprojects/lodepng)
    from the checkout that XENODON_REFERENCE names; without one, report
    whether it was compiled before."""
    ref = os.environ.get("XENODON_REFERENCE", "")
    if not ref or not (Path(ref) / "subprojects" / "lodepng" / "lodepng.cpp").exists():
        return REF_PNG.exists()
    subprocess.run(["make", "-s", "-C", str(HERE), "ref-png", f"REFERENCE={ref}"], check=True)
    return True


def build_ref_rect() -> bool:
    """Compile the reference's own rect_union (src/utility/rect_union.h) behind
    a driver, from the checkout that XENODON_REFERENCE names; without one,
    report whether it was compiled before."""
    ref = os.environ.get("XENODON_REFERENCE", "")
    if not ref or not (Path(ref) / "src" / "utility" / "rect_union.h").exists():
        return REF_RECT.exists()
    subprocess.run(["make", "-s", "-C", str(HERE), "ref-rect", f"REFERENCE={ref}"], check=True)
    return True


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        l = ctypes.CDLL(str(LIB_PATH))
        for name, ftype in (("xo_render_f32", ctypes.c_float), ("xo_render_f64", ctypes.c_double)):
            fn = getattr(l, name)
            fn.restype = ctypes.c_int64
            fn.argtypes = [ctypes.c_int, ctypes.POINTER(Volume), ctypes.POINTER(Camera),
                           ctypes.POINTER(View), ctypes.c_void_p, ctypes.c_void_p,
                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        l.xo_build_svo.restype = ctypes.c_int
        l.xo_build_svo.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint32 * 3), ctypes.c_int,
                                   ctypes.c_int, ctypes.c_double,
                                   ctypes.POINTER(ctypes.POINTER(ctypes.c_uint32)),
                                   ctypes.POINTER(BuildStats)]
        l.xo_free.restype = None
        l.xo_free.argtypes = [ctypes.c_void_p]
        _lib = l
    return _lib


def make_camera(forward, up, translation) -> Camera:
    c = Camera()
    c.forward[:] = [float(v) for v in forward]
    c.up[:] = [float(v) for v in up]
    c.translation[:] = [float(v) for v in translation]
    return c


def make_view(width, height, emission_coeff=1.0, voxel_ratio=(1.0, 1.0, 1.0),
              output_offset=(0, 0), output_extent=None, display_offset=(0, 0),
              display_extent=None) -> View:
    v = View()
    v.output_offset[:] = list(output_offset)
    v.output_extent[:] = list(output_extent or (width, height))
    v.display_offset[:] = list(display_offset)
    v.display_extent[:] = list(display_extent or (width, height))
    v.voxel_ratio[:] = [float(x) for x in voxel_ratio]
    v.emission_coeff = float(emission_coeff)
    return v


def render(traversal, *, grid=None, nodes=None, camera: Camera, view: View, f64=False,
           threads=None, want_loads=True):
    """Render one output region with the oracle.

    grid: uint8 array (dz, dy, dx, 4); nodes: uint32 array (n, 10).
    Returns dict(rgba (h, w, 4) u8, emission (h, w, 3), loads (h, w) u32,
    err (h, w) u8, errors int).
    """
    t = TRAVERSALS[traversal] if isinstance(traversal, str) else int(traversal)
    vol = Volume()
    keep = []
    if grid is not None:
        g = np.ascontiguousarray(grid, dtype=np.uint8)
        keep.append(g)
        vol.rgba = g.ctypes.data
        vol.dim[:] = [g.shape[2], g.shape[1], g.shape[0]]
    if nodes is not None:
        n = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(-1, 10)
        keep.append(n)
        vol.nodes = n.ctypes.data
        vol.n_nodes = n.shape[0]
    w, h = view.output_extent[0], view.output_extent[1]
    rgba = np.zeros((h, w, 4), np.uint8)
    em = np.zeros((h, w, 3), np.float64 if f64 else np.float32)
    loads = np.zeros((h, w), np.uint32) if want_loads else None
    err = np.zeros((h, w), np.uint8)
    fn = lib().xo_render_f64 if f64 else lib().xo_render_f32
    nthreads = threads or os.cpu_count() or 1
    r = fn(t, ctypes.byref(vol), ctypes.byref(camera), ctypes.byref(view), rgba.ctypes.data,
           em.ctypes.data, loads.ctypes.data if loads is not None else None, err.ctypes.data, nthreads)
    if r < 0:
        raise ValueError("oracle render: bad arguments")
    return {"rgba": rgba, "emission": em, "loads": loads, "err": err, "errors": int(r)}


def build_svo(grid, svo_type="sparse", heuristic="chan-diff", threshold=0.0):
    """Build an octree with the C restatement.  grid: uint8 (dz, dy, dx, 4).

    Returns (nodes uint32 (n, 10), stats dict)."""
    g = np.ascontiguousarray(grid, dtype=np.uint8)
    dim = (ctypes.c_uint32 * 3)(g.shape[2], g.shape[1], g.shape[0])
    out = ctypes.POINTER(ctypes.c_uint32)()
    st = BuildStats()
    r = lib().xo_build_svo(g.ctypes.data, ctypes.byref(dim), TYPES[svo_type], HEURISTICS[heuristic],
                           float(threshold), ctypes.byref(out), ctypes.byref(st))
    if r != 0:
        raise RuntimeError(f"oracle build failed ({r})")
    n = st.n_nodes
    arr = np.ctypeslib.as_array(out, shape=(n * 10,)).copy().reshape(n, 10)
    lib().xo_free(out)
    stats = {f: int(getattr(st, f)) for f, _ in BuildStats._fields_}
    return arr, stats


def svo_file_bytes(nodes, side) -> bytes:
    """Serialise in the XNDN-SVO layout (src/model/Octree.cpp:96-114)."""
    n = np.ascontiguousarray(nodes, dtype="<u4").reshape(-1, 10)
    return b"XNDN-SVO" + int(side).to_bytes(8, "little") + int(n.shape[0]).to_bytes(8, "little") + n.tobytes()


def ref_build_svo(grid, svo_type="sparse", heuristic="chan-diff", threshold=0, workdir=None):
    """Run the reference's own builder (oracle/_ref) and return (file bytes, stats)."""
    import tempfile
    if not REF_BUILDER.exists():
        raise FileNotFoundError(REF_BUILDER)
    g = np.ascontiguousarray(grid, dtype=np.uint8)
    with tempfile.TemporaryDirectory(dir=workdir) as d:
        raw = Path(d) / "grid.raw"
        out = Path(d) / "out.svo"
        raw.write_bytes(g.tobytes())
        val = str(int(threshold)) if heuristic == "chan-diff" else repr(float(threshold))
        p = subprocess.run([str(REF_BUILDER), str(raw), str(g.shape[2]), str(g.shape[1]), str(g.shape[0]),
                            svo_type, heuristic, val, str(out)], check=True, capture_output=True, text=True)
        f = p.stdout.split()
        stats = dict(zip(["total_leaves", "unique_leaves", "total_nodes", "depth", "side", "n_nodes"],
                         map(int, f)))
        return out.read_bytes(), stats

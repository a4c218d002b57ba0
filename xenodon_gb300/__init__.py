"""xenodon_gb300: GB300-native volume ray traversal (Xenodon's hot path).

Thin ctypes bindings over the C ABI in include/xenodon.h, implemented by
``xenodon_gb300/lib/libxenodon.so`` (CUDA kernels for sm_103a + host code).
There is no CPU fallback: if the library is missing, importing the bindings
raises.  Build it with ``python -m xenodon_gb300.build``.

Traversal names follow ``xenodon render -s`` (src/main_loop.cpp:37-43).
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libxenodon.so"
CLI_PATH = PKG / "bin" / "xenodon"

TRAVERSALS = {"dda": 0, "svo-naive": 1, "esvo": 2, "svo-df": 3, "svo-rope": 4}
SVO_TRAVERSALS = ("svo-naive", "esvo", "svo-df", "svo-rope")
SVO_TYPES = {"sparse": 0, "dag": 1, "rope": 2}
XN_BUILD_LEAN = 0x100  # xn_build_svo_volume: write the device layout directly (sparse trees)
XN_OUTPUT_DISCARD = 1  # xn_output_render: no read-back
HEURISTICS = {"chan-diff": 0, "std-dev": 1}

XN_OK = 0
XN_ERR_ARG, XN_ERR_CUDA, XN_ERR_NOMEM, XN_ERR_FORMAT = -1, -2, -3, -4
XN_ERR_BUDGET, XN_ERR_RAY_LIMIT, XN_ERR_IO, XN_ERR_STATE = -5, -6, -7, -8

# Every symbol include/xenodon.h declares.
EXPORTS = (
    "xn_create", "xn_destroy", "xn_last_error", "xn_abi_version", "xn_ctx_memory",
    "xn_volume_upload_grid", "xn_volume_upload_grid_device", "xn_build_svo_volume", "xn_volume_upload_svo", "xn_volume_release", "xn_volume_info_get",
    "xn_render", "xn_render_device", "xn_ray_errors", "xn_build_svo", "xn_build_svo_static", "xn_free",
    "xn_render_batch", "xn_autotune_batch", "xn_batch_graph_create", "xn_batch_graph_launch",
    "xn_batch_graph_destroy", "xn_server_create", "xn_server_destroy", "xn_server_add_grid",
    "xn_server_add_svo", "xn_server_add_volume", "xn_server_submit", "xn_server_wait", "xn_server_stats",
    "xn_svo_load", "xn_svo_save", "xn_volume_save", "xn_volume_load", "xn_tiff_load", "xn_tiff_save",
    "xn_png_save", "xn_build_svo_streamed", "xn_volume_upload_svo_fmt", "xn_output_create", "xn_output_render", "xn_output_wait", "xn_output_destroy",
)


class XenodonError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"{message} (status {code})")
        self.code = code


class Camera(ctypes.Structure):
    _fields_ = [("forward", ctypes.c_float * 3), ("up", ctypes.c_float * 3),
                ("translation", ctypes.c_float * 3)]


class Rect(ctypes.Structure):
    _fields_ = [("x", ctypes.c_int32), ("y", ctypes.c_int32),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32)]


class Params(ctypes.Structure):
    _fields_ = [("output_region", Rect), ("display_region", Rect),
                ("voxel_ratio", ctypes.c_float * 3), ("emission_coeff", ctypes.c_float)]


class VolumeInfo(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("dim", ctypes.c_uint32 * 3), ("side", ctypes.c_uint64),
                ("n_nodes", ctypes.c_uint64), ("device_bytes", ctypes.c_uint64), ("has_ropes", ctypes.c_int)]


class Job(ctypes.Structure):
    _fields_ = [("volume", ctypes.c_void_p), ("traversal", ctypes.c_int), ("camera", Camera),
                ("params", Params), ("d_rgba", ctypes.c_void_p)]


class BatchConfig(ctypes.Structure):
    _fields_ = [("tile_width", ctypes.c_uint32), ("block_threads", ctypes.c_uint32),
                ("blocks_per_sm", ctypes.c_uint32), ("chunk", ctypes.c_uint32)]

    def as_dict(self) -> dict:
        return {f: int(getattr(self, f)) for f, _ in self._fields_}


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget", ctypes.c_uint64), ("max_batch_jobs", ctypes.c_int), ("streams", ctypes.c_int),
                ("fold_max_pixels", ctypes.c_uint64), ("fold_idle_us", ctypes.c_uint32),
                ("fold_blocks_per_sm", ctypes.c_uint32), ("band_pixels", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64), ("batches", ctypes.c_uint64),
                ("uploads", ctypes.c_uint64), ("evictions", ctypes.c_uint64), ("rays", ctypes.c_uint64),
                ("hbm_used", ctypes.c_uint64), ("mean_batch", ctypes.c_double), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("max_ms", ctypes.c_double), ("mrays_per_s", ctypes.c_double),
                ("folded", ctypes.c_uint64), ("fold_launches", ctypes.c_uint64), ("republished", ctypes.c_uint64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


class BuildStats(ctypes.Structure):
    _fields_ = [("total_leaves", ctypes.c_uint64), ("unique_leaves", ctypes.c_uint64),
                ("total_nodes", ctypes.c_uint64), ("depth", ctypes.c_uint64),
                ("side", ctypes.c_uint64), ("n_nodes", ctypes.c_uint64)]


REGION_READER = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                 ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, ctypes.POINTER(ctypes.c_uint8))

_lib = None


def load_library(path: Path | str | None = None) -> ctypes.CDLL:
    """Load libxenodon.so; raises if it has not been built."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: build it with `python -m xenodon_gb300.build`")
    l = ctypes.CDLL(str(p))
    P = ctypes.POINTER
    vp, u32, u64, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int
    sig = {
        "xn_create": (i32, [i32, u64, P(vp)]),
        "xn_destroy": (i32, [vp]),
        "xn_last_error": (ctypes.c_char_p, []),
        "xn_abi_version": (i32, []),
        "xn_ctx_memory": (i32, [vp, P(u64), P(u64)]),
        "xn_volume_upload_grid": (i32, [vp, vp, u32, u32, u32, P(vp)]),
        "xn_volume_upload_svo": (i32, [vp, vp, u64, u64, P(vp)]),
        "xn_volume_upload_grid_device": (i32, [vp, vp, u32, u32, u32, P(vp)]),
        "xn_build_svo_volume": (i32, [vp, vp, u32, u32, u32, i32, i32, ctypes.c_double, P(vp), P(BuildStats)]),
        "xn_volume_release": (i32, [vp]),
        "xn_volume_info_get": (i32, [vp, P(VolumeInfo)]),
        "xn_render": (i32, [vp, vp, i32, P(Camera), P(Params), vp, vp, P(ctypes.c_float)]),
        "xn_render_device": (i32, [vp, vp, i32, P(Camera), P(Params), vp, vp, vp, vp]),
        "xn_ray_errors": (i32, [vp, P(u32), i32]),
        "xn_build_svo": (i32, [vp, vp, u32, u32, u32, i32, i32, ctypes.c_double, P(P(u32)), P(BuildStats)]),
        "xn_build_svo_static": (i32, [vp, u32, u32, u32, i32, i32, ctypes.c_double, vp, u64, P(BuildStats), vp]),
        "xn_free": (None, [vp]),
        "xn_render_batch": (i32, [vp, P(Job), i32, P(BatchConfig), vp]),
        "xn_autotune_batch": (i32, [vp, P(Job), i32, vp, P(BatchConfig), P(ctypes.c_float)]),
        "xn_batch_graph_create": (i32, [vp, i32, P(BatchConfig), vp, P(vp)]),
        "xn_batch_graph_launch": (i32, [vp, P(Job), i32]),
        "xn_batch_graph_destroy": (i32, [vp]),
        "xn_server_create": (i32, [vp, P(ServerConfig), P(vp)]),
        "xn_server_destroy": (i32, [vp]),
        "xn_server_add_grid": (i32, [vp, u32, vp, u32, u32, u32]),
        "xn_server_add_svo": (i32, [vp, u32, vp, u64, u64]),
        "xn_server_add_volume": (i32, [vp, u32, vp]),
        "xn_server_submit": (i32, [vp, u32, i32, P(Camera), P(Params), vp, P(u64)]),
        "xn_server_wait": (i32, [vp, u64, ctypes.c_double, P(ctypes.c_double)]),
        "xn_server_stats": (i32, [vp, P(ServerStats)]),
        "xn_svo_load": (i32, [ctypes.c_char_p, P(P(u32)), P(u64), P(u64)]),
        "xn_svo_save": (i32, [ctypes.c_char_p, vp, u64, u64]),
        "xn_volume_save": (i32, [vp, vp, ctypes.c_char_p]),
        "xn_volume_load": (i32, [vp, ctypes.c_char_p, ctypes.POINTER(vp)]),
        "xn_tiff_load": (i32, [ctypes.c_char_p, P(P(ctypes.c_uint8)), P(u32 * 3)]),
        "xn_tiff_save": (i32, [ctypes.c_char_p, vp, u32, u32, u32]),
        "xn_png_save": (i32, [ctypes.c_char_p, vp, u32, u32]),
        "xn_build_svo_streamed": (i32, [vp, u32, u32, u32, i32, ctypes.c_double, REGION_READER, vp,
                                        ctypes.c_char_p, P(BuildStats)]),
        "xn_volume_upload_svo_fmt": (i32, [vp, vp, u64, u64, i32, P(vp)]),
        "xn_output_create": (i32, [vp, u64, P(vp)]),
        "xn_output_render": (i32, [vp, vp, i32, P(Camera), P(Params), i32]),
        "xn_output_wait": (i32, [vp, P(P(ctypes.c_uint8)), P(ctypes.c_float)]),
        "xn_output_destroy": (i32, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(l, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = l
    return l


def _check(code: int) -> int:
    if code != XN_OK:
        raise XenodonError(code, load_library().xn_last_error().decode(errors="replace"))
    return code


def nodes_to_u64(nodes: np.ndarray) -> np.ndarray:
    """The reference's (n, 10) u32 nodes in the 64-bit node form (n, 72) u8."""
    n = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(-1, 10)
    out = np.zeros((n.shape[0], 18), np.uint32)
    out[:, 0:16:2] = n[:, :8]  # little-endian u64: low words
    out[:, 16] = n[:, 8]
    out[:, 17] = n[:, 9]
    return out.view(np.uint8).reshape(-1, 72)


def make_camera(forward, up, translation) -> Camera:
    c = Camera()
    c.forward[:] = [float(v) for v in forward]
    c.up[:] = [float(v) for v in up]
    c.translation[:] = [float(v) for v in translation]
    return c


def make_params(width, height, emission_coeff=1.0, voxel_ratio=(1.0, 1.0, 1.0), output_offset=(0, 0),
                output_extent=None, display_offset=(0, 0), display_extent=None) -> Params:
    p = Params()
    ow, oh = output_extent or (width, height)
    dw, dh = display_extent or (width, height)
    p.output_region = Rect(int(output_offset[0]), int(output_offset[1]), int(ow), int(oh))
    p.display_region = Rect(int(display_offset[0]), int(display_offset[1]), int(dw), int(dh))
    p.voxel_ratio[:] = [float(v) for v in voxel_ratio]
    p.emission_coeff = float(emission_coeff)
    return p


def _traversal(t) -> int:
    return TRAVERSALS[t] if isinstance(t, str) else int(t)


class Volume:
    """A volume resident in HBM (grid or octree)."""

    def __init__(self, ctx: "Context", handle: ctypes.c_void_p):
        self.ctx = ctx
        self.handle = handle

    def info(self) -> dict:
        vi = VolumeInfo()
        _check(load_library().xn_volume_info_get(self.handle, ctypes.byref(vi)))
        return {"kind": "grid" if vi.kind == 0 else "svo", "dim": tuple(vi.dim), "side": vi.side,
                "n_nodes": vi.n_nodes, "device_bytes": vi.device_bytes, "has_ropes": bool(vi.has_ropes)}

    def save(self, path) -> None:
        """Write an octree volume's device layout ("XNDN-SVC"; xn_volume_save)."""
        _check(load_library().xn_volume_save(self.ctx.handle, self.handle, str(path).encode()))

    def release(self) -> None:
        if self.handle:
            load_library().xn_volume_release(self.handle)
            self.handle = None

    def __del__(self):
        try:
            if self.handle and self.ctx.handle:
                self.release()
        except Exception:
            pass


class Context:
    """One CUDA device context (xn_create)."""

    def __init__(self, device: int = 0, hbm_budget: int = 0):
        self.lib = load_library()
        h = ctypes.c_void_p()
        _check(self.lib.xn_create(device, hbm_budget, ctypes.byref(h)))
        self.handle = h

    def close(self) -> None:
        if self.handle:
            self.lib.xn_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def memory(self) -> tuple[int, int]:
        used, budget = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self.lib.xn_ctx_memory(self.handle, ctypes.byref(used), ctypes.byref(budget)))
        return used.value, budget.value

    def upload_grid(self, grid: np.ndarray) -> Volume:
        """grid: uint8 (dz, dy, dx, 4), x fastest."""
        g = np.ascontiguousarray(grid, dtype=np.uint8)
        if g.ndim != 4 or g.shape[3] != 4:
            raise ValueError("grid must have shape (dz, dy, dx, 4)")
        h = ctypes.c_void_p()
        _check(self.lib.xn_volume_upload_grid(self.handle, g.ctypes.data, g.shape[2], g.shape[1], g.shape[0],
                                              ctypes.byref(h)))
        return Volume(self, h)

    def upload_grid_device(self, d_rgba: int, dims) -> Volume:
        """Grid already on the device: d_rgba points at dx*dy*dz packed RGBA8 texels; dims = (dx, dy, dz)."""
        h = ctypes.c_void_p()
        _check(self.lib.xn_volume_upload_grid_device(self.handle, d_rgba, dims[0], dims[1], dims[2], ctypes.byref(h)))
        return Volume(self, h)

    def build_svo_volume(self, d_rgba: int, dims, svo_type="rope", heuristic="chan-diff", threshold=0.0,
                         lean: bool = False):
        """Octree of a device grid, built and kept on the device.  Returns (Volume, stats).

        lean (sparse trees): write the device layout directly, without the
        reference node array or rope records (every traversal but svo-rope)."""
        h = ctypes.c_void_p()
        st = BuildStats()
        t = SVO_TYPES[svo_type] | (XN_BUILD_LEAN if lean else 0)
        _check(self.lib.xn_build_svo_volume(self.handle, d_rgba, dims[0], dims[1], dims[2], t,
                                            HEURISTICS[heuristic], float(threshold), ctypes.byref(h), ctypes.byref(st)))
        return Volume(self, h), {f: int(getattr(st, f)) for f, _ in BuildStats._fields_}

    def load_volume(self, path) -> Volume:
        """Read an "XNDN-SVC" octree volume file straight into HBM (xn_volume_load)."""
        h = ctypes.c_void_p()
        _check(self.lib.xn_volume_load(self.handle, str(path).encode(), ctypes.byref(h)))
        return Volume(self, h)

    def upload_svo(self, nodes: np.ndarray, side: int) -> Volume:
        """nodes: uint32 (n, 10) in the reference layout."""
        n = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(-1, 10)
        h = ctypes.c_void_p()
        _check(self.lib.xn_volume_upload_svo(self.handle, n.ctypes.data, n.shape[0], int(side), ctypes.byref(h)))
        return Volume(self, h)

    def upload_svo64(self, nodes64: np.ndarray, side: int) -> Volume:
        """nodes64: the 64-bit node form, a structured or uint8 array of 72-byte
        nodes (eight u64 child indices, u32 colour, u32 is_leaf_depth)."""
        raw = np.ascontiguousarray(nodes64).view(np.uint8).reshape(-1, 72)
        h = ctypes.c_void_p()
        _check(self.lib.xn_volume_upload_svo_fmt(self.handle, raw.ctypes.data, raw.shape[0], int(side), 1,
                                                 ctypes.byref(h)))
        return Volume(self, h)

    def render(self, vol: Volume, traversal, camera: Camera, params: Params, emission: bool = False,
               allow_ray_limit: bool = False, out: np.ndarray | None = None):
        """Render to host memory.  Returns (rgba (h, w, 4) u8, emission (h, w, 3) f32 or None, kernel_ms).

        `out`, when given, is a C-contiguous uint8 (h, w, 4) host array (pinned
        memory makes the copy asynchronous-capable and faster)."""
        w, h = params.output_region.width, params.output_region.height
        if out is not None:
            if out.dtype != np.uint8 or out.shape != (h, w, 4) or not out.flags["C_CONTIGUOUS"]:
                raise ValueError("out must be a C-contiguous uint8 array of shape (h, w, 4)")
            rgba = out
        else:
            rgba = np.empty((h, w, 4), np.uint8)
        em = np.empty((h, w, 3), np.float32) if emission else None
        ms = ctypes.c_float()
        r = self.lib.xn_render(self.handle, vol.handle, _traversal(traversal), ctypes.byref(camera),
                               ctypes.byref(params), rgba.ctypes.data, em.ctypes.data if em is not None else None,
                               ctypes.byref(ms))
        if not (allow_ray_limit and r == XN_ERR_RAY_LIMIT):
            _check(r)
        return rgba, em, ms.value

    def render_device(self, vol: Volume, traversal, camera: Camera, params: Params, d_rgba: int,
                      d_emission: int | None = None, d_loads: int | None = None, stream: int | None = None) -> None:
        """Launch into caller-owned device buffers (raw device pointers) on `stream`."""
        _check(self.lib.xn_render_device(self.handle, vol.handle, _traversal(traversal), ctypes.byref(camera),
                                         ctypes.byref(params), d_rgba, d_emission, d_loads, stream))

    def make_jobs(self, specs) -> ctypes.Array:
        """specs: iterable of (volume, traversal, camera, params, device pointer)."""
        specs = list(specs)
        arr = (Job * max(1, len(specs)))()
        for i, (vol, trav, cam, params, ptr) in enumerate(specs):
            arr[i] = Job(vol.handle, _traversal(trav), cam, params, ptr)
        return arr

    def render_batch(self, jobs, n: int, config: BatchConfig | None = None, stream: int | None = None) -> None:
        """One persistent launch over n jobs (see make_jobs); asynchronous on `stream`."""
        _check(self.lib.xn_render_batch(self.handle, jobs, n, ctypes.byref(config) if config else None, stream))

    def autotune_batch(self, jobs, n: int, stream: int | None = None) -> tuple[BatchConfig, float]:
        best = BatchConfig()
        ms = ctypes.c_float()
        _check(self.lib.xn_autotune_batch(self.handle, jobs, n, stream, ctypes.byref(best), ctypes.byref(ms)))
        return best, ms.value

    def batch_graph(self, capacity: int, config: BatchConfig | None = None, stream: int | None = None):
        return BatchGraph(self, capacity, config, stream)

    def ray_errors(self, reset: bool = True) -> int:
        bits = ctypes.c_uint32()
        _check(self.lib.xn_ray_errors(self.handle, ctypes.byref(bits), int(reset)))
        return bits.value

    def build_svo(self, grid: np.ndarray, svo_type="sparse", heuristic="chan-diff", threshold=0.0):
        """Build the reference octree of an RGBA8 grid on the GPU.  Returns (nodes (n, 10) u32, stats)."""
        g = np.ascontiguousarray(grid, dtype=np.uint8)
        out = ctypes.POINTER(ctypes.c_uint32)()
        st = BuildStats()
        _check(self.lib.xn_build_svo(self.handle, g.ctypes.data, g.shape[2], g.shape[1], g.shape[0],
                                     SVO_TYPES[svo_type], HEURISTICS[heuristic], float(threshold),
                                     ctypes.byref(out), ctypes.byref(st)))
        n = st.n_nodes
        try:
            arr = np.ctypeslib.as_array(out, shape=(n * 10,)).copy().reshape(n, 10) if n else np.zeros((0, 10), np.uint32)
        finally:
            self.lib.xn_free(out)
        return arr, {f: int(getattr(st, f)) for f, _ in BuildStats._fields_}

    def build_svo_streamed(self, dims, read_region, path, heuristic="chan-diff", threshold=0.0) -> dict:
        """Sparse octree of a dx*dy*dz grid built one top-level cube at a time
        and written to `path` (an XNDN-SVO file).  read_region(x0, y0, z0, nx,
        ny, nz) returns that box as a uint8 (nz, ny, nx, 4) array.  Returns the
        build stats."""
        failure = []

        def cb(_user, x0, y0, z0, nx, ny, nz, dst):
            try:
                box = np.ascontiguousarray(read_region(x0, y0, z0, nx, ny, nz), dtype=np.uint8)
                if box.shape != (nz, ny, nx, 4):
                    raise ValueError(f"read_region returned {box.shape}, wanted {(nz, ny, nx, 4)}")
                ctypes.memmove(dst, box.ctypes.data, box.nbytes)
                return 0
            except Exception as exc:  # reported after the build returns
                failure.append(exc)
                return 1

        fn = REGION_READER(cb)
        st = BuildStats()
        r = self.lib.xn_build_svo_streamed(self.handle, dims[0], dims[1], dims[2], HEURISTICS[heuristic],
                                           float(threshold), fn, None, str(path).encode(), ctypes.byref(st))
        if failure:
            raise failure[0]
        _check(r)
        return {f: int(getattr(st, f)) for f, _ in BuildStats._fields_}


class BatchGraph:
    """xn_batch_graph: a captured batch launch replayed per batch."""

    def __init__(self, ctx: Context, capacity: int, config: BatchConfig | None, stream: int | None):
        self.ctx = ctx
        h = ctypes.c_void_p()
        _check(ctx.lib.xn_batch_graph_create(ctx.handle, capacity, ctypes.byref(config) if config else None,
                                             stream, ctypes.byref(h)))
        self.handle = h

    def launch(self, jobs, n: int) -> None:
        _check(self.ctx.lib.xn_batch_graph_launch(self.handle, jobs, n))

    def close(self) -> None:
        if self.handle:
            self.ctx.lib.xn_batch_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Output:
    """xn_output: renders queued on the context's stream, each frame copied
    into pinned host memory on the output's own stream; wait() is the fence.
    Two outputs used in turn keep the GPU busy while the host takes the
    previous frame."""

    def __init__(self, ctx: "Context", max_pixels: int):
        self.ctx = ctx
        self.lib = ctx.lib
        h = ctypes.c_void_p()
        _check(self.lib.xn_output_create(ctx.handle, int(max_pixels), ctypes.byref(h)))
        self.handle = h
        self._shape = None

    def render(self, vol: "Volume", traversal: str, camera: Camera, params: Params, discard: bool = False) -> None:
        _check(self.lib.xn_output_render(self.handle, vol.handle, _traversal(traversal), ctypes.byref(camera),
                                         ctypes.byref(params), XN_OUTPUT_DISCARD if discard else 0))
        self._shape = (params.output_region.height, params.output_region.width, 4)

    def wait(self, out: np.ndarray | None = None):
        """Blocks until the queued render and copy are done; copies the frame
        into `out` (uint8, height x width x 4) when given and returns
        (image, kernel ms).  Without `out` the image is a view of the pinned
        buffer, valid until the next render into this output."""
        px = ctypes.POINTER(ctypes.c_uint8)()
        ms = ctypes.c_float()
        _check(self.lib.xn_output_wait(self.handle, ctypes.byref(px), ctypes.byref(ms)))
        h, w, c = self._shape
        view = np.ctypeslib.as_array(px, shape=(h * w * c,)).reshape(h, w, c)
        if out is not None:
            np.copyto(out, view)
            return out, ms.value
        return view, ms.value

    def close(self) -> None:
        if self.handle:
            self.lib.xn_output_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Server:
    """xn_server: continuous batching of render requests on one context."""

    def __init__(self, ctx: Context, hbm_budget: int = 0, max_batch_jobs: int = 1024, streams: int = 2,
                 fold_max_pixels: int = 0, fold_idle_us: int = 0, fold_blocks_per_sm: int = 0,
                 band_pixels: int = 0):
        """max_batch_jobs: job slots of a folding ring; streams: large frames in
        flight; frames below fold_max_pixels (0: 2^19) fold into the
        persistent kernel, which leaves after fold_idle_us (0: 300) idle;
        band_pixels: large frames in bands of rows of about that many pixels
        (0: one launch per frame)."""
        self.ctx = ctx
        self.lib = ctx.lib
        cfg = ServerConfig(hbm_budget, max_batch_jobs, streams, fold_max_pixels, fold_idle_us, fold_blocks_per_sm,
                           band_pixels)
        h = ctypes.c_void_p()
        _check(self.lib.xn_server_create(ctx.handle, ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h
        self._outputs = {}

    def add_grid(self, volume_id: int, grid: np.ndarray) -> None:
        g = np.ascontiguousarray(grid, dtype=np.uint8)
        _check(self.lib.xn_server_add_grid(self.handle, volume_id, g.ctypes.data, g.shape[2], g.shape[1], g.shape[0]))

    def add_svo(self, volume_id: int, nodes: np.ndarray, side: int) -> None:
        n = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(-1, 10)
        _check(self.lib.xn_server_add_svo(self.handle, volume_id, n.ctypes.data, n.shape[0], int(side)))

    def add_volume(self, volume_id: int, volume: "Volume") -> None:
        """A volume already resident in the context; the caller keeps owning it."""
        _check(self.lib.xn_server_add_volume(self.handle, volume_id, volume.handle))

    def submit(self, volume_id: int, traversal, camera: Camera, params: Params, out: np.ndarray | None = None) -> int:
        w, h = params.output_region.width, params.output_region.height
        if out is None:
            out = np.empty((h, w, 4), np.uint8)
        t = ctypes.c_uint64()
        _check(self.lib.xn_server_submit(self.handle, volume_id, _traversal(traversal), ctypes.byref(camera),
                                         ctypes.byref(params), out.ctypes.data, ctypes.byref(t)))
        self._outputs[t.value] = out
        return t.value

    def wait(self, ticket: int, timeout: float = -1.0):
        """Returns (rgba, latency_ms)."""
        lat = ctypes.c_double()
        try:
            _check(self.lib.xn_server_wait(self.handle, ticket, float(timeout), ctypes.byref(lat)))
        finally:
            out = self._outputs.pop(ticket, None)
        return out, lat.value

    def stats(self) -> dict:
        st = ServerStats()
        _check(self.lib.xn_server_stats(self.handle, ctypes.byref(st)))
        return st.as_dict()

    def close(self) -> None:
        if self.handle:
            self.lib.xn_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def svo_load(path) -> tuple[np.ndarray, int]:
    lib = load_library()
    out = ctypes.POINTER(ctypes.c_uint32)()
    n, side = ctypes.c_uint64(), ctypes.c_uint64()
    _check(lib.xn_svo_load(str(path).encode(), ctypes.byref(out), ctypes.byref(n), ctypes.byref(side)))
    try:
        arr = np.ctypeslib.as_array(out, shape=(n.value * 10,)).copy().reshape(-1, 10) if n.value else \
            np.zeros((0, 10), np.uint32)
    finally:
        lib.xn_free(out)
    return arr, side.value


def svo_save(path, nodes: np.ndarray, side: int) -> None:
    n = np.ascontiguousarray(nodes, dtype=np.uint32).reshape(-1, 10)
    _check(load_library().xn_svo_save(str(path).encode(), n.ctypes.data, n.shape[0], int(side)))


def tiff_load(path) -> np.ndarray:
    """Stacked TIFF -> uint8 (dz, dy, dx, 4), as the reference's Grid::load_tiff sees it."""
    lib = load_library()
    out = ctypes.POINTER(ctypes.c_uint8)()
    dims = (ctypes.c_uint32 * 3)()
    _check(lib.xn_tiff_load(str(path).encode(), ctypes.byref(out), ctypes.byref(dims)))
    try:
        n = dims[0] * dims[1] * dims[2] * 4
        arr = np.ctypeslib.as_array(out, shape=(n,)).copy().reshape(dims[2], dims[1], dims[0], 4)
    finally:
        lib.xn_free(out)
    return arr


def tiff_save(path, grid: np.ndarray) -> None:
    g = np.ascontiguousarray(grid, dtype=np.uint8)
    _check(load_library().xn_tiff_save(str(path).encode(), g.ctypes.data, g.shape[2], g.shape[1], g.shape[0]))


def png_save(path, rgba: np.ndarray) -> None:
    a = np.ascontiguousarray(rgba, dtype=np.uint8)
    _check(load_library().xn_png_save(str(path).encode(), a.ctypes.data, a.shape[1], a.shape[0]))

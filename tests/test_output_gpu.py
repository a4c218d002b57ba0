"""Asynchronous output regions (xn_output_*): renders queued into two outputs
in turn, read back through pinned memory, equal xn_render's pixels; misuse
is refused with a status."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_alternating_outputs_equal_synchronous_renders(ctx):
    import xenodon_gb300 as xg
    from xenodon_gb300 import cameras, volumes
    lib = xg.load_library()
    g = volumes.blobs(48, seed=3)
    nodes, st = ctx.build_svo(g, "rope")
    vg, vs = ctx.upload_grid(g), ctx.upload_svo(nodes, st["side"])
    w, h = 96, 64
    path = cameras.orbit(np.array([0.5, 0.5, 0.5]), 2.0, 6)
    outs = []
    for _ in range(2):
        o = ctypes.c_void_p()
        assert lib.xn_output_create(ctx.handle, w * h, ctypes.byref(o)) == 0, lib.xn_last_error()
        outs.append(o)
    try:
        for trav in xg.TRAVERSALS:
            vol = vg if trav == "dda" else vs
            params = xg.make_params(w, h, emission_coeff=10.0)
            pending = None
            for i, c in enumerate(path + [None]):
                if c is not None:
                    cam = xg.make_camera(*c)
                    r = lib.xn_output_render(outs[i % 2], vol.handle, xg.TRAVERSALS[trav], ctypes.byref(cam),
                                             ctypes.byref(params), 0)
                    assert r == 0, lib.xn_last_error()
                if pending is not None:
                    j, cam_prev = pending
                    px = ctypes.POINTER(ctypes.c_uint8)()
                    ms = ctypes.c_float()
                    r = lib.xn_output_wait(outs[j % 2], ctypes.byref(px), ctypes.byref(ms))
                    assert r == 0, lib.xn_last_error()
                    got = np.ctypeslib.as_array(px, shape=(h, w, 4)).copy()
                    want, _, _ = ctx.render(vol, trav, xg.make_camera(*cam_prev), params)
                    assert np.array_equal(got, want), (trav, j)
                    assert ms.value > 0
                pending = (i, c) if c is not None else None
    finally:
        for o in outs:
            lib.xn_output_destroy(o)
        vg.release()
        vs.release()


def test_output_misuse_is_refused(ctx):
    import xenodon_gb300 as xg
    from xenodon_gb300 import volumes
    lib = xg.load_library()
    g = volumes.blobs(16, seed=1)
    vg = ctx.upload_grid(g)
    o = ctypes.c_void_p()
    assert lib.xn_output_create(ctx.handle, 32 * 32, ctypes.byref(o)) == 0
    try:
        cam = xg.make_camera((0, 0, -1), (0, 1, 0), (0.5, 0.5, 2.5))
        px = ctypes.POINTER(ctypes.c_uint8)()
        assert lib.xn_output_wait(o, ctypes.byref(px), None) == xg.XN_ERR_STATE
        big = xg.make_params(64, 64, emission_coeff=1.0)
        assert lib.xn_output_render(o, vg.handle, 0, ctypes.byref(cam), ctypes.byref(big), 0) == xg.XN_ERR_ARG
        p = xg.make_params(32, 32, emission_coeff=1.0)
        assert lib.xn_output_render(o, vg.handle, 0, ctypes.byref(cam), ctypes.byref(p), 0) == 0
        assert lib.xn_output_render(o, vg.handle, 0, ctypes.byref(cam), ctypes.byref(p), 0) == xg.XN_ERR_STATE
        assert lib.xn_output_wait(o, ctypes.byref(px), None) == 0
        # discard: rendered and fenced, no read-back
        assert lib.xn_output_render(o, vg.handle, 0, ctypes.byref(cam), ctypes.byref(p), 1) == 0
        assert lib.xn_output_wait(o, None, None) == 0
    finally:
        lib.xn_output_destroy(o)
        vg.release()


def test_output_wrapper_pipeline_into_caller_buffers(ctx):
    """Output (the Python face of xn_output): each frame is copied on the
    output's own stream while the next frame renders; frames taken into the
    caller's buffers equal xn_render's, for every traversal."""
    import xenodon_gb300 as xg
    from xenodon_gb300 import cameras, volumes
    g = volumes.blobs(64, seed=5)
    nodes, st = ctx.build_svo(g, "rope")
    vg, vs = ctx.upload_grid(g), ctx.upload_svo(nodes, st["side"])
    w, h = 640, 360
    params = xg.make_params(w, h, emission_coeff=10.0)
    path = cameras.orbit(np.array([0.5, 0.5, 0.5]), 1.6, 4)
    jobs = [(t, c) for c in path for t in xg.TRAVERSALS]
    got = [np.empty((h, w, 4), np.uint8) for _ in jobs]
    with xg.Output(ctx, w * h) as a, xg.Output(ctx, w * h) as b:
        outs, pending = (a, b), None
        for i, (t, c) in enumerate(jobs):
            outs[i % 2].render(vg if t == "dda" else vs, t, xg.make_camera(*c), params)
            if pending is not None:
                pending[0].wait(out=got[pending[1]])
            pending = (outs[i % 2], i)
        pending[0].wait(out=got[pending[1]])
    for (t, c), img in zip(jobs, got):
        want, _, _ = ctx.render(vg if t == "dda" else vs, t, xg.make_camera(*c), params)
        assert np.array_equal(img, want), t
    vg.release()
    vs.release()

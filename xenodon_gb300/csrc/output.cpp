// Asynchronous output regions (xn_output_*): the CUDA form of the headless
// backend's per-output image, staging buffer and fence
// (src/backend/headless/HeadlessOutput.cpp:38-136).  The reference waits on
// the fence and then copies the image through a mapped staging buffer, one
// row at a time, before the next frame is recorded (HeadlessOutput.cpp:90-136,
// HeadlessDisplay.cpp:39-54).  Here a render queues the kernel on the
// context's stream and the copy into pinned host memory on the output's own
// copy stream (after an event), and returns; the wait is an event
// synchronisation.  So the next render's kernel runs while this frame is
// copied, and a caller with two outputs per region encodes frame n while
// frame n+1 renders.
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>

#include <cuda_runtime.h>

#include "../../include/xenodon.h"
#include "xn_ctx.h"
#include "xn_internal.h"

namespace xn {

int make_launch(const Volume* v, int traversal, const xn_camera* cam, const xn_params* p, RenderLaunch& L);

struct Output {
    Ctx* ctx = nullptr;
    uint64_t max_pixels = 0;
    void* d_rgba = nullptr;
    uint8_t* h_rgba = nullptr;      // pinned
    uint32_t* d_err = nullptr;      // this output's ray error bits
    uint32_t* h_err = nullptr;      // pinned copy
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, done = nullptr;
    cudaStream_t copy = nullptr;    // this output's device-to-host copies
    bool pending = false;           // a render was queued and not yet waited for
};

}  // namespace xn

using namespace xn;

XN_API int xn_output_create(xn_ctx* h, uint64_t max_pixels, xn_output** out) {
    if (!h || !out) return fail(XN_ERR_ARG, "xn_output_create: NULL argument");
    *out = nullptr;
    if (max_pixels == 0) return fail(XN_ERR_ARG, "xn_output_create: max_pixels is 0");
    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    Output* o = new (std::nothrow) Output();
    if (!o) return fail(XN_ERR_NOMEM, "xn_output_create: out of host memory");
    o->ctx = c;
    o->max_pixels = max_pixels;
    auto undo = [&](int code) {
        c->device_free(o->d_rgba, max_pixels * 4);
        c->device_free(o->d_err, 4);
        if (o->h_rgba) cudaFreeHost(o->h_rgba);
        if (o->h_err) cudaFreeHost(o->h_err);
        if (o->ev0) cudaEventDestroy(o->ev0);
        if (o->ev1) cudaEventDestroy(o->ev1);
        if (o->done) cudaEventDestroy(o->done);
        if (o->copy) cudaStreamDestroy(o->copy);
        delete o;
        return code;
    };
    if ((r = c->device_alloc(&o->d_rgba, max_pixels * 4, "xn_output_create: image"))) return undo(r);
    if ((r = c->device_alloc(reinterpret_cast<void**>(&o->d_err), 4, "xn_output_create: error word"))) return undo(r);
    cudaError_t e = cudaMallocHost(reinterpret_cast<void**>(&o->h_rgba), max_pixels * 4);
    if (e == cudaSuccess) e = cudaMallocHost(reinterpret_cast<void**>(&o->h_err), 4);
    if (e == cudaSuccess) e = cudaEventCreate(&o->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&o->ev1);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&o->done, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&o->copy, cudaStreamNonBlocking);
    if (e != cudaSuccess) return undo(cuda_fail(e, "xn_output_create"));
    *o->h_err = 0;
    *out = reinterpret_cast<xn_output*>(o);
    return XN_OK;
}

XN_API int xn_output_render(xn_output* oh, const xn_volume* vh, int traversal, const xn_camera* cam,
                            const xn_params* params, int flags) {
    if (!oh || !vh || !cam || !params) return fail(XN_ERR_ARG, "xn_output_render: NULL argument");
    Output* o = reinterpret_cast<Output*>(oh);
    Ctx* c = o->ctx;
    const Volume* v = reinterpret_cast<const Volume*>(vh);
    if (v->ctx != c) return fail(XN_ERR_ARG, "xn_output_render: volume belongs to another context");
    if (o->pending) return fail(XN_ERR_STATE, "xn_output_render: the previous render was not waited for");
    if (flags & ~XN_OUTPUT_DISCARD) return fail(XN_ERR_ARG, "xn_output_render: unknown flags 0x%x", flags);
    RenderLaunch L;
    int r = make_launch(v, traversal, cam, params, L);
    if (r) return r;
    const uint64_t npix = (uint64_t)L.out_w * L.out_h;
    if (npix > o->max_pixels)
        return fail(XN_ERR_ARG, "xn_output_render: %ux%u pixels exceed the output's %llu", L.out_w, L.out_h,
                    (unsigned long long)o->max_pixels);
    L.d_rgba = o->d_rgba;
    L.d_emission = nullptr;
    L.d_loads = nullptr;
    L.d_err_word = o->d_err;
    std::lock_guard<std::mutex> lk(c->mu);
    if ((r = c->activate())) return r;
    cudaError_t e = cudaMemsetAsync(o->d_err, 0, 4, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(o->ev0, c->stream);
    if (e == cudaSuccess) e = launch_render(L, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(o->ev1, c->stream);
    // the copies wait for the kernel on the output's stream, so the context's
    // stream is free for the next render meanwhile
    if (e == cudaSuccess) e = cudaStreamWaitEvent(o->copy, o->ev1, 0);
    if (e == cudaSuccess && !(flags & XN_OUTPUT_DISCARD))
        e = cudaMemcpyAsync(o->h_rgba, o->d_rgba, npix * 4, cudaMemcpyDeviceToHost, o->copy);
    if (e == cudaSuccess) e = cudaMemcpyAsync(o->h_err, o->d_err, 4, cudaMemcpyDeviceToHost, o->copy);
    if (e == cudaSuccess) e = cudaEventRecord(o->done, o->copy);
    if (e != cudaSuccess) return cuda_fail(e, "xn_output_render");
    o->pending = true;
    return XN_OK;
}

XN_API int xn_output_wait(xn_output* oh, const uint8_t** rgba, float* kernel_ms) {
    if (!oh) return fail(XN_ERR_ARG, "xn_output_wait: NULL argument");
    Output* o = reinterpret_cast<Output*>(oh);
    if (!o->pending) return fail(XN_ERR_STATE, "xn_output_wait: nothing was rendered into this output");
    cudaError_t e = cudaSetDevice(o->ctx->device);
    if (e == cudaSuccess) e = cudaEventSynchronize(o->done);
    o->pending = false;
    if (e != cudaSuccess) return cuda_fail(e, "xn_output_wait");
    if (kernel_ms && (e = cudaEventElapsedTime(kernel_ms, o->ev0, o->ev1)) != cudaSuccess)
        return cuda_fail(e, "xn_output_wait: event timing");
    if (rgba) *rgba = o->h_rgba;
    if (*o->h_err)
        return fail(XN_ERR_RAY_LIMIT, "xn_output_wait: a ray hit an iteration or stack limit (bits 0x%x)", *o->h_err);
    return XN_OK;
}

XN_API int xn_output_destroy(xn_output* oh) {
    if (!oh) return XN_OK;
    Output* o = reinterpret_cast<Output*>(oh);
    Ctx* c = o->ctx;
    std::lock_guard<std::mutex> lk(c->mu);
    c->activate();
    if (o->pending) cudaEventSynchronize(o->done);
    c->device_free(o->d_rgba, o->max_pixels * 4);
    c->device_free(o->d_err, 4);
    cudaFreeHost(o->h_rgba);
    cudaFreeHost(o->h_err);
    cudaEventDestroy(o->ev0);
    cudaEventDestroy(o->ev1);
    cudaEventDestroy(o->done);
    cudaStreamDestroy(o->copy);
    delete o;
    return XN_OK;
}

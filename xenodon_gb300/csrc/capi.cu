// C-ABI layer (include/xenodon.h): contexts, volumes, render entry points.
//
// Replaces the reference's per-device Vulkan plumbing
// (src/render/Renderer.cpp, src/render/DdaRaytraceAlgorithm.cpp,
// src/render/SvoRaytraceAlgorithm.cpp, src/backend/headless/HeadlessOutput.cpp)
// with one CUDA device context per xn_ctx.  No C++ exception crosses the ABI:
// every entry point catches, records a message for xn_last_error() and
// returns a status.
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "../../include/xenodon.h"
#include "xn_internal.h"

#include "xn_ctx.h"

namespace {

thread_local std::string g_last_error;

}  // namespace

namespace xn {

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? XN_ERR_NOMEM : XN_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

int Ctx::device_alloc(void** p, uint64_t bytes, const char* what) {
    *p = nullptr;
    if (bytes == 0) return XN_OK;
    uint64_t cur = used.load();
    if (budget && cur + bytes > budget)
        return fail(XN_ERR_BUDGET, "%s: %llu bytes exceed the HBM budget (%llu of %llu bytes in use)", what,
                    (unsigned long long)bytes, (unsigned long long)cur, (unsigned long long)budget);
    cudaError_t e = cudaMalloc(p, bytes);
    if (e != cudaSuccess) {
        *p = nullptr;
        return cuda_fail(e, what);
    }
    used += bytes;
    return XN_OK;
}

void Ctx::device_free(void* p, uint64_t bytes) {
    if (!p) return;
    cudaFree(p);
    used -= bytes;
}

int Ctx::ensure_buffer(DeviceBuffer& b, uint64_t bytes, const char* what) {
    if (b.bytes >= bytes) return XN_OK;
    device_free(b.ptr, b.bytes);
    b.ptr = nullptr;
    b.bytes = 0;
    int r = device_alloc(&b.ptr, bytes, what);
    if (r == XN_OK) b.bytes = bytes;
    return r;
}

void Ctx::release_extra() {
    if (batch_copied) {
        cudaEventSynchronize(batch_copied);
        cudaEventDestroy(batch_copied);
    }
    if (batch_host) cudaFreeHost(batch_host);
}

int Ctx::activate() {
    cudaError_t e = cudaSetDevice(device);
    return e == cudaSuccess ? XN_OK : cuda_fail(e, "cudaSetDevice");
}

}  // namespace xn

using namespace xn;

// ---------------------------------------------------------------- context ---

XN_API const char* xn_last_error(void) { return g_last_error.c_str(); }

XN_API int xn_abi_version(void) { return XN_ABI_VERSION; }

XN_API int xn_create(int device, uint64_t hbm_budget_bytes, xn_ctx** out) {
    if (!out) return fail(XN_ERR_ARG, "xn_create: out is NULL");
    *out = nullptr;
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess) return cuda_fail(e, "xn_create: cudaGetDeviceCount");
    if (device < 0 || device >= count) return fail(XN_ERR_ARG, "xn_create: no CUDA device %d (%d present)", device, count);
    Ctx* c = new (std::nothrow) Ctx();
    if (!c) return fail(XN_ERR_NOMEM, "xn_create: out of host memory");
    c->device = device;
    c->budget = hbm_budget_bytes;
    int r = c->activate();
    if (r) { delete c; return r; }
    if ((e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreate(&c->ev0)) != cudaSuccess || (e = cudaEventCreate(&c->ev1)) != cudaSuccess) {
        r = cuda_fail(e, "xn_create");
        xn_destroy(reinterpret_cast<xn_ctx*>(c));
        return r;
    }
    r = c->device_alloc(reinterpret_cast<void**>(&c->d_err), sizeof(uint32_t), "xn_create: error word");
    if (r) { xn_destroy(reinterpret_cast<xn_ctx*>(c)); return r; }
    cudaMemsetAsync(c->d_err, 0, sizeof(uint32_t), c->stream);
    cudaStreamSynchronize(c->stream);
    *out = reinterpret_cast<xn_ctx*>(c);
    return XN_OK;
}

XN_API int xn_destroy(xn_ctx* h) {
    if (!h) return XN_OK;
    Ctx* c = reinterpret_cast<Ctx*>(h);
    c->activate();
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->device_free(c->out_rgba.ptr, c->out_rgba.bytes);
    c->device_free(c->out_emission.ptr, c->out_emission.bytes);
    c->device_free(c->d_err, sizeof(uint32_t));
    c->release_extra();
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return XN_OK;
}

XN_API int xn_ctx_memory(const xn_ctx* h, uint64_t* used_bytes, uint64_t* budget_bytes) {
    if (!h) return fail(XN_ERR_ARG, "xn_ctx_memory: ctx is NULL");
    const Ctx* c = reinterpret_cast<const Ctx*>(h);
    if (used_bytes) *used_bytes = c->used.load();
    if (budget_bytes) *budget_bytes = c->budget;
    return XN_OK;
}

// ---------------------------------------------------------------- volumes ---

namespace {

__global__ void validate_nodes_kernel(const uint32_t* w, uint64_t n, uint32_t* bad) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t local = 0;
    for (; i < n * 8; i += stride) {
        uint64_t node = i >> 3, k = i & 7;
        if (w[node * 10 + k] >= n) local = 1;
    }
    if (local) atomicOr(bad, 1u);
}

__global__ void detect_ropes_kernel(const uint32_t* w, uint64_t n, uint32_t* any) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t local = 0;
    for (; i < n; i += stride) {
        const uint32_t* p = w + i * 10;
        if (p[9] >= 0x80000000u && (p[0] | p[1] | p[2] | p[3] | p[4] | p[5])) local = 1;
    }
    if (local) atomicOr(any, 1u);
}

}  // namespace

namespace {

__device__ __forceinline__ float unorm8_exact(uint32_t c) {
    const float r = 1.0f / 255.0f;
    float cf = __uint2float_rn(c);
    float q0 = cf * r;
    return fmaf(fmaf(-q0, 255.0f, cf), r, q0);
}

// Counts the bytes for which the texture unit's UNORM8 -> float differs from
// byte/255 correctly rounded; all 256 fetches are in range.
__global__ void tex_unorm_check_kernel(cudaTextureObject_t t, unsigned* mismatches) {
    const unsigned i = threadIdx.x;
    float4 v = tex3D<float4>(t, i + 0.5f, 0.5f, 0.5f);
    const float e = unorm8_exact(i), f = unorm8_exact(255 - i);
    unsigned bad = (v.x != e) + (v.y != f) + (v.z != e) + (v.w != f);
    if (bad) atomicAdd(mismatches, bad);
}

cudaTextureObject_t make_texture(cudaArray_t a, bool normalized) {
    cudaResourceDesc rd = {};
    rd.resType = cudaResourceTypeArray;
    rd.res.array.array = a;
    cudaTextureDesc td = {};
    td.addressMode[0] = td.addressMode[1] = td.addressMode[2] = cudaAddressModeBorder;  // border colour 0
    td.filterMode = cudaFilterModePoint;
    td.readMode = normalized ? cudaReadModeNormalizedFloat : cudaReadModeElementType;
    td.normalizedCoords = 0;
    cudaTextureObject_t t = 0;
    if (cudaCreateTextureObject(&t, &rd, &td, nullptr) != cudaSuccess) return 0;
    return t;
}

// Whether this device's texture unit returns exactly byte/255 (decided once
// per context by comparing all 256 values; otherwise the kernels convert the
// raw bytes themselves).
int texture_unorm_exact(Ctx* c) {
    if (c->tex_norm_exact >= 0) return c->tex_norm_exact;
    c->tex_norm_exact = 0;
    cudaChannelFormatDesc d = cudaCreateChannelDesc<uchar4>();
    cudaArray_t a = nullptr;
    if (cudaMalloc3DArray(&a, &d, make_cudaExtent(256, 1, 1)) != cudaSuccess) return 0;
    uchar4 h[256];
    for (int i = 0; i < 256; ++i) h[i] = make_uchar4(i, 255 - i, i, 255 - i);
    cudaMemcpy3DParms p = {};
    p.srcPtr = make_cudaPitchedPtr(h, sizeof h, 256, 1);
    p.dstArray = a;
    p.extent = make_cudaExtent(256, 1, 1);
    p.kind = cudaMemcpyHostToDevice;
    unsigned* bad = nullptr;
    cudaTextureObject_t t = 0;
    unsigned hb = 1;
    if (cudaMemcpy3DAsync(&p, c->stream) == cudaSuccess && (t = make_texture(a, true)) != 0 &&
        cudaMallocAsync(reinterpret_cast<void**>(&bad), 4, c->stream) == cudaSuccess &&
        cudaMemsetAsync(bad, 0, 4, c->stream) == cudaSuccess) {
        tex_unorm_check_kernel<<<1, 256, 0, c->stream>>>(t, bad);
        if (cudaMemcpyAsync(&hb, bad, 4, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess) hb = 1;
        if (cudaStreamSynchronize(c->stream) != cudaSuccess) hb = 1;
    }
    if (bad) cudaFreeAsync(bad, c->stream);
    cudaStreamSynchronize(c->stream);
    if (t) cudaDestroyTextureObject(t);
    cudaFreeArray(a);
    c->tex_norm_exact = hb == 0 ? 1 : 0;
    return c->tex_norm_exact;
}

}  // namespace

namespace {

int upload_grid(xn_ctx* h, const uint8_t* rgba, bool from_device, uint32_t dx, uint32_t dy, uint32_t dz,
                xn_volume** out) {
    if (!h || !rgba || !out) return fail(XN_ERR_ARG, "xn_volume_upload_grid: NULL argument");
    const cudaMemcpyKind kind = from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    *out = nullptr;
    if (!dx || !dy || !dz) return fail(XN_ERR_ARG, "xn_volume_upload_grid: empty grid %ux%ux%u", dx, dy, dz);
    if ((uint64_t)dx + dy + dz > (1ull << 30)) return fail(XN_ERR_ARG, "xn_volume_upload_grid: grid too large");
    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    Volume* v = new (std::nothrow) Volume();
    if (!v) return fail(XN_ERR_NOMEM, "xn_volume_upload_grid: out of host memory");
    v->ctx = c;
    v->kind = XN_VOLUME_GRID;
    v->dim[0] = dx;
    v->dim[1] = dy;
    v->dim[2] = dz;
    const uint64_t bytes = (uint64_t)dx * dy * dz * 4;
    // texture form unless XN_GRID_LAYOUT=linear or the device's 3D texture
    // limits are exceeded
    const char* lay = std::getenv("XN_GRID_LAYOUT");
    const bool bricked = lay && std::strcmp(lay, "bricked") == 0;
    const bool hybrid = lay && std::strcmp(lay, "hybrid") == 0;
    bool use_tex = !(lay && (std::strcmp(lay, "linear") == 0 || bricked));
    if (use_tex) {
        cudaDeviceProp prop;
        if (cudaGetDeviceProperties(&prop, c->device) != cudaSuccess || (int)dx > prop.maxTexture3D[0] ||
            (int)dy > prop.maxTexture3D[1] || (int)dz > prop.maxTexture3D[2])
            use_tex = false;
    }
    cudaError_t e = cudaSuccess;
    if (use_tex) {
        // the texture unit converts to float when it gives byte/255 exactly,
        // unless XN_TEX_READ=raw (four bytes per fetch, converted in the
        // kernel) or packed (one 32-bit word per fetch, converted in the
        // kernel)
        const char* rd = std::getenv("XN_TEX_READ");
        const bool packed = rd && std::strcmp(rd, "packed") == 0;
        const bool norm = !packed && !(rd && std::strcmp(rd, "raw") == 0) && texture_unorm_exact(c) == 1;
        if (c->budget && c->used.load() + bytes > c->budget) {
            delete v;
            return fail(XN_ERR_BUDGET, "xn_volume_upload_grid: %llu bytes exceed the HBM budget",
                        (unsigned long long)bytes);
        }
        cudaChannelFormatDesc d = packed ? cudaCreateChannelDesc<unsigned int>() : cudaCreateChannelDesc<uchar4>();
        e = cudaMalloc3DArray(&v->array, &d, make_cudaExtent(dx, dy, dz));
        if (e != cudaSuccess) {
            delete v;
            return cuda_fail(e, "xn_volume_upload_grid: array");
        }
        v->array_bytes = bytes;
        c->used += bytes;
        cudaMemcpy3DParms p = {};
        p.srcPtr = make_cudaPitchedPtr(const_cast<uint8_t*>(rgba), (size_t)dx * 4, dx, dy);
        p.dstArray = v->array;
        p.extent = make_cudaExtent(dx, dy, dz);
        p.kind = kind;
        e = cudaMemcpy3DAsync(&p, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e == cudaSuccess) {
            v->tex = make_texture(v->array, norm);
            v->tex_normalized = packed ? 2 : norm ? 1 : 0;
            if (!v->tex) e = cudaErrorInvalidValue;
        }
        if (e == cudaSuccess && hybrid && v->tex_normalized == 1) {
            // and the x-fastest copy the hybrid DDA's other warps read
            if ((r = c->device_alloc(&v->data, bytes, "xn_volume_upload_grid: linear copy"))) {
                cudaDestroyTextureObject(v->tex);
                cudaFreeArray(v->array);
                c->used -= bytes;
                delete v;
                return r;
            }
            v->bytes = bytes;
            v->hybrid = 1;
            e = cudaMemcpyAsync(v->data, rgba, bytes, kind, c->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
            if (e != cudaSuccess) {
                cudaDestroyTextureObject(v->tex);
                c->device_free(v->data, v->bytes);
            }
        }
        if (e != cudaSuccess) {
            cudaFreeArray(v->array);
            c->used -= bytes;
            delete v;
            return cuda_fail(e, "xn_volume_upload_grid: texture");
        }
        *out = reinterpret_cast<xn_volume*>(v);
        return XN_OK;
    }
    if (bricked) {
        // the x-fastest grid (the caller's device copy, or a temporary one),
        // rewritten into bricks
        if (from_device && (reinterpret_cast<uintptr_t>(rgba) & 3)) {
            delete v;
            return fail(XN_ERR_ARG, "xn_volume_upload_grid_device: the grid must be 4-byte aligned");
        }
        v->bytes = brick_grid_bytes(dx, dy, dz);
        v->bricked = 1;
        if ((r = c->device_alloc(&v->data, v->bytes, "xn_volume_upload_grid: bricks"))) {
            delete v;
            return r;
        }
        void* src = const_cast<uint8_t*>(rgba);
        if (!from_device && (r = c->device_alloc(&src, bytes, "xn_volume_upload_grid: staging"))) {
            c->device_free(v->data, v->bytes);
            delete v;
            return r;
        }
        e = cudaMemsetAsync(v->data, 0, v->bytes, c->stream);
        if (e == cudaSuccess && !from_device) e = cudaMemcpyAsync(src, rgba, bytes, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = brick_grid(static_cast<const uint32_t*>(src), dx, dy, dz, v->data, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (!from_device) c->device_free(src, bytes);
        if (e != cudaSuccess) {
            c->device_free(v->data, v->bytes);
            delete v;
            return cuda_fail(e, "xn_volume_upload_grid: bricks");
        }
        *out = reinterpret_cast<xn_volume*>(v);
        return XN_OK;
    }
    v->bytes = bytes;
    r = c->device_alloc(&v->data, v->bytes, "xn_volume_upload_grid");
    if (r) { delete v; return r; }
    e = cudaMemcpyAsync(v->data, rgba, v->bytes, kind, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) {
        c->device_free(v->data, v->bytes);
        delete v;
        return cuda_fail(e, "xn_volume_upload_grid: copy");
    }
    *out = reinterpret_cast<xn_volume*>(v);
    return XN_OK;
}

}  // namespace

XN_API int xn_volume_upload_grid(xn_ctx* h, const uint8_t* rgba, uint32_t dx, uint32_t dy, uint32_t dz,
                                 xn_volume** out) {
    return upload_grid(h, rgba, false, dx, dy, dz, out);
}

XN_API int xn_volume_upload_grid_device(xn_ctx* h, const void* d_rgba, uint32_t dx, uint32_t dy, uint32_t dz,
                                        xn_volume** out) {
    return upload_grid(h, static_cast<const uint8_t*>(d_rgba), true, dx, dy, dz, out);
}

XN_API int xn_volume_upload_svo(xn_ctx* h, const uint32_t* nodes, uint64_t n_nodes, uint64_t side, xn_volume** out) {
    if (!h || !nodes || !out) return fail(XN_ERR_ARG, "xn_volume_upload_svo: NULL argument");
    *out = nullptr;
    if (n_nodes == 0) return fail(XN_ERR_FORMAT, "xn_volume_upload_svo: octree has no nodes");
    if (n_nodes > 0xFFFFFFFFull) return fail(XN_ERR_FORMAT, "xn_volume_upload_svo: more than 2^32 nodes need the 64-bit format");
    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    Volume* v = new (std::nothrow) Volume();
    if (!v) return fail(XN_ERR_NOMEM, "xn_volume_upload_svo: out of host memory");
    v->ctx = c;
    v->kind = XN_VOLUME_SVO;
    v->side = side;
    v->n_nodes = n_nodes;
    uint64_t s = side > 0xFFFFFFFFull ? 0xFFFFFFFFull : side;
    v->dim[0] = v->dim[1] = v->dim[2] = (uint32_t)s;
    v->bytes = n_nodes * 40;
    r = c->device_alloc(&v->data, v->bytes, "xn_volume_upload_svo");
    if (r) { delete v; return r; }
    cudaError_t e = cudaMemcpyAsync(v->data, nodes, v->bytes, cudaMemcpyHostToDevice, c->stream);
    uint32_t* flags = nullptr;  // [0] = bad index, [1] = has ropes
    if (e == cudaSuccess) e = cudaMallocAsync(reinterpret_cast<void**>(&flags), 8, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, 8, c->stream);
    if (e == cudaSuccess) {
        validate_nodes_kernel<<<1024, 256, 0, c->stream>>>(static_cast<const uint32_t*>(v->data), n_nodes, flags);
        detect_ropes_kernel<<<1024, 256, 0, c->stream>>>(static_cast<const uint32_t*>(v->data), n_nodes, flags + 1);
        e = cudaGetLastError();
    }
    uint32_t hf[2] = {0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hf, flags, 8, cudaMemcpyDeviceToHost, c->stream);
    if (flags) cudaFreeAsync(flags, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess || hf[0]) {
        c->device_free(v->data, v->bytes);
        delete v;
        if (e != cudaSuccess) return cuda_fail(e, "xn_volume_upload_svo");
        return fail(XN_ERR_FORMAT, "xn_volume_upload_svo: a child index is >= the node count (%llu)",
                    (unsigned long long)n_nodes);
    }
    v->has_ropes = hf[1] != 0;
    if ((r = build_svo_layout(c, v))) {
        c->device_free(v->data, v->bytes);
        delete v;
        return r;
    }
    *out = reinterpret_cast<xn_volume*>(v);
    return XN_OK;
}

XN_API int xn_volume_release(xn_volume* h) {
    if (!h) return XN_OK;
    Volume* v = reinterpret_cast<Volume*>(h);
    Ctx* c = v->ctx;
    std::lock_guard<std::mutex> lk(c->mu);
    c->activate();
    cudaStreamSynchronize(c->stream);
    c->device_free(v->data, v->bytes);
    v->release_layout();
    if (v->tex) cudaDestroyTextureObject(v->tex);
    if (v->array) {
        cudaFreeArray(v->array);
        c->used -= v->array_bytes;
    }
    delete v;
    return XN_OK;
}

XN_API int xn_volume_info_get(const xn_volume* h, xn_volume_info* info) {
    if (!h || !info) return fail(XN_ERR_ARG, "xn_volume_info_get: NULL argument");
    const Volume* v = reinterpret_cast<const Volume*>(h);
    info->kind = v->kind;
    for (int i = 0; i < 3; ++i) info->dim[i] = v->dim[i];
    info->side = v->side;
    info->n_nodes = v->n_nodes;
    info->device_bytes = v->bytes + v->array_bytes + (v->layout == XN_LAYOUT_COMPACT ? v->layout_bytes() : 0);
    info->has_ropes = v->has_ropes;
    return XN_OK;
}

// ----------------------------------------------------------------- render ---

namespace xn {

int make_launch(const Volume* v, int traversal, const xn_camera* cam, const xn_params* p, RenderLaunch& L) {
    if (traversal < XN_DDA || traversal > XN_SVO_ROPE) return fail(XN_ERR_ARG, "invalid traversal %d", traversal);
    if (traversal == XN_DDA && v->kind != XN_VOLUME_GRID)
        return fail(XN_ERR_ARG, "traversal 'dda' requires a grid volume (tiff)");
    if (traversal != XN_DDA && v->kind != XN_VOLUME_SVO)
        return fail(XN_ERR_ARG, "octree traversals require an octree volume (svo)");
    if (p->output_region.width == 0 || p->output_region.height == 0)
        return fail(XN_ERR_ARG, "empty output region");
    if (p->display_region.width == 0 || p->display_region.height == 0)
        return fail(XN_ERR_ARG, "empty display region");
    for (int i = 0; i < 3; ++i)
        if (!(p->voxel_ratio[i] > 0.0f)) return fail(XN_ERR_ARG, "voxel ratio components must be > 0");
    if (!(p->emission_coeff >= 0.0f)) return fail(XN_ERR_ARG, "emission coefficient must be >= 0");
    std::memset(&L, 0, sizeof L);
    L.traversal = traversal;
    for (int i = 0; i < 3; ++i) {
        L.forward[i] = cam->forward[i];
        L.up[i] = cam->up[i];
        L.voxel_ratio[i] = p->voxel_ratio[i];
        // src/render/Renderer.cpp:62: translation pre-divided by the voxel ratio
        L.translation[i] = cam->translation[i] / p->voxel_ratio[i];
    }
    L.aspect = (float)p->display_region.height / (float)p->display_region.width;
    L.emission_coeff = p->emission_coeff;
    L.out_x = p->output_region.x;
    L.out_y = p->output_region.y;
    L.out_w = p->output_region.width;
    L.out_h = p->output_region.height;
    L.disp_x = p->display_region.x;
    L.disp_y = p->display_region.y;
    L.disp_w = p->display_region.width;
    L.disp_h = p->display_region.height;
    if (v->kind == XN_VOLUME_GRID) {
        L.grid = v->data;
        L.tex = v->tex;
        L.tex_normalized = v->tex_normalized;
        L.grid_bricked = v->bricked;
        L.grid_hybrid = v->hybrid;
    } else {
        L.nodes = v->data;
        L.layout = v->layout;
        L.inner = v->inner;
        L.rinner = v->rinner;
        L.inner_depth = v->inner_depth;
        L.leaves = v->leaves;
        L.depth_consistent = v->depth_consistent;
        if (traversal == XN_TRAV_SVO_ROPE && v->layout == XN_LAYOUT_COMPACT && !v->rinner)
            return fail(XN_ERR_ARG, "svo-rope: the octree was built lean, without rope records");
        // traversal stacks: esvo's in shared memory, svo-df's in local memory
        // (measured fastest); XN_STACKS=local / shared puts both in one place
        const char* es = std::getenv("XN_STACKS");
        const bool all_local = es && std::strcmp(es, "local") == 0;
        const bool all_shared = es && std::strcmp(es, "shared") == 0;
        L.shared_stacks = all_local ? 0 : (all_shared || traversal == XN_TRAV_ESVO) ? 1 : 0;
        // svo-naive's find resumes from the last path unless XN_NAIVE_FIND=root
        const char* nf = std::getenv("XN_NAIVE_FIND");
        L.naive_resume = !(nf && std::strcmp(nf, "root") == 0);
        // masked svo-df walked by the whole warp unless XN_DF_PACKET=0
        const char* pk = std::getenv("XN_DF_PACKET");
        L.df_packet = !(pk && pk[0] == '0');
        // the nodes just above the deepest internal nodes are walked by each
        // lane alone (render.cu, lane_walk), unless XN_DF_LANE_WALK=0
        const char* lw = std::getenv("XN_DF_LANE_WALK");
        const uint32_t dmax = v->max_inner_depth;
        // two levels (from the nodes two above the deepest internal ones)
        // unless the tree is shallower or XN_DF_LANE_LEVELS=1
        const char* ll = std::getenv("XN_DF_LANE_LEVELS");
        L.df_lane_levels = (ll && ll[0] == '1') || dmax < 2u ? 1 : 2;
        L.df_lane_side = (lw && lw[0] == '0') || !v->depth_consistent || dmax < 1u || dmax > 120u
                             ? 0.0f
                             : std::ldexp(1.0f, -(int)dmax + (L.df_lane_levels - 1));
    }
    for (int i = 0; i < 3; ++i) L.dim[i] = v->dim[i];
    return XN_OK;
}

}  // namespace xn

XN_API int xn_render_device(xn_ctx* h, const xn_volume* vh, int traversal, const xn_camera* cam,
                            const xn_params* params, void* d_rgba, float* d_emission, uint32_t* d_loads,
                            void* stream) {
    if (!h || !vh || !cam || !params || !d_rgba) return fail(XN_ERR_ARG, "xn_render_device: NULL argument");
    Ctx* c = reinterpret_cast<Ctx*>(h);
    const Volume* v = reinterpret_cast<const Volume*>(vh);
    if (v->ctx != c) return fail(XN_ERR_ARG, "xn_render_device: volume belongs to another context");
    RenderLaunch L;
    int r = make_launch(v, traversal, cam, params, L);
    if (r) return r;
    L.d_rgba = d_rgba;
    L.d_emission = d_emission;
    L.d_loads = d_loads;
    L.d_err_word = c->d_err;
    r = c->activate();
    if (r) return r;
    cudaError_t e = launch_render(L, static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? XN_OK : cuda_fail(e, "xn_render_device: launch");
}

XN_API int xn_render(xn_ctx* h, const xn_volume* vh, int traversal, const xn_camera* cam, const xn_params* params,
                     uint8_t* out_rgba, float* out_emission, float* kernel_ms) {
    if (!h || !vh || !cam || !params) return fail(XN_ERR_ARG, "xn_render: NULL argument");
    Ctx* c = reinterpret_cast<Ctx*>(h);
    const Volume* v = reinterpret_cast<const Volume*>(vh);
    if (v->ctx != c) return fail(XN_ERR_ARG, "xn_render: volume belongs to another context");
    RenderLaunch L;
    int r = make_launch(v, traversal, cam, params, L);
    if (r) return r;
    std::lock_guard<std::mutex> lk(c->mu);
    if ((r = c->activate())) return r;
    const uint64_t npix = (uint64_t)L.out_w * L.out_h;
    if ((r = c->ensure_buffer(c->out_rgba, npix * 4, "xn_render: output image"))) return r;
    if (out_emission && (r = c->ensure_buffer(c->out_emission, npix * 12, "xn_render: emission buffer"))) return r;
    L.d_rgba = c->out_rgba.ptr;
    L.d_emission = out_emission ? static_cast<float*>(c->out_emission.ptr) : nullptr;
    L.d_loads = nullptr;
    L.d_err_word = c->d_err;
    cudaError_t e = cudaMemsetAsync(c->d_err, 0, sizeof(uint32_t), c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev0, c->stream);
    if (e == cudaSuccess) e = launch_render(L, c->stream);
    if (e == cudaSuccess) e = cudaEventRecord(c->ev1, c->stream);
    if (e == cudaSuccess && out_rgba)
        e = cudaMemcpyAsync(out_rgba, c->out_rgba.ptr, npix * 4, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && out_emission)
        e = cudaMemcpyAsync(out_emission, c->out_emission.ptr, npix * 12, cudaMemcpyDeviceToHost, c->stream);
    uint32_t err_bits = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&err_bits, c->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "xn_render");
    if (kernel_ms) {
        e = cudaEventElapsedTime(kernel_ms, c->ev0, c->ev1);
        if (e != cudaSuccess) return cuda_fail(e, "xn_render: event timing");
    }
    if (err_bits) return fail(XN_ERR_RAY_LIMIT, "xn_render: a ray hit an iteration or stack limit (bits 0x%x)", err_bits);
    return XN_OK;
}

XN_API int xn_ray_errors(xn_ctx* h, uint32_t* bits, int reset) {
    if (!h || !bits) return fail(XN_ERR_ARG, "xn_ray_errors: NULL argument");
    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    cudaError_t e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(bits, c->d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && reset) e = cudaMemset(c->d_err, 0, sizeof(uint32_t));
    return e == cudaSuccess ? XN_OK : cuda_fail(e, "xn_ray_errors");
}

XN_API void xn_free(void* p) { std::free(p); }

// Octree upload from 64-bit node arrays (xn_volume_upload_svo_fmt with
// XN_NODES_U64): the reference's node (src/model/Octree.h:35-45,
// resources/octree.glsl:6-10) with its eight child indices widened to u64, so
// trees of 2^32 nodes or more -- past the reference format's 32-bit indices
// (src/model/OctreeConstruction.h:74-76, README.md:91-96) -- can be handed
// over.  At 72 bytes a node such an array is larger than HBM, so it is never
// held on the device: it streams through a chunk buffer twice and only the
// device layout (svo_layout.cu: 36 bytes per internal node) stays.
//
//   pass 1, per chunk: every node's descriptor word -- an internal node's rank
//           among the internal nodes (a prefix count carried across chunks), a
//           leaf's bit 31 | RGB -- and a range check of internal nodes' child
//           indices;
//   pass 2, per chunk: internal node of rank j writes inner[8j + k] = the
//           descriptor of child k, and inner_depth[j] its is_leaf_depth.
//
// That is the layout build_svo_layout makes from 32-bit nodes (without the
// rope records: ropes of a 64-bit array are not converted, so svo-rope is
// refused on such a volume, as on lean builds).
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>

#include "../../include/xenodon.h"
#include "xn_ctx.h"
#include "xn_internal.h"
#include "xn_scan.cuh"

namespace xn {
namespace {

constexpr uint32_t LEAF = 0x80000000u;

struct Node64 {  // 72 bytes, little-endian
    unsigned long long child[8];
    uint32_t color;
    uint32_t is_leaf_depth;
};
static_assert(sizeof(Node64) == 72, "64-bit node layout");

__global__ void flags64_kernel(const Node64* nodes, uint64_t n, uint8_t* internal) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        internal[i] = nodes[i].is_leaf_depth < LEAF ? 1 : 0;
}

// Descriptor words of one chunk; flags[0] |= 1 for a child index >= total.
__global__ void describe64_kernel(const Node64* nodes, uint64_t n, uint64_t total, const unsigned* local_rank,
                                  uint64_t rank_base, uint32_t* desc, uint32_t* flags) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t bad = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const Node64& p = nodes[i];
        if (p.is_leaf_depth < LEAF) {
            desc[i] = (uint32_t)(rank_base + local_rank[i]);
            for (int k = 0; k < 8; ++k)
                if (p.child[k] >= total) bad = 1;
        } else {
            desc[i] = LEAF | (p.color & 0xFFFFFFu);
        }
    }
    if (bad) atomicOr(flags, 1u);
}

__global__ void inner64_kernel(const Node64* nodes, uint64_t n, const uint32_t* chunk_desc, const uint32_t* desc,
                               uint32_t* inner, uint32_t* inner_depth) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const Node64& p = nodes[i];
        if (p.is_leaf_depth >= LEAF) continue;
        const uint64_t j = chunk_desc[i];
        uint32_t c[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) c[k] = __ldg(desc + p.child[k]);
        uint4* out = reinterpret_cast<uint4*>(inner + j * 8);
        out[0] = make_uint4(c[0], c[1], c[2], c[3]);
        out[1] = make_uint4(c[4], c[5], c[6], c[7]);
        inner_depth[j] = p.is_leaf_depth;
    }
}

uint64_t chunk_nodes() {
    const char* e = std::getenv("XN_UPLOAD_CHUNK_NODES");
    uint64_t c = e ? std::strtoull(e, nullptr, 10) : 0;
    const uint64_t max_chunk = scan::SCAN_CHUNK * scan::SCAN_CHUNK;  // two scan levels
    if (c == 0 || c > max_chunk) c = 1ull << 22;
    return c;
}

int upload_u64(Ctx* c, const Node64* host, uint64_t n, uint64_t side, Volume** out) {
    cudaStream_t s = c->stream;
    Volume* v = new (std::nothrow) Volume();
    if (!v) return fail(XN_ERR_NOMEM, "xn_volume_upload_svo_fmt: out of host memory");
    v->ctx = c;
    v->kind = XN_VOLUME_SVO;
    v->side = side;
    v->n_nodes = n;
    const uint64_t sd = side > 0xFFFFFFFFull ? 0xFFFFFFFFull : side;
    v->dim[0] = v->dim[1] = v->dim[2] = (uint32_t)sd;
    v->has_ropes = 0;
    if (host[0].is_leaf_depth >= LEAF) {  // a leaf root: the one-node reference layout
        const uint32_t node[10] = {0, 0, 0, 0, 0, 0, 0, 0, host[0].color, host[0].is_leaf_depth};
        v->layout = XN_LAYOUT_REFERENCE;
        v->bytes = 40;
        int r = c->device_alloc(&v->data, 40, "xn_volume_upload_svo_fmt");
        cudaError_t e = r ? cudaSuccess : cudaMemcpyAsync(v->data, node, 40, cudaMemcpyHostToDevice, s);
        if (!r && e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (r || e != cudaSuccess) {
            c->device_free(v->data, v->bytes);
            delete v;
            return r ? r : cuda_fail(e, "xn_volume_upload_svo_fmt");
        }
        *out = v;
        return XN_OK;
    }
    const uint64_t C = chunk_nodes();
    const uint64_t nb = (C + scan::SCAN_CHUNK - 1) / scan::SCAN_CHUNK;
    struct Bufs {
        Ctx* c;
        Node64* chunk = nullptr;
        uint8_t* flags = nullptr;
        unsigned* rank = nullptr;
        unsigned* sums = nullptr;
        unsigned* offs = nullptr;
        uint32_t* desc = nullptr;
        uint32_t* err = nullptr;
        uint64_t C = 0, nb = 0, n = 0;
        ~Bufs() {
            cudaStreamSynchronize(c->stream);
            c->device_free(chunk, C * sizeof(Node64));
            c->device_free(flags, C);
            c->device_free(rank, C * 4);
            c->device_free(sums, nb * 4);
            c->device_free(offs, nb * 4);
            c->device_free(desc, n * 4);
            c->device_free(err, 4);
        }
    } b{c};
    b.C = C;
    b.nb = nb;
    b.n = n;
    auto drop = [&](int code) {
        cudaStreamSynchronize(s);
        v->release_layout();
        delete v;
        return code;
    };
    int r;
    if ((r = c->device_alloc(reinterpret_cast<void**>(&b.chunk), C * sizeof(Node64), "xn_volume_upload_svo_fmt: chunk")) ||
        (r = c->device_alloc(reinterpret_cast<void**>(&b.flags), C, "xn_volume_upload_svo_fmt: flags")) ||
        (r = c->device_alloc(reinterpret_cast<void**>(&b.rank), C * 4, "xn_volume_upload_svo_fmt: ranks")) ||
        (r = c->device_alloc(reinterpret_cast<void**>(&b.sums), nb * 4, "xn_volume_upload_svo_fmt: scan")) ||
        (r = c->device_alloc(reinterpret_cast<void**>(&b.offs), nb * 4, "xn_volume_upload_svo_fmt: scan")) ||
        (r = c->device_alloc(reinterpret_cast<void**>(&b.desc), n * 4, "xn_volume_upload_svo_fmt: descriptors")) ||
        (r = c->device_alloc(reinterpret_cast<void**>(&b.err), 4, "xn_volume_upload_svo_fmt: flags")))
        return drop(r);
    cudaError_t e = cudaMemsetAsync(b.err, 0, 4, s);
    // pass 1: ranks and descriptors
    uint64_t n_inner = 0;
    for (uint64_t off = 0; off < n && e == cudaSuccess; off += C) {
        const uint64_t m = n - off < C ? n - off : C;
        const uint64_t mb = (m + scan::SCAN_CHUNK - 1) / scan::SCAN_CHUNK;
        e = cudaMemcpyAsync(b.chunk, host + off, m * sizeof(Node64), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) break;
        flags64_kernel<<<1024, 256, 0, s>>>(b.chunk, m, b.flags);
        scan::scan_reduce_kernel<uint8_t><<<(unsigned)mb, scan::SCAN_T, 0, s>>>(b.flags, m, b.sums);
        scan::scan_apply_kernel<unsigned><<<1, scan::SCAN_T, 0, s>>>(b.sums, mb, nullptr, b.offs);
        scan::scan_apply_kernel<uint8_t><<<(unsigned)mb, scan::SCAN_T, 0, s>>>(b.flags, m, b.offs, b.rank);
        describe64_kernel<<<1024, 256, 0, s>>>(b.chunk, m, n, b.rank, n_inner, b.desc + off, b.err);
        unsigned last_rank = 0;
        uint8_t last_flag = 0;
        uint32_t bad = 0;
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaMemcpyAsync(&last_rank, b.rank + (m - 1), 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&last_flag, b.flags + (m - 1), 1, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, b.err, 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) break;
        if (bad)
            return drop(fail(XN_ERR_FORMAT, "xn_volume_upload_svo_fmt: a child index is >= the node count (%llu)",
                             (unsigned long long)n));
        n_inner += (uint64_t)last_rank + last_flag;
        if (n_inner >= LEAF)
            return drop(fail(XN_ERR_FORMAT, "xn_volume_upload_svo_fmt: more than 2^31 internal nodes"));
    }
    if (e != cudaSuccess) return drop(cuda_fail(e, "xn_volume_upload_svo_fmt: first pass"));
    v->n_inner = n_inner;
    v->n_leaves = 0;
    if ((r = c->device_alloc(reinterpret_cast<void**>(&v->inner), n_inner * 32, "xn_volume_upload_svo_fmt: inner")) ||
        (r = c->device_alloc(reinterpret_cast<void**>(&v->inner_depth), n_inner * 4,
                             "xn_volume_upload_svo_fmt: depths")))
        return drop(r);
    // pass 2: the internal nodes' child words
    for (uint64_t off = 0; off < n && e == cudaSuccess; off += C) {
        const uint64_t m = n - off < C ? n - off : C;
        e = cudaMemcpyAsync(b.chunk, host + off, m * sizeof(Node64), cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) break;
        inner64_kernel<<<2048, 256, 0, s>>>(b.chunk, m, b.desc + off, b.desc, v->inner, v->inner_depth);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return drop(cuda_fail(e, "xn_volume_upload_svo_fmt: second pass"));
    if ((r = validate_compact_layout(c, v, "xn_volume_upload_svo_fmt"))) return drop(r);
    v->layout = XN_LAYOUT_COMPACT;
    if ((r = measure_inner_depth(c, v))) return drop(r);
    *out = v;
    return XN_OK;
}

}  // namespace
}  // namespace xn

using namespace xn;

XN_API int xn_volume_upload_svo_fmt(xn_ctx* h, const void* nodes, uint64_t n_nodes, uint64_t side, int node_fmt,
                                    xn_volume** out) {
    if (node_fmt == XN_NODES_U32) return xn_volume_upload_svo(h, static_cast<const uint32_t*>(nodes), n_nodes, side, out);
    if (!h || !nodes || !out) return fail(XN_ERR_ARG, "xn_volume_upload_svo_fmt: NULL argument");
    *out = nullptr;
    if (node_fmt != XN_NODES_U64) return fail(XN_ERR_ARG, "xn_volume_upload_svo_fmt: invalid node format %d", node_fmt);
    if (n_nodes == 0) return fail(XN_ERR_FORMAT, "xn_volume_upload_svo_fmt: octree has no nodes");
    if (reinterpret_cast<uintptr_t>(nodes) & 7) return fail(XN_ERR_ARG, "xn_volume_upload_svo_fmt: nodes must be 8-byte aligned");
    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    Volume* v = nullptr;
    if ((r = upload_u64(c, static_cast<const Node64*>(nodes), n_nodes, side, &v))) return r;
    *out = reinterpret_cast<xn_volume*>(v);
    return XN_OK;
}

// Device layout of an uploaded octree.
//
// The reference keeps 40-byte nodes (resources/octree.glsl:6-10) and every
// traversal step reads a child index from the parent and then the child's
// is_leaf_depth (and colour) from the child: two dependent loads per visited
// child.  Here the reference nodes are converted once, on upload, into
//
//   inner[8*j + k]   child word k of internal node j (one 32-byte sector);
//                    bit 31 set: the child is a leaf, bits 0..23 its RGB
//                    (the shaders read only .rgb of a leaf colour);
//                    bit 31 clear: the index of the internal child
//   inner_depth[j]   is_leaf_depth of internal node j (read by svo-df when it
//                    pops a node, and by svo-rope for rope targets)
//   rinner[8*j + k]  the same children for svo-rope, where a leaf child word
//                    holds bit 31 | the leaf's record index
//   leaves[8*l ...]  per leaf: colour, the six rope words (as rinner words;
//                    a rope to node 0, the reference's "no neighbour", becomes
//                    ROPE_EXIT), and its is_leaf_depth
//
// so a visited child costs one load.  Depth fields are copied, not recomputed,
// so the traversals read exactly the values the reference shaders would.  A
// tree whose root is a leaf keeps the reference layout (the shaders then read
// the leaf's own child words).
#include <cstdint>

#include "../../include/xenodon.h"
#include "xn_ctx.h"
#include "xn_internal.h"
#include "xn_scan.cuh"
#include <type_traits>

namespace xn {
namespace {

constexpr uint32_t LEAF = 0x80000000u;

__global__ void internal_flags_kernel(const uint32_t* w, uint64_t n, uint8_t* internal) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        internal[i] = w[i * 10 + 9] < LEAF ? 1 : 0;
}

struct LayoutArgs {
    const uint32_t* w;       // reference nodes
    uint64_t n;
    const unsigned* rank;    // internal nodes before node i (exclusive scan)
    uint32_t* inner;
    uint32_t* rinner;
    uint32_t* inner_depth;
    uint32_t* leaves;
};

__device__ __forceinline__ bool is_leaf_node(const LayoutArgs& a, uint64_t i) { return a.w[i * 10 + 9] >= LEAF; }
__device__ __forceinline__ uint32_t leaf_index(const LayoutArgs& a, uint64_t i) { return (uint32_t)(i - a.rank[i]); }

__global__ void layout_kernel(LayoutArgs a) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < a.n; i += stride) {
        const uint32_t* node = a.w + i * 10;
        if (node[9] < LEAF) {
            const uint64_t j = a.rank[i];
            uint32_t c[8], r[8];
#pragma unroll
            for (int k = 0; k < 8; ++k) {
                const uint32_t ch = node[k];
                if (is_leaf_node(a, ch)) {
                    c[k] = LEAF | (a.w[(uint64_t)ch * 10 + 8] & 0xFFFFFFu);
                    r[k] = LEAF | leaf_index(a, ch);
                } else {
                    c[k] = a.rank[ch];
                    r[k] = a.rank[ch];
                }
            }
            uint4* pc = reinterpret_cast<uint4*>(a.inner + j * 8);
            pc[0] = make_uint4(c[0], c[1], c[2], c[3]);
            pc[1] = make_uint4(c[4], c[5], c[6], c[7]);
            uint4* pr = reinterpret_cast<uint4*>(a.rinner + j * 8);
            pr[0] = make_uint4(r[0], r[1], r[2], r[3]);
            pr[1] = make_uint4(r[4], r[5], r[6], r[7]);
            a.inner_depth[j] = node[9];
        } else {
            const uint64_t l = leaf_index(a, i);
            uint32_t rope[6];
#pragma unroll
            for (int k = 0; k < 6; ++k) {
                const uint32_t t = node[k];
                rope[k] = t == 0 ? ROPE_EXIT : (is_leaf_node(a, t) ? (LEAF | leaf_index(a, t)) : a.rank[t]);
            }
            uint4* p = reinterpret_cast<uint4*>(a.leaves + l * 8);
            p[0] = make_uint4(node[8], rope[0], rope[1], rope[2]);
            p[1] = make_uint4(rope[3], rope[4], rope[5], node[9]);
        }
    }
}

// Flags an internal node whose internal child's depth field is not its own
// plus one (svo-df's masked form relies on depth fields matching the tree).
__global__ void depth_check_kernel(const uint32_t* w, uint64_t n, uint32_t* bad) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t local = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t d = w[i * 10 + 9];
        if (d >= LEAF) continue;
        if (i == 0 && d != 0) local = 1;
        for (int k = 0; k < 8; ++k) {
            const uint32_t cd = w[(uint64_t)w[i * 10 + k] * 10 + 9];
            if (cd < LEAF && cd != d + 1) local = 1;
        }
    }
    if (local) atomicOr(bad, 1u);
}

// The largest depth field of the internal nodes.
__global__ void max_inner_depth_kernel(const uint32_t* depth, uint64_t n, uint32_t* out) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t m = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        m = max(m, depth[i] & 0x7FFFFFFFu);
    m = __reduce_max_sync(0xFFFFFFFFu, m);
    if ((threadIdx.x & 31u) == 0) atomicMax(out, m);
}

}  // namespace

int measure_inner_depth(Ctx* c, Volume* v) {
    v->max_inner_depth = 0xFFFFFFFFu;
    if (!v->depth_consistent || !v->inner_depth || v->n_inner == 0) return XN_OK;
    uint32_t* d = nullptr;
    uint32_t h = 0xFFFFFFFFu;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&d), 4, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(d, 0, 4, c->stream);
    if (e == cudaSuccess) {
        max_inner_depth_kernel<<<1024, 256, 0, c->stream>>>(v->inner_depth, v->n_inner, d);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, 4, cudaMemcpyDeviceToHost, c->stream);
    if (d) cudaFreeAsync(d, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, "octree depth");
    v->max_inner_depth = h;
    return XN_OK;
}

int build_svo_layout(Ctx* c, Volume* v) {
    const uint64_t n = v->n_nodes;
    cudaStream_t s = c->stream;
    const uint32_t* w = static_cast<const uint32_t*>(v->data);
    uint32_t root_word = 0;
    cudaError_t e = cudaMemcpyAsync(&root_word, w + 9, 4, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e, "octree layout");
    if (root_word >= LEAF) {  // a leaf root: keep the reference layout
        v->layout = XN_LAYOUT_REFERENCE;
        return XN_OK;
    }
    uint8_t* internal = nullptr;
    unsigned* rank = nullptr;
    int r;
    if ((r = c->device_alloc(reinterpret_cast<void**>(&internal), n, "octree layout: flags"))) return r;
    if ((r = c->device_alloc(reinterpret_cast<void**>(&rank), n * 4, "octree layout: ranks"))) {
        c->device_free(internal, n);
        return r;
    }
    // exclusive scan over the internal flags (recursive over block sums)
    struct Tmp {
        Ctx* c;
        void* p[8] = {};
        uint64_t b[8] = {};
        int k = 0;
        ~Tmp() {
            for (int i = 0; i < k; ++i) c->device_free(p[i], b[i]);
        }
    } tmp{c};
    auto scan_level = [&](auto&& self, auto* in, uint64_t count, unsigned* out) -> int {
        using In = std::remove_pointer_t<decltype(in)>;
        const uint64_t nb = (count + scan::SCAN_CHUNK - 1) / scan::SCAN_CHUNK;
        if (nb <= 1) {
            scan::scan_apply_kernel<In><<<1, scan::SCAN_T, 0, s>>>(in, count, nullptr, out);
            return XN_OK;
        }
        if (tmp.k + 2 > 8) return fail(XN_ERR_ARG, "octree layout: too many nodes");
        unsigned* sums = nullptr;
        unsigned* offs = nullptr;
        int rr = c->device_alloc(reinterpret_cast<void**>(&sums), nb * 4, "octree layout: scan");
        if (rr) return rr;
        tmp.p[tmp.k] = sums;
        tmp.b[tmp.k++] = nb * 4;
        if ((rr = c->device_alloc(reinterpret_cast<void**>(&offs), nb * 4, "octree layout: scan"))) return rr;
        tmp.p[tmp.k] = offs;
        tmp.b[tmp.k++] = nb * 4;
        scan::scan_reduce_kernel<In><<<(unsigned)nb, scan::SCAN_T, 0, s>>>(in, count, sums);
        if ((rr = self(self, sums, nb, offs))) return rr;
        scan::scan_apply_kernel<In><<<(unsigned)nb, scan::SCAN_T, 0, s>>>(in, count, offs, out);
        return XN_OK;
    };
    internal_flags_kernel<<<1024, 256, 0, s>>>(w, n, internal);
    r = scan_level(scan_level, internal, n, rank);
    unsigned last_rank = 0;
    uint8_t last_flag = 0;
    if (!r) {
        e = cudaMemcpyAsync(&last_rank, rank + (n - 1), 4, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&last_flag, internal + (n - 1), 1, cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) r = cuda_fail(e, "octree layout: ranks");
    }
    const uint64_t n_inner = (uint64_t)last_rank + last_flag;
    const uint64_t n_leaves = n - n_inner;
    if (!r && (n_inner >= LEAF || n_leaves >= ROPE_EXIT - LEAF))
        r = fail(XN_ERR_FORMAT, "octree layout: more than 2^31 internal nodes or leaves");
    if (!r) {
        v->n_inner = n_inner;
        v->n_leaves = n_leaves;
    }
    if (!r) r = c->device_alloc(reinterpret_cast<void**>(&v->inner), n_inner * 32, "octree layout: inner");
    if (!r) r = c->device_alloc(reinterpret_cast<void**>(&v->rinner), n_inner * 32, "octree layout: rope inner");
    if (!r) r = c->device_alloc(reinterpret_cast<void**>(&v->inner_depth), n_inner * 4, "octree layout: depths");
    if (!r) r = c->device_alloc(reinterpret_cast<void**>(&v->leaves), n_leaves * 32, "octree layout: leaves");
    if (!r) {
        LayoutArgs a{w, n, rank, v->inner, v->rinner, v->inner_depth, v->leaves};
        layout_kernel<<<2048, 256, 0, s>>>(a);
        uint32_t* bad = reinterpret_cast<uint32_t*>(internal);  // the flags are no longer needed
        uint32_t hbad = 1;
        e = cudaMemsetAsync(bad, 0, 4, s);
        if (e == cudaSuccess) {
            depth_check_kernel<<<1024, 256, 0, s>>>(w, n, bad);
            e = cudaMemcpyAsync(&hbad, bad, 4, cudaMemcpyDeviceToHost, s);
        }
        if (e == cudaSuccess) e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) r = cuda_fail(e, "octree layout");
        v->depth_consistent = hbad == 0;
    }
    c->device_free(internal, n);
    c->device_free(rank, n * 4);
    if (r) {
        v->release_layout();
        return r;
    }
    v->layout = XN_LAYOUT_COMPACT;
    if ((r = measure_inner_depth(c, v))) {
        v->release_layout();
        return r;
    }
    // the reference nodes are no longer needed on the device
    c->device_free(v->data, v->bytes);
    v->data = nullptr;
    v->bytes = 0;
    return XN_OK;
}

}  // namespace xn

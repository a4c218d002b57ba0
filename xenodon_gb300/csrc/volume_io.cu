// Device-layout octree files ("XNDN-SVC"): the resident form of an octree
// volume (svo_layout.cu) written to disk and read back without passing
// through the reference's 40-byte node array.
//
// The reference's format (src/model/Octree.cpp:21,50-114; xn_svo_load/save)
// indexes nodes with 32-bit words, so it cannot hold trees of 2^32 nodes or
// more, and at 40 bytes per node such trees (a 2048^3 gas field has about
// 8e9) exceed both HBM and host memory.  The device layout stores internal
// nodes only (leaf colours sit in their parents' child words): 36 bytes per
// internal node, about 4.5 bytes per tree node.  The file holds exactly those
// arrays, little-endian:
//
//   0  "XNDN-SVC"
//   8  u32 version (1)
//  12  u32 flags: 1 = rope records follow, 2 = the tree was a rope tree
//  16  u64 side
//  24  u64 node count of the reference tree (reported, not used)
//  32  u64 internal nodes n_inner
//  40  u64 leaf records n_leaves (0 without rope records)
//  48  u32 root colour, u32 root is_leaf_depth (used when n_inner == 0: the
//      root is a leaf)
//  56  u64 reserved (0)
//  64  inner: n_inner x 8 u32; inner_depth: n_inner x u32;
//      with rope records: rinner: n_inner x 8 u32; leaves: n_leaves x 8 u32
//
// The size must match the header exactly (as Octree::load_svo requires).
// Arrays move between HBM and the file in chunks through two pinned buffers,
// so a copy overlaps the file I/O of the previous chunk and no host copy of
// the whole tree exists.  Loaded arrays are validated on the device (every
// index in range) before any traversal can read them; the depth-consistency
// property that selects the masked svo-df is recomputed, not trusted.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <new>

#include "../../include/xenodon.h"
#include "xn_ctx.h"
#include "xn_internal.h"

#if !defined(__BYTE_ORDER__) || __BYTE_ORDER__ != __ORDER_LITTLE_ENDIAN__
#error "volume files are written from little-endian host memory"
#endif

namespace xn {
namespace {

const char SVC_ID[8] = {'X', 'N', 'D', 'N', '-', 'S', 'V', 'C'};
constexpr uint32_t SVC_VERSION = 1;
constexpr uint32_t SVC_ROPE_RECORDS = 1, SVC_ROPE_TREE = 2;
constexpr uint64_t SVC_HEADER = 64;
constexpr uint32_t LEAF = 0x80000000u;
constexpr uint64_t CHUNK = 32ull << 20;

struct Header {
    char id[8];
    uint32_t version, flags;
    uint64_t side, n_nodes, n_inner, n_leaves;
    uint32_t root_color, root_depth;
    uint64_t reserved;
};
static_assert(sizeof(Header) == SVC_HEADER, "header layout");

struct File {
    std::FILE* f;
    explicit File(std::FILE* f) : f(f) {}
    ~File() {
        if (f) std::fclose(f);
    }
};

// Two pinned chunk buffers with an event each; pending[k]: a copy from or to
// buffer k may still be running (shared by every array streamed through them).
struct Staging {
    void* buf[2] = {nullptr, nullptr};
    cudaEvent_t ev[2] = {nullptr, nullptr};
    bool pending[2] = {false, false};
    ~Staging() {
        for (int k = 0; k < 2; ++k) {
            if (ev[k]) {
                cudaEventSynchronize(ev[k]);
                cudaEventDestroy(ev[k]);
            }
            if (buf[k]) cudaFreeHost(buf[k]);
        }
    }
    int init() {
        for (int k = 0; k < 2; ++k) {
            if (cudaHostAlloc(&buf[k], CHUNK, cudaHostAllocDefault) != cudaSuccess)
                return fail(XN_ERR_NOMEM, "volume file: pinned staging");
            if (cudaEventCreateWithFlags(&ev[k], cudaEventDisableTiming) != cudaSuccess)
                return fail(XN_ERR_CUDA, "volume file: event");
        }
        return XN_OK;
    }
};

// HBM -> file: the copy of chunk i+1 runs while chunk i is written.
int stream_out(cudaStream_t s, Staging& st, std::FILE* f, const void* d, uint64_t bytes, const char* path) {
    const char* src = static_cast<const char*>(d);
    const uint64_t n = (bytes + CHUNK - 1) / CHUNK;
    auto issue = [&](uint64_t i) -> cudaError_t {
        const uint64_t off = i * CHUNK, take = bytes - off < CHUNK ? bytes - off : CHUNK;
        cudaError_t e = cudaMemcpyAsync(st.buf[i & 1], src + off, take, cudaMemcpyDeviceToHost, s);
        return e == cudaSuccess ? cudaEventRecord(st.ev[i & 1], s) : e;
    };
    if (n && issue(0) != cudaSuccess) return fail(XN_ERR_CUDA, "'%s': device read failed", path);
    for (uint64_t i = 0; i < n; ++i) {
        if (cudaEventSynchronize(st.ev[i & 1]) != cudaSuccess) return fail(XN_ERR_CUDA, "'%s': device read failed", path);
        if (i + 1 < n && issue(i + 1) != cudaSuccess) return fail(XN_ERR_CUDA, "'%s': device read failed", path);
        const uint64_t off = i * CHUNK, take = bytes - off < CHUNK ? bytes - off : CHUNK;
        if (std::fwrite(st.buf[i & 1], 1, take, f) != take) return fail(XN_ERR_IO, "'%s': write failed", path);
    }
    return XN_OK;
}

// file -> HBM: chunk i+1 is read while chunk i is copied.
int stream_in(cudaStream_t s, Staging& st, std::FILE* f, void* d, uint64_t bytes, const char* path) {
    char* dst = static_cast<char*>(d);
    const uint64_t n = (bytes + CHUNK - 1) / CHUNK;
    for (uint64_t i = 0; i < n; ++i) {
        const int k = (int)(i & 1);
        if (st.pending[k] && cudaEventSynchronize(st.ev[k]) != cudaSuccess)
            return fail(XN_ERR_CUDA, "'%s': device write failed", path);
        const uint64_t off = i * CHUNK, take = bytes - off < CHUNK ? bytes - off : CHUNK;
        if (std::fread(st.buf[k], 1, take, f) != take) return fail(XN_ERR_IO, "'%s': short read", path);
        if (cudaMemcpyAsync(dst + off, st.buf[k], take, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaEventRecord(st.ev[k], s) != cudaSuccess)
            return fail(XN_ERR_CUDA, "'%s': device write failed", path);
        st.pending[k] = true;
    }
    return XN_OK;
}

// Flags [0]: an index out of range; [1]: a depth field that does not match
// the tree (the root's is not 0, or an internal child's is not its parent's
// plus one).
__global__ void check_layout_kernel(const uint32_t* inner, const uint32_t* depth, const uint32_t* rinner,
                                    const uint32_t* leaves, uint64_t n_inner, uint64_t n_leaves, uint32_t* flags) {
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t bad = 0, inconsistent = 0;
    for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n_inner + n_leaves; j += stride) {
        if (j < n_inner) {
            if (j == 0 && depth[0] != 0) inconsistent = 1;
            for (int k = 0; k < 8; ++k) {
                const uint32_t w = inner[j * 8 + k];
                if (!(w & LEAF)) {
                    if (w >= n_inner) bad = 1;
                    else if (depth[w] != depth[j] + 1) inconsistent = 1;
                }
                if (rinner) {
                    const uint32_t r = rinner[j * 8 + k];
                    if ((r & LEAF) ? (r & ~LEAF) >= n_leaves : r >= n_inner) bad = 1;
                    if (((r & LEAF) != 0) != ((w & LEAF) != 0)) bad = 1;
                }
            }
        } else {
            const uint64_t l = j - n_inner;
            for (int k = 1; k <= 6; ++k) {
                const uint32_t r = leaves[l * 8 + k];
                if (r == ROPE_EXIT) continue;
                if ((r & LEAF) ? (r & ~LEAF) >= n_leaves : r >= n_inner) bad = 1;
            }
        }
    }
    if (bad) atomicOr(flags, 1u);
    if (inconsistent) atomicOr(flags + 1, 1u);
}

}  // namespace

// Checks a compact-layout volume's arrays on the device (every index in
// range) and records whether its depth fields match the tree.
int validate_compact_layout(Ctx* c, Volume* v, const char* what) {
    uint32_t* flags = nullptr;
    uint32_t hf[2] = {1, 1};
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void**>(&flags), 8, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(flags, 0, 8, c->stream);
    if (e == cudaSuccess) {
        check_layout_kernel<<<1024, 256, 0, c->stream>>>(v->inner, v->inner_depth, v->rinner, v->leaves, v->n_inner,
                                                           v->rinner ? v->n_leaves : 0, flags);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(hf, flags, 8, cudaMemcpyDeviceToHost, c->stream);
    if (flags) cudaFreeAsync(flags, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) return cuda_fail(e, what);
    if (hf[0]) return fail(XN_ERR_FORMAT, "%s: an index is out of range", what);
    v->depth_consistent = hf[1] == 0;
    return XN_OK;
}

}  // namespace xn

using namespace xn;

XN_API int xn_volume_save(xn_ctx* h, const xn_volume* vh, const char* path) {
    if (!h || !vh || !path) return fail(XN_ERR_ARG, "xn_volume_save: NULL argument");
    Ctx* c = reinterpret_cast<Ctx*>(h);
    const Volume* v = reinterpret_cast<const Volume*>(vh);
    if (v->ctx != c) return fail(XN_ERR_ARG, "xn_volume_save: volume belongs to another context");
    if (v->kind != XN_VOLUME_SVO) return fail(XN_ERR_ARG, "xn_volume_save: not an octree volume");
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    Header hd{};
    std::memcpy(hd.id, SVC_ID, 8);
    hd.version = SVC_VERSION;
    hd.side = v->side;
    hd.n_nodes = v->n_nodes;
    hd.flags = v->has_ropes ? SVC_ROPE_TREE : 0;
    if (v->layout == XN_LAYOUT_REFERENCE) {
        // a leaf root keeps the reference node: store its colour and depth word
        uint32_t node[10];
        cudaError_t e = cudaMemcpyAsync(node, v->data, 40, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return cuda_fail(e, "xn_volume_save");
        if (node[9] < LEAF) return fail(XN_ERR_STATE, "xn_volume_save: octree has no device layout");
        hd.root_color = node[8];
        hd.root_depth = node[9];
    } else {
        hd.n_inner = v->n_inner;
        if (v->rinner && v->leaves) {
            hd.flags |= SVC_ROPE_RECORDS;
            hd.n_leaves = v->n_leaves;
        }
    }
    File out(std::fopen(path, "wb"));
    if (!out.f) return fail(XN_ERR_IO, "Failed to open '%s'", path);
    if (std::fwrite(&hd, 1, sizeof hd, out.f) != sizeof hd) return fail(XN_ERR_IO, "'%s': write failed", path);
    Staging st;
    if ((r = st.init())) return r;
    if (hd.n_inner) {
        if ((r = stream_out(c->stream, st, out.f, v->inner, hd.n_inner * 32, path)) ||
            (r = stream_out(c->stream, st, out.f, v->inner_depth, hd.n_inner * 4, path)))
            return r;
        if (hd.flags & SVC_ROPE_RECORDS) {
            if ((r = stream_out(c->stream, st, out.f, v->rinner, hd.n_inner * 32, path)) ||
                (r = stream_out(c->stream, st, out.f, v->leaves, hd.n_leaves * 32, path)))
                return r;
        }
    }
    if (std::fflush(out.f) != 0) return fail(XN_ERR_IO, "'%s': write failed", path);
    return XN_OK;
}

XN_API int xn_volume_load(xn_ctx* h, const char* path, xn_volume** out) {
    if (!h || !path || !out) return fail(XN_ERR_ARG, "xn_volume_load: NULL argument");
    *out = nullptr;
    File in(std::fopen(path, "rb"));
    if (!in.f) return fail(XN_ERR_IO, "Failed to open '%s'", path);
    Header hd{};
    if (std::fread(&hd, 1, sizeof hd, in.f) != sizeof hd) return fail(XN_ERR_FORMAT, "'%s': truncated header", path);
    if (std::memcmp(hd.id, SVC_ID, 8) != 0) return fail(XN_ERR_FORMAT, "'%s': Invalid format id", path);
    if (hd.version != SVC_VERSION) return fail(XN_ERR_FORMAT, "'%s': unsupported version %u", path, hd.version);
    if (hd.flags & ~(SVC_ROPE_RECORDS | SVC_ROPE_TREE)) return fail(XN_ERR_FORMAT, "'%s': unknown flags", path);
    if (hd.n_inner >= LEAF || hd.n_leaves >= ROPE_EXIT - LEAF)
        return fail(XN_ERR_FORMAT, "'%s': more than 2^31 internal nodes or leaves", path);
    if (!(hd.flags & SVC_ROPE_RECORDS) && hd.n_leaves)
        return fail(XN_ERR_FORMAT, "'%s': leaf records without the rope flag", path);
    if (hd.n_inner == 0 && (hd.root_depth < LEAF || (hd.flags & SVC_ROPE_RECORDS)))
        return fail(XN_ERR_FORMAT, "'%s': a tree without internal nodes needs a leaf root", path);
    const uint64_t body = hd.n_inner * 36 + ((hd.flags & SVC_ROPE_RECORDS) ? hd.n_inner * 32 + hd.n_leaves * 32 : 0);
    if (std::fseek(in.f, 0, SEEK_END) != 0) return fail(XN_ERR_IO, "'%s': Failed to tell", path);
    const long end = std::ftell(in.f);
    if (end < 0) return fail(XN_ERR_IO, "'%s': Failed to tell", path);
    if ((uint64_t)end != SVC_HEADER + body)
        return fail(XN_ERR_FORMAT, "'%s': File size does not match the header", path);
    if (std::fseek(in.f, (long)SVC_HEADER, SEEK_SET) != 0) return fail(XN_ERR_IO, "'%s': seek failed", path);

    Ctx* c = reinterpret_cast<Ctx*>(h);
    std::lock_guard<std::mutex> lk(c->mu);
    int r = c->activate();
    if (r) return r;
    Volume* v = new (std::nothrow) Volume();
    if (!v) return fail(XN_ERR_NOMEM, "xn_volume_load: out of host memory");
    v->ctx = c;
    v->kind = XN_VOLUME_SVO;
    v->side = hd.side;
    v->n_nodes = hd.n_nodes;
    const uint64_t sd = hd.side > 0xFFFFFFFFull ? 0xFFFFFFFFull : hd.side;
    v->dim[0] = v->dim[1] = v->dim[2] = (uint32_t)sd;
    v->has_ropes = (hd.flags & SVC_ROPE_TREE) != 0;
    auto drop = [&](int code) {
        cudaStreamSynchronize(c->stream);
        c->device_free(v->data, v->bytes);
        v->release_layout();
        delete v;
        return code;
    };
    if (hd.n_inner == 0) {
        // a leaf root: the one-node reference layout
        const uint32_t node[10] = {0, 0, 0, 0, 0, 0, 0, 0, hd.root_color, hd.root_depth};
        v->bytes = 40;
        v->layout = XN_LAYOUT_REFERENCE;
        if ((r = c->device_alloc(&v->data, 40, "xn_volume_load"))) return drop(r);
        cudaError_t e = cudaMemcpyAsync(v->data, node, 40, cudaMemcpyHostToDevice, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) return drop(cuda_fail(e, "xn_volume_load"));
        *out = reinterpret_cast<xn_volume*>(v);
        return XN_OK;
    }
    const bool ropes = (hd.flags & SVC_ROPE_RECORDS) != 0;
    v->n_inner = hd.n_inner;
    v->n_leaves = hd.n_leaves;
    if ((r = c->device_alloc(reinterpret_cast<void**>(&v->inner), hd.n_inner * 32, "xn_volume_load: inner")) ||
        (r = c->device_alloc(reinterpret_cast<void**>(&v->inner_depth), hd.n_inner * 4, "xn_volume_load: depths")))
        return drop(r);
    if (ropes &&
        ((r = c->device_alloc(reinterpret_cast<void**>(&v->rinner), hd.n_inner * 32, "xn_volume_load: rope inner")) ||
         (r = c->device_alloc(reinterpret_cast<void**>(&v->leaves), hd.n_leaves * 32, "xn_volume_load: leaves"))))
        return drop(r);
    {
        Staging st;
        if ((r = st.init())) return drop(r);
        if ((r = stream_in(c->stream, st, in.f, v->inner, hd.n_inner * 32, path)) ||
            (r = stream_in(c->stream, st, in.f, v->inner_depth, hd.n_inner * 4, path)))
            return drop(r);
        if (ropes && ((r = stream_in(c->stream, st, in.f, v->rinner, hd.n_inner * 32, path)) ||
                      (r = stream_in(c->stream, st, in.f, v->leaves, hd.n_leaves * 32, path))))
            return drop(r);
    }
    if ((r = validate_compact_layout(c, v, path))) return drop(r);
    v->layout = XN_LAYOUT_COMPACT;
    if ((r = measure_inner_depth(c, v))) return drop(r);
    *out = reinterpret_cast<xn_volume*>(v);
    return XN_OK;
}

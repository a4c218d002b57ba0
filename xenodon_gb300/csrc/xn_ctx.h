// Host-side state behind the opaque xn_ctx / xn_volume handles.
#pragma once

#include <atomic>
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

#include "../../include/xenodon.h"

namespace xn {

struct DeviceBuffer {
    void* ptr = nullptr;
    uint64_t bytes = 0;
};

// One CUDA device, its stream, and the HBM budget every allocation of this
// context is checked against.
struct Ctx {
    int device = 0;
    uint64_t budget = 0;  // 0 = no cap
    std::atomic<uint64_t> used{0};
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint32_t* d_err = nullptr;  // ray error bits
    DeviceBuffer out_rgba, out_emission;
    int tex_norm_exact = -1;  // texture UNORM8 conversion equals byte/255 (-1: not checked yet)
    // batches (batch.cu)
    int sms = 0;
    void* batch_host = nullptr;  // pinned job table
    uint64_t batch_host_bytes = 0;
    cudaEvent_t batch_copied = nullptr;
    xn_batch_config tuned[32] = {};
    int tuned_valid[32] = {};
    std::mutex mu;

    int sm_count();

    int activate();
    int device_alloc(void** p, uint64_t bytes, const char* what);
    void device_free(void* p, uint64_t bytes);
    int ensure_buffer(DeviceBuffer& b, uint64_t bytes, const char* what);
    void release_extra();
};

struct Volume {
    Ctx* ctx = nullptr;
    int kind = 0;          // xn_volume_kind
    uint32_t dim[3] = {0, 0, 0};
    uint64_t side = 0;
    uint64_t n_nodes = 0;
    int has_ropes = 0;
    void* data = nullptr;  // grid texels or reference node words
    uint64_t bytes = 0;
    // grid texture form (xn_volume_upload_grid)
    cudaArray_t array = nullptr;
    cudaTextureObject_t tex = 0;
    int tex_normalized = 0;  // texel form: 0 bytes (converted in the kernel), 1 byte/255 from the texture unit, 2 one packed word
    int bricked = 0;  // grid kept in the bricked form (XN_GRID_LAYOUT=bricked)
    int hybrid = 0;   // texture plus an x-fastest copy (XN_GRID_LAYOUT=hybrid)
    uint64_t array_bytes = 0;
    // octree device layout (svo_layout.cu)
    int layout = 0;
    uint64_t n_inner = 0, n_leaves = 0;
    uint32_t* inner = nullptr;
    uint32_t* rinner = nullptr;
    uint32_t* inner_depth = nullptr;
    uint32_t* leaves = nullptr;
    int depth_consistent = 0;  // internal nodes' depth fields match the tree (svo_layout.cu)
    uint32_t max_inner_depth = 0xFFFFFFFFu;  // deepest internal node of a depth-consistent tree, else ~0

    uint64_t layout_bytes() const {
        return (inner ? n_inner * 32 : 0) + (rinner ? n_inner * 32 : 0) + (inner_depth ? n_inner * 4 : 0) +
               (leaves ? n_leaves * 32 : 0);
    }
    void release_layout() {
        if (!ctx) return;
        ctx->device_free(inner, n_inner * 32);
        ctx->device_free(rinner, n_inner * 32);
        ctx->device_free(inner_depth, n_inner * 4);
        ctx->device_free(leaves, n_leaves * 32);
        inner = rinner = inner_depth = leaves = nullptr;
    }
};

int build_svo_layout(Ctx* c, Volume* v);
// Sets v->max_inner_depth from the internal nodes' depth fields when the tree
// is depth-consistent (svo_layout.cu).
int measure_inner_depth(Ctx* c, Volume* v);
// Range-checks a compact-layout volume's arrays on the device and sets its
// depth_consistent flag (volume_io.cu).
int validate_compact_layout(Ctx* c, Volume* v, const char* what);

// Octree build on the device (svo_build.cu).  With lean == nullptr: the
// reference node array in *d_nodes.  With lean: only the device layout's
// inner / inner_depth arrays, written into *lean (sparse trees; no rope
// records); returns LEAN_LEAF_ROOT when the root is a leaf (no internal nodes).
constexpr int LEAN_LEAF_ROOT = 1;
// A build of one cube of a larger tree (the streamed convert): the cube's
// side (a power of two at least the grid's dims, where the grid is the part of
// the whole grid inside the cube), the depth of its root in the whole tree,
// and on return the root cell's scan statistics (the heuristic's statistics
// struct, at most 64 bytes) for the decision of the whole tree's root.
struct SubBuild {
    uint64_t side = 0;
    int depth_offset = 0;
    unsigned char root_stats[64] = {};
};
int build_svo_device(Ctx* c, const uint32_t* d_vox, uint32_t dx, uint32_t dy, uint32_t dz, int type, int heuristic,
                     double threshold, uint32_t** d_nodes, uint64_t* d_nodes_bytes, xn_build_stats* stats,
                     Volume* lean = nullptr, SubBuild* sub = nullptr);

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int cuda_fail(cudaError_t e, const char* what);

}  // namespace xn

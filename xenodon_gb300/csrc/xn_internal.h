// Internal interfaces between the C-ABI layer and the CUDA kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace xn {

// device octree layouts (see svo_layout.cu)
enum { XN_LAYOUT_REFERENCE = 0, XN_LAYOUT_COMPACT = 1 };
// rope word meaning "no neighbour" in the compact layout (the reference's rope to node 0)
constexpr uint32_t ROPE_EXIT = 0xFFFFFFFFu;

enum {
    XN_TRAV_DDA = 0,
    XN_TRAV_SVO_NAIVE = 1,
    XN_TRAV_ESVO = 2,
    XN_TRAV_SVO_DF = 3,
    XN_TRAV_SVO_ROPE = 4,
    XN_TRAV_SVO_DF_MASKED = 5,  // svo-df on an octree with consistent depth fields (render.cu)
    XN_TRAV_SVO_NAIVE_ROOT = 6  // svo-naive with every find from the root
};

// Everything one traversal launch needs; built by the C-ABI layer from an
// xn_camera + xn_params + volume.
struct RenderLaunch {
    int traversal;
    float forward[3], up[3];
    float translation[3];  // divided by voxel_ratio on the host
    float voxel_ratio[3];
    float aspect;
    float emission_coeff;
    int32_t out_x, out_y;
    uint32_t out_w, out_h;
    int32_t disp_x, disp_y;
    uint32_t disp_w, disp_h;
    // volume
    const void* grid;   // uchar4 texels, x fastest (DDA, linear form)
    unsigned long long tex;  // cudaTextureObject_t of the texture form, or 0
    int tex_normalized;      // 1: the texture returns byte/255 itself; 0: four bytes; 2: one packed word
    int grid_bricked;        // `grid` is the bricked form (render.cu BrickGrid), not x-fastest
    int grid_hybrid;         // both `tex` and an x-fastest `grid`: some warps read each (render.cu)
    uint32_t dim[3];
    const void* nodes;  // reference node words (octree traversals, reference layout)
    int layout;
    const uint32_t* inner;        // compact layout (svo_layout.cu)
    const uint32_t* rinner;
    const uint32_t* inner_depth;
    const uint32_t* leaves;
    int depth_consistent;         // every internal node's depth field = its depth in the tree
    int shared_stacks;            // esvo and masked svo-df with their stacks in shared memory
    int naive_resume;             // svo-naive's find resumes from the previous step's path
    int df_packet;                // masked svo-df walked by the whole warp (df_packet_kernel)
    float df_lane_side;           // child size of the nodes below which the lanes walk alone: 2^-D
                                  // (one level; D the deepest internal node's depth) or 2^-(D-1)
                                  // (two levels), or 0
    int df_lane_levels;           // 1 or 2
    // outputs (device pointers)
    void* d_rgba;
    float* d_emission;
    uint32_t* d_loads;
    uint32_t* d_err_word;
};

cudaError_t launch_render(const RenderLaunch& launch, cudaStream_t stream);
// The bricked grid form (render.cu): 8x8x8-texel bricks of 2 KB, one brick of
// zeros around the grid on every side; within a brick, 16-byte groups of 2x2x1
// texels.  Bytes for a dx x dy x dz grid:
uint64_t brick_grid_bytes(uint32_t dx, uint32_t dy, uint32_t dz);
// Writes the bricked form of an x-fastest device grid into `bricks`
// (brick_grid_bytes of zeroed device memory).
cudaError_t brick_grid(const uint32_t* src, uint32_t dx, uint32_t dy, uint32_t dz, void* bricks, cudaStream_t s);

// One job of a persistent batch launch (device copy of a RenderLaunch plus its
// place in the batch's tile sequence).
struct alignas(16) BatchJob {
    float forward[3], up[3], translation[3], voxel_ratio[3];
    float aspect, emission_coeff;
    int32_t out_x, out_y;
    uint32_t out_w, out_h;
    int32_t disp_x, disp_y;
    uint32_t disp_w, disp_h;
    int32_t traversal, layout;  // layout: grids 0 linear / 1 texture / 2 bricked; octrees XN_LAYOUT_*
    uint32_t dim[3];
    int32_t tex_normalized;
    int32_t depth_consistent;
    int32_t form;  // XN_BATCH_* form of this job (batch_spec)
    float df_lane_side;  // svo-df: child size 2^-D of the nodes whose children the lanes walk alone, or 0
    unsigned long long tex;
    const void* grid;
    const void* nodes;
    const uint32_t* inner;
    const uint32_t* rinner;
    const uint32_t* inner_depth;
    const uint32_t* leaves;
    void* rgba;
    uint32_t tiles_x, tiles_y;
    unsigned long long tile_begin;  // first tile of this job in the batch
};

struct alignas(16) BatchHeader {
    uint32_t n_jobs, pad;
    unsigned long long total_tiles;
};

BatchJob make_batch_job(const RenderLaunch& L);
// Batch kernel forms: one traversal (and layout) inlined when every job of
// the batch shares it, else the generic per-pixel dispatch.
enum { XN_BATCH_ANY = 0, XN_BATCH_DDA_TEX_NORM, XN_BATCH_DDA_TEX_RAW, XN_BATCH_ESVO, XN_BATCH_NAIVE, XN_BATCH_DF,
       XN_BATCH_ROPE, XN_BATCH_FORMS };
// The form a job needs (XN_BATCH_*).
int batch_spec(const BatchJob& j);
// Launches the persistent kernel over a job table already in device memory
// (header followed by the jobs).  tile_w is the warp tile's width in pixels
// (4, 8, 16 or 32; height 32/tile_w); spec is the form every job shares, or
// XN_BATCH_ANY.
cudaError_t launch_batch(const void* d_table, unsigned long long* d_queue, uint32_t* d_err, uint32_t tile_w,
                         uint32_t threads, uint32_t blocks, uint32_t chunk, int spec, cudaStream_t s);
int batch_kernel_blocks_per_sm(uint32_t tile_w, uint32_t block_threads);

// Control words of a folding ring (render.cu fold_kernel), in device memory.
struct alignas(16) FoldCtl {
    unsigned long long published;  // tiles published (host writes, by copy)
    unsigned long long taken;      // tiles claimed (device)
    uint32_t closed;               // host: no more jobs; exit once every published tile is taken
    uint32_t exit_flag;            // device: the ring went idle; no warp claims a tile after it
    uint32_t status;               // device: bit 0, left because idle
    uint32_t pad;
};
// Launches the persistent folding kernel (blocks of `threads`, 32 or 128;
// the generic per-pixel form, warp tiles of tile_w x 32/tile_w) over a ring
// of `cap` job slots; done_flags is mapped host memory: one word per slot,
// then one word the kernel sets when it decides to leave.
cudaError_t launch_fold(FoldCtl* ctl, const BatchJob* ring, uint32_t cap, uint32_t* done_tiles,
                        uint32_t* done_flags_mapped, uint32_t* err, uint32_t tile_w, uint32_t threads, uint32_t blocks,
                        unsigned long long idle_ns, cudaStream_t s);

}  // namespace xn

/*
 * xenodon-gb300: C ABI of the GB300 volume ray-traversal library.
 *
 * Plain C types only: opaque handles, pointers and sizes.  Every function
 * returns an int status (XN_OK = 0, negative = error); the message of the last
 * error on the calling thread is available from xn_last_error().  No C++
 * exception crosses this boundary.  Host buffers belong to the caller; device
 * memory belongs to the library (a context and the volumes created from it),
 * except for the xn_*_device entry points, which write into caller-owned
 * device buffers on a caller-given CUDA stream.
 *
 * Each declaration names the reference interface it stands in for
 * (paths relative to the reference project root).
 */
#ifndef XENODON_H
#define XENODON_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
#define XN_EXTERN extern "C"
#else
#define XN_EXTERN extern
#endif
#define XN_API XN_EXTERN __attribute__((visibility("default")))

#define XN_ABI_VERSION 1

/* ---- status codes ---- */
enum {
    XN_OK = 0,
    XN_ERR_ARG = -1,       /* invalid argument */
    XN_ERR_CUDA = -2,      /* a CUDA call failed */
    XN_ERR_NOMEM = -3,     /* host or device allocation failed */
    XN_ERR_FORMAT = -4,    /* malformed file or octree */
    XN_ERR_BUDGET = -5,    /* the context's HBM budget does not admit the request */
    XN_ERR_RAY_LIMIT = -6, /* a ray hit an iteration cap or a stack limit (output still written) */
    XN_ERR_IO = -7,        /* file could not be opened, read or written */
    XN_ERR_STATE = -8      /* call not valid in the current state */
};

/* Traversal algorithms, in the order of src/main_loop.cpp:37-43 (SHADER_OPTIONS). */
typedef enum {
    XN_DDA = 0,       /* resources/dda.comp */
    XN_SVO_NAIVE = 1, /* resources/svo_naive.comp */
    XN_ESVO = 2,      /* resources/esvo.comp */
    XN_SVO_DF = 3,    /* resources/svo_df.comp */
    XN_SVO_ROPE = 4   /* resources/svo_rope.comp */
} xn_traversal;

typedef enum { XN_VOLUME_GRID = 0, XN_VOLUME_SVO = 1 } xn_volume_kind;

/* Octree types and split heuristics of `xenodon convert` (src/convert.cpp:24-37,
 * src/model/Octree.h:16-20, src/model/OctreeConstruction.h:32-48). */
typedef enum { XN_SVO_SPARSE = 0, XN_SVO_DAG = 1, XN_SVO_ROPE_TREE = 2 } xn_svo_type;
typedef enum { XN_HEUR_CHANNEL_DIFF = 0, XN_HEUR_STD_DEV = 1 } xn_heuristic;

typedef struct xn_ctx xn_ctx;
typedef struct xn_volume xn_volume;

/* src/camera/Camera.h:6-10; one line of a camera script (ScriptCameraController.cpp:17-40). */
typedef struct {
    float forward[3];
    float up[3];
    float translation[3]; /* raw: the library divides by voxel_ratio (src/render/Renderer.cpp:62) */
} xn_camera;

/* vk::Rect2D as used by the UBO of resources/common.glsl:12-15,29-33. */
typedef struct {
    int32_t x, y;
    uint32_t width, height;
} xn_rect;

/* UBO contents (resources/common.glsl:17-21,29-33; src/render/RenderContext.h:16-20).
 * model_dim is taken from the volume. */
typedef struct {
    xn_rect output_region;  /* the pixels this call renders */
    xn_rect display_region; /* the union rectangle uv is computed against */
    float voxel_ratio[3];   /* --voxel-ratio, default 1:1:1 */
    float emission_coeff;   /* -e, default 1 */
} xn_params;

typedef struct {
    int kind;              /* xn_volume_kind */
    uint32_t dim[3];       /* grid dimensions, or side^3 for an octree */
    uint64_t side;         /* octree side (power of two), 0 for grids */
    uint64_t n_nodes;      /* octree nodes in the reference layout, 0 for grids */
    uint64_t device_bytes; /* HBM held by this volume */
    int has_ropes;         /* octree leaves carry rope links (svo-rope is valid) */
} xn_volume_info;

/* ConstructionStats (src/model/OctreeConstruction.h:50-62) plus the result size. */
typedef struct {
    uint64_t total_leaves;
    uint64_t unique_leaves;
    uint64_t total_nodes;
    uint64_t depth;
    uint64_t side;
    uint64_t n_nodes;
} xn_build_stats;

/* ------------------------------------------------------------- context --- */

/* Replaces the per-device Vulkan setup of src/backend/headless/HeadlessOutput.cpp:38-63
 * and src/render/Renderer.cpp:17-30: one CUDA device context.  hbm_budget_bytes
 * caps what volumes and render targets of this context may hold (0 = no cap). */
XN_API int xn_create(int device, uint64_t hbm_budget_bytes, xn_ctx** out);
XN_API int xn_destroy(xn_ctx* ctx);
/* Message of the last failed call on this thread ("" if none). */
XN_API const char* xn_last_error(void);
XN_API int xn_abi_version(void);
/* Device memory currently held by the context's volumes and buffers. */
XN_API int xn_ctx_memory(const xn_ctx* ctx, uint64_t* used_bytes, uint64_t* budget_bytes);

/* -------------------------------------------------------------- volumes --- */

/* Replaces DdaRaytraceAlgorithm::upload_resources / DdaRaytraceResources
 * (src/render/DdaRaytraceAlgorithm.cpp:15-97): uploads an RGBA8 grid, x fastest
 * (src/model/Grid.h:50-52), dx*dy*dz*4 bytes from host memory. */
XN_API int xn_volume_upload_grid(xn_ctx* ctx, const uint8_t* rgba, uint32_t dx, uint32_t dy,
                                 uint32_t dz, xn_volume** out);

/* Replaces SvoRaytraceAlgorithm::upload_resources / SvoRaytraceResources
 * (src/render/SvoRaytraceAlgorithm.cpp:12-48): uploads n_nodes nodes of 10
 * little-endian u32 words (resources/octree.glsl:6-10, src/model/Octree.h:35-45).
 * The octree is validated (every child index < n_nodes) and re-laid out on the
 * device for traversal. */
XN_API int xn_volume_upload_svo(xn_ctx* ctx, const uint32_t* nodes, uint64_t n_nodes, uint64_t side,
                                xn_volume** out);
/* xn_volume_upload_svo with a choice of node format (the plugin boundary's
 * node_fmt):
 *   XN_NODES_U32  the reference's nodes, 10 little-endian u32 (as above);
 *   XN_NODES_U64  72-byte nodes: the eight child indices as u64, then the u32
 *                 colour and the u32 is_leaf_depth -- the reference's node
 *                 with 64-bit indices, for trees of 2^32 nodes or more (no
 *                 counterpart in the reference, whose indices are u32,
 *                 src/model/OctreeConstruction.h:74-76).  Such an array does
 *                 not fit in HBM: it is read twice from host memory in chunks
 *                 and only the device layout is kept (36 bytes per internal
 *                 node, at most 2^31 - 1 of them).  Rope words are not
 *                 converted: svo-rope is refused on the volume.
 * 8-byte aligned host memory. */
#define XN_NODES_U32 0
#define XN_NODES_U64 1
XN_API int xn_volume_upload_svo_fmt(xn_ctx* ctx, const void* nodes, uint64_t n_nodes, uint64_t side, int node_fmt,
                                    xn_volume** out);
/* xn_volume_upload_grid from a grid already in device memory (no host copy). */
XN_API int xn_volume_upload_grid_device(xn_ctx* ctx, const void* d_rgba, uint32_t dx, uint32_t dy, uint32_t dz,
                                        xn_volume** out);
XN_API int xn_volume_release(xn_volume* vol);
XN_API int xn_volume_info_get(const xn_volume* vol, xn_volume_info* info);

/* -------------------------------------------------------------- render --- */

/* Replaces Renderer::render + HeadlessOutput::synchronize/download
 * (src/render/Renderer.cpp:55-103, src/backend/headless/HeadlessOutput.cpp:90-136):
 * renders params->output_region with the given traversal and copies the result
 * to host memory.
 *   out_rgba      width*height*4 bytes (row pitch width*4), or NULL
 *   out_emission  width*height*3 floats: colour after the emission coefficient,
 *                 before the UNORM clamp, or NULL
 *   kernel_ms     device time of the traversal kernel (the quantity of
 *                 src/render/RenderStats.cpp:59-83), or NULL
 * Returns XN_ERR_RAY_LIMIT, with the outputs written, when a ray hit an
 * iteration cap (where the reference shader would not terminate). */
XN_API int xn_render(xn_ctx* ctx, const xn_volume* vol, int traversal, const xn_camera* cam,
                     const xn_params* params, uint8_t* out_rgba, float* out_emission,
                     float* kernel_ms);

/* Device-side form of xn_render: writes into caller-owned device buffers on
 * `stream` (a cudaStream_t, NULL = the legacy default stream) and returns
 * without synchronising.  d_loads, when not NULL, receives per ray the number
 * of 32-bit words the reference shader reads (texels for DDA, node words for
 * the octree traversals). */
XN_API int xn_render_device(xn_ctx* ctx, const xn_volume* vol, int traversal, const xn_camera* cam,
                            const xn_params* params, void* d_rgba, float* d_emission,
                            uint32_t* d_loads, void* stream);

/* An output region's render target with its host read-back buffer and its
 * fence: the asynchronous form of xn_render, replacing HeadlessOutput's image,
 * staging buffer and fence (src/backend/headless/HeadlessOutput.cpp:38-136).
 * The read-back goes into pinned host memory with an asynchronous copy, so a
 * caller renders the next frame into a second output while it encodes this
 * one.
 *   xn_output_create   an output of up to max_pixels pixels (device image,
 *                      pinned host image, events, error word, copy stream)
 *   xn_output_render   queues the render of params->output_region (at most
 *                      max_pixels pixels) on the context's stream, timed by
 *                      events, then the copy into the pinned image on the
 *                      output's own stream, so the next render's kernel does
 *                      not wait for it (the copy is skipped with
 *                      XN_OUTPUT_DISCARD, the reference's --discard-output);
 *                      returns at once.  The previous render into this output
 *                      must have been waited for.
 *   xn_output_wait     the fence: blocks until the queued render and copy are
 *                      done; *rgba (width*height*4 bytes, row pitch width*4)
 *                      stays valid until the next xn_output_render on this
 *                      output; *kernel_ms as xn_render.  Returns
 *                      XN_ERR_RAY_LIMIT like xn_render.
 * Outputs of one context share its stream, so their renders run in the order
 * they were queued; waits may come from any thread. */
typedef struct xn_output xn_output;
#define XN_OUTPUT_DISCARD 1
XN_API int xn_output_create(xn_ctx* ctx, uint64_t max_pixels, xn_output** out);
XN_API int xn_output_render(xn_output* out, const xn_volume* vol, int traversal, const xn_camera* cam,
                            const xn_params* params, int flags);
XN_API int xn_output_wait(xn_output* out, const uint8_t** rgba, float* kernel_ms);
XN_API int xn_output_destroy(xn_output* out);

/* ---------------------------------------------------------- batching --- */

/* One frame of a batch (no counterpart in the reference, which renders one
 * frame per dispatch): a volume, a traversal, a camera, the regions, and a
 * caller-owned device buffer of output_region.width*height*4 bytes. */
typedef struct {
    const xn_volume* volume;
    int traversal;
    xn_camera camera;
    xn_params params;
    void* d_rgba;
} xn_job;

/* Launch shape of the persistent batch kernel, or (tile_width XN_BATCH_PLAIN)
 * the plain form: each job through the single-frame kernels, one launch per
 * frame, in order. */
#define XN_BATCH_PLAIN 0
typedef struct {
    uint32_t tile_width;    /* warp tile width in pixels: 4, 8, 16 or 32 (height = 32/width); 0: plain */
    uint32_t block_threads; /* threads per block: a multiple of 32, at most 1024 */
    uint32_t blocks_per_sm; /* resident blocks per SM; 0 = as many as fit */
    uint32_t chunk;         /* warp tiles a warp takes per pop of the work queue; 0: no queue, a grid of
                               one warp per tile (batch graphs use 1 instead) */
} xn_batch_config;

/* Renders n_jobs frames of any mix of volumes, traversals and resolutions in
 * one launch on `stream` (returns without synchronising).  With a queue
 * (chunk >= 1) resident warps pull tiles from one global counter; with chunk
 * 0, a grid holds one warp per tile.  cfg NULL means the configuration the
 * autotuner chose for this mix of traversals, else 4x8 tiles in blocks of 256
 * with no queue. */
XN_API int xn_render_batch(xn_ctx* ctx, const xn_job* jobs, int n_jobs, const xn_batch_config* cfg, void* stream);

/* Times xn_render_batch over a sweep of launch shapes, the plain form among
 * them, on the given jobs and keeps the fastest for their mix of traversals
 * (used when cfg is NULL): every shape once on up to 8 jobs spread over the
 * batch, then the three fastest and the plain form twice on the whole batch. */
XN_API int xn_autotune_batch(xn_ctx* ctx, const xn_job* jobs, int n_jobs, void* stream, xn_batch_config* best,
                             float* best_ms);

/* A batch launch captured once as a CUDA graph (job-table upload, queue reset,
 * persistent kernel) and replayed per batch; two graph instances alternate so
 * the host fills the next job table while the previous batch runs. */
typedef struct xn_batch_graph xn_batch_graph;
XN_API int xn_batch_graph_create(xn_ctx* ctx, int capacity_jobs, const xn_batch_config* cfg, void* stream,
                                 xn_batch_graph** out);
XN_API int xn_batch_graph_launch(xn_batch_graph* g, const xn_job* jobs, int n_jobs);
XN_API int xn_batch_graph_destroy(xn_batch_graph* g);

/* ----------------------------------------------------------- serving --- */

/* A render server (no counterpart in the reference).  A worker thread keeps
 * registered volumes resident with least-recently-used eviction under an HBM
 * budget (a volume is uploaded when it is registered, if it fits) and admits
 * requests in arrival order as memory allows.  Frames below fold_max_pixels
 * are folded into a persistent kernel while it runs: each is appended to a
 * job ring in device memory that the kernel reads as it goes, on a
 * high-priority stream, and copied out as soon as its own tiles are done.
 * The kernel leaves after fold_idle_us without work (its waits are bounded)
 * and is launched again when frames arrive.  Larger frames (each fills the GPU
 * alone) run through the single-frame kernels on low-priority streams,
 * `streams` of them in flight, whole or in bands of rows.  A copy thread
 * moves finished frames into the callers' buffers. */
typedef struct xn_server xn_server;
typedef struct {
    uint64_t hbm_budget;   /* bytes for resident volumes and in-flight frames; 0 = the context's budget */
    int max_batch_jobs;    /* job slots of a folding ring: frames one persistent launch takes (default 1024) */
    int streams;           /* large frames in flight at once, one stream each (default 2, at most 16) */
    uint64_t fold_max_pixels;    /* frames below this many pixels are folded (0: 2^19) */
    uint32_t fold_idle_us;       /* the persistent kernel leaves after this long without work (0: 300) */
    uint32_t fold_blocks_per_sm; /* its blocks of 4 warps per SM, 1 to 4 (0: 2) */
    uint64_t band_pixels;  /* large frames are launched in bands of rows of about this many pixels (0: whole) */
} xn_server_config;
typedef struct {
    uint64_t completed, failed, batches, uploads, evictions, rays, hbm_used;
    double mean_batch;   /* requests per launch (persistent or single-frame) */
    double p50_ms, p99_ms, max_ms; /* submit -> result in host memory */
    double mrays_per_s;  /* rays of completed requests / time from the first submit to the last result */
    uint64_t folded;         /* frames appended to a running or starting persistent kernel */
    uint64_t fold_launches;  /* persistent kernel launches */
    uint64_t republished;    /* frames that reached a ring after its kernel left, appended again */
} xn_server_metrics;

XN_API int xn_server_create(xn_ctx* ctx, const xn_server_config* cfg, xn_server** out);
XN_API int xn_server_destroy(xn_server* server);
/* Register a volume by id; the host copy is kept so the volume can be
 * uploaded again after an eviction. */
XN_API int xn_server_add_grid(xn_server* server, uint32_t volume_id, const uint8_t* rgba, uint32_t dx, uint32_t dy,
                              uint32_t dz);
XN_API int xn_server_add_svo(xn_server* server, uint32_t volume_id, const uint32_t* nodes, uint64_t n_nodes,
                             uint64_t side);
/* Queue a frame; out_rgba (width*height*4 bytes of host memory) must stay
 * valid until xn_server_wait returns for the ticket. */
/* A volume already resident in the server's context (built on the device,
 * loaded from an XNDN-SVC file, ...): the caller keeps owning it, the server
 * counts it against the budget and never evicts or releases it. */
XN_API int xn_server_add_volume(xn_server* server, uint32_t volume_id, xn_volume* volume);
XN_API int xn_server_submit(xn_server* server, uint32_t volume_id, int traversal, const xn_camera* cam,
                            const xn_params* params, uint8_t* out_rgba, uint64_t* ticket);
/* Wait for a ticket (timeout_s < 0: no limit); releases the ticket. */
XN_API int xn_server_wait(xn_server* server, uint64_t ticket, double timeout_s, double* latency_ms);
XN_API int xn_server_stats(xn_server* server, xn_server_metrics* out);

/* Error bits raised by rays since the last call (1 = iteration cap, 2 = stack
 * limit); reset clears them.  Synchronises the context's device. */
XN_API int xn_ray_errors(xn_ctx* ctx, uint32_t* bits, int reset);

/* ------------------------------------------------------------ SVO build --- */

/* Replaces build_octree + Octree::generate_ropes as driven by `xenodon convert`
 * (src/model/OctreeConstruction.h:197-237, src/model/Octree.cpp:181-201,
 * src/convert.cpp:76-85): builds the octree of an RGBA8 grid on the GPU, bit
 * for bit the reference's node array.  *nodes_out is malloc'd host memory
 * (n_nodes*10 u32) that the caller frees with xn_free. */
XN_API int xn_build_svo(xn_ctx* ctx, const uint8_t* rgba, uint32_t dx, uint32_t dy, uint32_t dz,
                        int type, int heuristic, double threshold, uint32_t** nodes_out,
                        xn_build_stats* stats);
XN_API void xn_free(void* p);

/* `xenodon convert` followed by an upload, without leaving the device: builds
 * the octree of a grid in device memory (d_rgba: packed RGBA8 texels, x
 * fastest; a host pointer is copied to the device first) and makes it a
 * resident volume.  The node array is the one xn_build_svo returns.
 *
 * type | XN_BUILD_LEAN (sparse trees only) writes the device layout directly
 * and never holds the 40-byte node array: about 36 bytes per internal node
 * instead of 40 per node plus the layout, so grids whose trees exceed 2^32
 * nodes (the node array's index range) still build, as long as they have
 * fewer than 2^31 internal nodes.  The volume renders every traversal but
 * svo-rope (it has no rope records) with the same results as the full build;
 * the stats are the same as well. */
#define XN_BUILD_LEAN 0x100
XN_API int xn_build_svo_volume(xn_ctx* ctx, const void* d_rgba, uint32_t dx, uint32_t dy, uint32_t dz, int type,
                               int heuristic, double threshold, xn_volume** out, xn_build_stats* stats);

/* Supplies the part of a grid inside a box: nx*ny*nz RGBA8 texels starting at
 * (x0, y0, z0), x fastest, into rgba.  Returns 0, or non-zero to stop the
 * build (which then fails with XN_ERR_IO). */
typedef int (*xn_region_reader)(void* user, uint32_t x0, uint32_t y0, uint32_t z0, uint32_t nx, uint32_t ny,
                                uint32_t nz, uint8_t* rgba);

/* build_octree + save_svo (src/model/OctreeConstruction.h:197-237,
 * src/model/Octree.cpp:96-114) for grids that are never resident on the device
 * as a whole: the sparse octree of a dx*dy*dz grid, built one top-level cube
 * (side/2 on each axis) at a time from the texels `read` supplies, each cube's
 * nodes written to out_path as they are done.  The file is byte-identical to
 * xn_build_svo + xn_svo_save of the whole grid (the reference's node order is
 * the root followed by the eight cubes' own trees, each rebased by the node
 * count before it).  The device holds one cube's grid, build scratch and nodes
 * at a time.  Sparse trees only: ropes and DAG deduplication relate nodes of
 * different cubes.  Fails with XN_ERR_FORMAT past 2^32 nodes (the format's
 * 32-bit indices). */
XN_API int xn_build_svo_streamed(xn_ctx* ctx, uint32_t dx, uint32_t dy, uint32_t dz, int heuristic, double threshold,
                                 xn_region_reader read, void* user, const char* out_path, xn_build_stats* stats);

/* No counterpart in the reference.  The same octree build as xn_build_svo, for
 * callers that cannot allocate device memory: code that runs inside another
 * framework's memory pool or under a fixed HBM budget, and host loops that must
 * not take the device-wide synchronisation cudaMalloc/cudaFree can cause.  It
 * allocates nothing: the grid (d_rgba: dx*dy*dz packed RGBA8 texels, x fastest,
 * 4-byte aligned) and the node buffer (d_nodes: node_capacity nodes of 10 u32,
 * 8-byte aligned) are the caller's device memory, and all scratch comes from one
 * fixed 32 MiB device array that every GPU loading the library holds until the
 * process exits.  A grid whose build needs more scratch than that (about 2
 * million voxels for sparse or rope trees) is rejected with XN_ERR_BUDGET before
 * anything runs.  A DAG's deduplication buffers depend on the node count, so a
 * DAG that outgrows the array is found, and rejected the same way, only after
 * the bottom-up and top-down passes.  A node buffer that is too small is
 * rejected with XN_ERR_ARG and stats->n_nodes set to the size needed.  Work is
 * queued on `stream`, which must belong to the current device (XN_ERR_ARG
 * otherwise), and the call returns once it is done.  The first call on a
 * device, and the first after its context changed (another context made
 * current, or the device reset), looks up the scratch array's device address,
 * so make that first call before any stream capture.  Every call reuses the
 * same array and clears what it needs; calls that overlap on the GPU race. */
XN_API int xn_build_svo_static(const uint32_t* d_rgba, uint32_t dx, uint32_t dy, uint32_t dz, int type,
                               int heuristic, double threshold, uint32_t* d_nodes, uint64_t node_capacity,
                               xn_build_stats* stats, void* stream);

/* --------------------------------------------------------- file formats --- */

/* Octree::load_svo / save_svo (src/model/Octree.cpp:50-114): "XNDN-SVO", u64
 * side, u64 node count, nodes of 10 LE u32.  load returns malloc'd nodes. */
XN_API int xn_svo_load(const char* path, uint32_t** nodes_out, uint64_t* n_nodes, uint64_t* side);
XN_API int xn_svo_save(const char* path, const uint32_t* nodes, uint64_t n_nodes, uint64_t side);

/* The format extension for octrees the reference's format cannot hold (2^32
 * nodes or more; no counterpart in the reference): a resident octree volume's
 * device layout written to disk ("XNDN-SVC", versioned; internal nodes only,
 * 36 bytes each, plus the rope records when the volume has them) and read
 * back straight into HBM.  Both stream through pinned chunks; load validates
 * every index on the device before the volume can be rendered. */
XN_API int xn_volume_save(xn_ctx* ctx, const xn_volume* volume, const char* path);
XN_API int xn_volume_load(xn_ctx* ctx, const char* path, xn_volume** out);

/* Grid::load_tiff (src/model/Grid.cpp:27-79): a stacked TIFF, one page per z
 * slice, read the way TIFFReadRGBAImage hands it to the reference (rows
 * bottom-up, gray expanded to RGB, alpha 255 when absent, unassociated alpha
 * premultiplied).  8-bit gray/RGB/RGBA, strips or tiles, classic TIFF or
 * BigTIFF; uncompressed, LZW, Deflate or PackBits, with or without the
 * horizontal predictor.  *rgba_out is malloc'd (dims[0]*dims[1]*dims[2]*4 bytes,
 * x fastest); free it with xn_free. */
XN_API int xn_tiff_load(const char* path, uint8_t** rgba_out, uint32_t dims_out[3]);
/* Writes a grid as an uncompressed RGBA BigTIFF that xn_tiff_load (and
 * libtiff's TIFFReadRGBAImage) reads back unchanged. */
XN_API int xn_tiff_save(const char* path, const uint8_t* rgba, uint32_t dx, uint32_t dy, uint32_t dz);
/* HeadlessDisplay::save's PNG output (src/backend/headless/HeadlessDisplay.cpp:80-85):
 * width*height RGBA8 pixels, row-major, top row first.  Adaptive scanline
 * filters and deflate (LZ77 + dynamic Huffman codes), the rows compressed in
 * bands on the host's cores. */
XN_API int xn_png_save(const char* path, const uint8_t* rgba, uint32_t width, uint32_t height);

#endif

/*
 * Oracle for the Xenodon volume ray-traversal path -- TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference's five traversal shaders
 * (resources/dda.comp, svo_naive.comp, svo_df.comp, esvo.comp, svo_rope.comp,
 * with resources/common.glsl and resources/octree.glsl) and of the sparse voxel
 * octree build (src/model/OctreeConstruction.h, src/model/Octree.cpp,
 * src/model/Grid.cpp).  It exists to check the CUDA product path and to time a
 * CPU baseline.  Nothing in the product (the C-ABI library, the CLI) links or
 * calls it; only tests, the smoke check and the benchmark's CPU leg do.
 *
 * The restatement is pinned to the reference's own code: the shaders, compiled
 * for the CPU from their sources by oracle/glsl_ref.py, wrote the golden images
 * and per-ray colours of tests/golden/glsl_golden.npz, which this restatement
 * reproduces bit for bit; the octree build is pinned by golden SVO files
 * produced by the reference's own builder compiled from its sources.
 */
#ifndef XO_H
#define XO_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    XO_DDA = 0,
    XO_SVO_NAIVE = 1,
    XO_ESVO = 2,
    XO_SVO_DF = 3,
    XO_SVO_ROPE = 4
};

/* Camera as read from a camera script line (src/camera/Camera.h:6-10). The
 * translation is the raw value; the host-side division by the voxel ratio
 * (src/render/Renderer.cpp:62) happens inside the oracle. */
typedef struct {
    float forward[3];
    float up[3];
    float translation[3];
} xo_camera;

/* UBO contents of resources/common.glsl:29-33 minus model_dim, which is taken
 * from the volume (src/main_loop.cpp:197-201). */
typedef struct {
    int32_t output_offset[2];
    uint32_t output_extent[2];
    int32_t display_offset[2];
    uint32_t display_extent[2];
    float voxel_ratio[3];
    float emission_coeff;
} xo_view;

typedef struct {
    /* uniform grid, RGBA8, x fastest (src/model/Grid.h:50-52) */
    const uint8_t* rgba;
    uint32_t dim[3];
    /* octree: n_nodes x 10 little-endian u32 words (resources/octree.glsl:6-10) */
    const uint32_t* nodes;
    uint64_t n_nodes;
} xo_volume;

/* Per-ray error bits; rays that set one of them left the reference's defined
 * behaviour (an endless loop or an overflowing stack in the shader). */
enum {
    XO_ERR_ITER = 1,
    XO_ERR_STACK = 2,
    XO_ERR_INDEX = 4
};

/*
 * Render one output region.  Any output pointer may be NULL.
 *   out_rgba      extent.x*extent.y*4 bytes, row-major
 *   out_emission  extent.x*extent.y*3 floats (doubles for _f64): the colour
 *                 after the emission coefficient, before clamping
 *   out_loads     extent.x*extent.y u32: 32-bit words the shader reads per ray
 *                 (texels for DDA, node words for the octree shaders)
 *   out_err       extent.x*extent.y u8 error bits
 * Returns the number of rays with error bits, or -1 on bad arguments.
 */
int64_t xo_render_f32(int traversal, const xo_volume* vol, const xo_camera* cam,
                      const xo_view* view, uint8_t* out_rgba, float* out_emission,
                      uint32_t* out_loads, uint8_t* out_err, int nthreads);
int64_t xo_render_f64(int traversal, const xo_volume* vol, const xo_camera* cam,
                      const xo_view* view, uint8_t* out_rgba, double* out_emission,
                      uint32_t* out_loads, uint8_t* out_err, int nthreads);

/* ---- octree build (src/model/OctreeConstruction.h) ---- */

enum { XO_TYPE_SPARSE = 0, XO_TYPE_DAG = 1, XO_TYPE_ROPE = 2 };
enum { XO_HEUR_CHANNEL_DIFF = 0, XO_HEUR_STD_DEV = 1 };

typedef struct {
    uint64_t total_leaves;
    uint64_t unique_leaves;
    uint64_t total_nodes;
    uint64_t depth;
    uint64_t side;
    uint64_t n_nodes;
} xo_build_stats;

/* Builds the octree into a malloc'd array of n_nodes*10 u32 words that the
 * caller releases with xo_free.  Returns 0 on success. */
int xo_build_svo(const uint8_t* rgba, const uint32_t dim[3], int type, int heuristic,
                 double threshold, uint32_t** nodes_out, xo_build_stats* stats);
void xo_free(void* p);

#ifdef __cplusplus
}
#endif

#endif

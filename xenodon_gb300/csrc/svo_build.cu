// GPU octree build (src/model/OctreeConstruction.h) -- argument checks only
// until the level-by-level builder lands.
#include <cstdint>
#include "../../include/xenodon.h"
#include "xn_ctx.h"

using xn::fail;

XN_API int xn_build_svo(xn_ctx* ctx, const uint8_t* rgba, uint32_t dx, uint32_t dy, uint32_t dz, int type,
                        int heuristic, double threshold, uint32_t** nodes_out, xn_build_stats* stats) {
    if (!ctx || !rgba || !nodes_out || !stats) return fail(XN_ERR_ARG, "xn_build_svo: NULL argument");
    (void)dx; (void)dy; (void)dz; (void)type; (void)heuristic; (void)threshold;
    return fail(XN_ERR_STATE, "xn_build_svo: not available in this build");
}

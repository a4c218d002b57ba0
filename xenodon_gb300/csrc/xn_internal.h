// Internal interfaces between the C-ABI layer and the CUDA kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace xn {

enum {
    XN_TRAV_DDA = 0,
    XN_TRAV_SVO_NAIVE = 1,
    XN_TRAV_ESVO = 2,
    XN_TRAV_SVO_DF = 3,
    XN_TRAV_SVO_ROPE = 4
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
    const void* grid;   // uchar4 texels, x fastest (DDA)
    uint32_t dim[3];
    const void* nodes;  // reference node words (octree traversals)
    // outputs (device pointers)
    void* d_rgba;
    float* d_emission;
    uint32_t* d_loads;
    uint32_t* d_err_word;
};

cudaError_t launch_render(const RenderLaunch& launch, cudaStream_t stream);

}  // namespace xn

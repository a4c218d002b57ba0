// Block-wide exclusive prefix sums of small counts into u32, used by the
// octree build (DAG ranks) and the device octree layout (node renumbering).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace xn {
namespace scan {


constexpr int SCAN_T = 256;
constexpr int SCAN_ITEMS = 16;
constexpr uint64_t SCAN_CHUNK = (uint64_t)SCAN_T * SCAN_ITEMS;

__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v) {
    __shared__ unsigned warp_sums[SCAN_T / 32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned incl = v;
    for (int o = 1; o < 32; o <<= 1) {
        unsigned t = __shfl_up_sync(0xFFFFFFFFu, incl, o);
        if (lane >= (unsigned)o) incl += t;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < SCAN_T / 32 ? warp_sums[lane] : 0u;
        unsigned wi = w;
        for (int o = 1; o < 32; o <<= 1) {
            unsigned t = __shfl_up_sync(0xFFFFFFFFu, wi, o);
            if (lane >= (unsigned)o) wi += t;
        }
        if (lane < SCAN_T / 32) warp_sums[lane] = wi - w;
    }
    __syncthreads();
    return warp_sums[warp] + incl - v;
}

template <class In>
__global__ void scan_reduce_kernel(const In* in, uint64_t n, unsigned* block_sums) {
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_CHUNK + (uint64_t)threadIdx.x * SCAN_ITEMS;
    unsigned s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j)
        if (base + j < n) s += (unsigned)in[base + j];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xFFFFFFFFu, s, o);
    __shared__ unsigned ws[SCAN_T / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = 0;
        for (int w = 0; w < SCAN_T / 32; ++w) t += ws[w];
        block_sums[blockIdx.x] = t;
    }
}

template <class In>
__global__ void scan_apply_kernel(const In* in, uint64_t n, const unsigned* block_offsets, unsigned* out) {
    const uint64_t base = (uint64_t)blockIdx.x * SCAN_CHUNK + (uint64_t)threadIdx.x * SCAN_ITEMS;
    unsigned v[SCAN_ITEMS];
    unsigned s = 0;
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        v[j] = base + j < n ? (unsigned)in[base + j] : 0u;
        s += v[j];
    }
    unsigned run = block_exclusive_scan(s) + (block_offsets ? block_offsets[blockIdx.x] : 0u);
#pragma unroll
    for (int j = 0; j < SCAN_ITEMS; ++j) {
        if (base + j < n) out[base + j] = run;
        run += v[j];
    }
}


}  // namespace scan
}  // namespace xn

// Host-side state behind the opaque xn_ctx / xn_volume handles.
#pragma once

#include <atomic>
#include <cstdint>
#include <mutex>

#include <cuda_runtime.h>

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
    std::mutex mu;

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
};

int fail(int code, const char* fmt, ...) __attribute__((format(printf, 2, 3)));
int cuda_fail(cudaError_t e, const char* what);

}  // namespace xn

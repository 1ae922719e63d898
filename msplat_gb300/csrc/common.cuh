// Shared helpers for the sm_103a rasteriser kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include <utility>

#include "msplat_gb300.h"

namespace msplat {

constexpr int kTile = 16;  // 16x16-pixel tiles (reference config.h:7-8)
constexpr int kTilePixels = kTile * kTile;

// Records the detail message for msplat_last_error() and returns `code`.
int set_error(int code, const char *fmt, ...);

inline int check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return set_error(MSPLAT_ERR_LAUNCH, "%s: %s", what, cudaGetErrorString(e));
    return MSPLAT_OK;
}

__host__ __device__ inline int ceil_div(int a, int b) { return (a + b - 1) / b; }
__host__ __device__ inline int64_t ceil_div64(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Counts one kernel launch (read back by msplat_kernel_launches()).
void note_launch();

// Every kernel of the library is launched through here so that the launch
// count is exact.
template <typename... KArgs, typename... Args>
inline void launch(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                   Args &&...args) {
    note_launch();
    kernel<<<grid, block, smem, stream>>>(std::forward<Args>(args)...);
}

// Number of SMs of the current device (cached per device).
int num_sms();

// Carves aligned sub-buffers out of a caller-provided workspace.
struct Workspace {
    char *base;
    size_t size;
    size_t used = 0;
    bool overflow = false;
    Workspace(void *p, size_t n) : base((char *)p), size(n) {}
    template <typename T>
    T *take(size_t count) {
        size_t off = (used + 255) & ~size_t(255);
        size_t bytes = count * sizeof(T);
        if (off + bytes > size || (base == nullptr && bytes > 0)) {
            overflow = true;
            used = off + bytes;
            return nullptr;
        }
        used = off + bytes;
        return reinterpret_cast<T *>(base + off);
    }
};

// Same carving arithmetic without a buffer, for *_workspace_size queries.
struct WorkspaceSizer {
    size_t used = 0;
    template <typename T>
    void take(size_t count) {
        size_t off = (used + 255) & ~size_t(255);
        used = off + count * sizeof(T);
    }
};

// Tile rectangle covered by a circle of integer radius around p, clamped to
// the grid: [min, max) in tile units.  The float operations and their order
// are those of the reference's get_rect (msplat/include/utils.h:17-36), so
// the rectangle -- and with it tiles_touched and the key list -- is
// bit-identical: lo = trunc((p - r) / 16), hi = trunc(((p + r) + 16 - 1) / 16)
// (three separate float roundings), both clamped to [0, grid].
__device__ __forceinline__ void tile_rect(float px, float py, int r, int gx,
                                          int gy, int &x0, int &y0, int &x1,
                                          int &y1) {
    const float fr = (float)r;
    const float inv = 1.0f / (float)kTile;  // exact power of two
    x0 = min(gx, max(0, (int)(__fsub_rn(px, fr) * inv)));
    y0 = min(gy, max(0, (int)(__fsub_rn(py, fr) * inv)));
    x1 = min(gx, max(0, (int)(__fsub_rn(__fadd_rn(__fadd_rn(px, fr), (float)kTile), 1.0f) * inv)));
    y1 = min(gy, max(0, (int)(__fsub_rn(__fadd_rn(__fadd_rn(py, fr), (float)kTile), 1.0f) * inv)));
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace msplat

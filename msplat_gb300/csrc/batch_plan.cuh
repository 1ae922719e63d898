// The layout of a multi-camera batch (one key space over all cameras).
//
// A batch renders B cameras, each of a scene of P_b Gaussians, in one set
// of launches.  Per-camera per-Gaussian arrays (uv, depth, conic, radius,
// tiles, colour and their gradients) are stacked camera after camera:
// camera b's rows start at row_off_b = sum of P over the cameras before
// it.  Tiles are numbered globally (camera b's tiles start at tile_off_b),
// and so are pixels (final T, contributor counts; images add a factor of C
// per pixel): camera b's image is [C, H_b, W_b] at C * pix_off_b.
// Opacity (and shared features) are indexed per scene: camera b reads
// opacity[op_off_b + g].
//
// The plan is built on the host (msplat_batch_plan) and copied to the
// device by the caller; kernels read it from device memory.
#pragma once

#include "common.cuh"

namespace msplat {

struct BatchCam {               // 64 bytes
    int32_t W, H, gx, gy;       // image and tile grid
    int32_t P;                  // Gaussians of the camera's scene
    int32_t tile_off;           // first global tile
    int32_t dtile;              // first sort tile of the camera's depth-key segment
    int32_t pad0;
    int64_t row_off;            // first row in the stacked per-camera arrays
    int64_t op_off;             // first row of the scene in opacity / shared features
    int64_t pix_off;            // first global pixel
    int64_t pad1;
};

// Plan blob: BatchCam[B], then int32 dtile_start[B + 1] (depth segments, in
// sort tiles), int64 dcount[B] (= P_b), int32 tile_start[B + 1] (global tile
// offsets, the last = total tiles).
struct BatchPlanView {
    const BatchCam *cams;
    const int32_t *dtile_start;
    const int64_t *dcount;
    const int32_t *tile_start;
    int B;
};

__host__ __device__ inline size_t batch_plan_off_dtile(int B) { return (size_t)B * sizeof(BatchCam); }
__host__ __device__ inline size_t batch_plan_off_dcount(int B) {
    return (batch_plan_off_dtile(B) + (size_t)(B + 1) * 4 + 7) & ~(size_t)7;
}
__host__ __device__ inline size_t batch_plan_off_tiles(int B) { return batch_plan_off_dcount(B) + (size_t)B * 8; }
__host__ __device__ inline size_t batch_plan_bytes(int B) { return batch_plan_off_tiles(B) + (size_t)(B + 1) * 4; }

inline BatchPlanView batch_plan_view(const void *plan, int B) {
    const char *p = static_cast<const char *>(plan);
    return {reinterpret_cast<const BatchCam *>(p), reinterpret_cast<const int32_t *>(p + batch_plan_off_dtile(B)),
            reinterpret_cast<const int64_t *>(p + batch_plan_off_dcount(B)),
            reinterpret_cast<const int32_t *>(p + batch_plan_off_tiles(B)), B};
}

// Largest i in [0, n) with start[i] <= v, for a non-decreasing start[0..n]
// with start[0] <= v < start[n].
__device__ __forceinline__ int upper_index(const int32_t *__restrict__ start, int n, int64_t v) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (start[mid] <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The camera of global tile t.
__device__ __forceinline__ int batch_camera_of_tile(const BatchPlanView &pv, int t) {
    return upper_index(pv.tile_start, pv.B, t);
}

}  // namespace msplat

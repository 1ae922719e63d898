// Tile/depth ordering of the Gaussian-tile intersections.
//
// The reference (msplat/sort_gaussian.py:41-52) scans tiles_touched, writes
// one 64-bit key (tile << 32 | depth bits) per intersection in Gaussian
// order (msplat/src/sort_gaussian.cu:17-43), sorts all keys with
// torch.sort, gathers the ids, and finds tile boundaries (:45-71).
//
// Two paths produce exactly the reference's idx_sorted and tile_range:
//
// * reference layout -- the same key array (including the zero keys of
//   slots nobody fills), a stable signed-int64 LSD radix sort, and boundary
//   detection.  Mirrors the reference step by step; used when the caller's
//   tiles[] disagree with the rectangles (zero slots exist).
//
// * fast path -- since a stable sort by (tile, depth) equals a stable sort
//   by tile of a list already in depth order, Gaussians are first sorted by
//   depth (P keys, 32 bits), their intersections emitted in that order, and
//   the I intersections sorted by tile only (ceil(log2(tiles + 1)) bits,
//   2 passes at 1080p instead of 6-8 over 64-bit keys).  Depth keys are the
//   float bits with the sign bit flipped, i.e. signed-int32 order, matching
//   the reference's sign-extended keys; negative-depth Gaussians get tile
//   key 0 so they lead idx_sorted and stay out of every tile's range, as in
//   the reference (which writes their range out of bounds; we skip that).
#include "radix_sort.cuh"

namespace msplat {

// --------------------------------------------------------- reference layout
__global__ void __launch_bounds__(256)
gaussian_key_kernel(int P, const float2 *__restrict__ uv, const float *__restrict__ depth,
                    const int32_t *__restrict__ radius, const int32_t *__restrict__ cumsum,
                    int gx, int gy, int64_t I, int64_t *__restrict__ keys,
                    int32_t *__restrict__ idx) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= P || radius[g] <= 0) return;
    int x0, y0, x1, y1;
    const float2 p = uv[g];
    tile_rect(p.x, p.y, radius[g], gx, gy, x0, y0, x1, y1);
    int64_t cur = g == 0 ? 0 : cumsum[g - 1];
    const int64_t dk = (int64_t)__float_as_int(depth[g]);  // sign-extended
    for (int ty = y0; ty < y1; ++ty)
        for (int tx = x0; tx < x1; ++tx) {
            if (cur >= 0 && cur < I) {  // the reference does not bound this
                keys[cur] = ((int64_t)(ty * gx + tx) << 32) | dk;
                idx[cur] = g;
            }
            ++cur;
        }
}

__global__ void __launch_bounds__(256)
range_from_i64_kernel(int64_t I, const int64_t *__restrict__ keys, int ntiles,
                      int2 *__restrict__ range) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= I) return;
    const int t = (int)(keys[i] >> 32);
    const bool ok = t >= 0 && t < ntiles;
    if (i == 0 || (int)(keys[i - 1] >> 32) != t) {
        if (ok) range[t].x = (int)i;
    }
    if (i == I - 1 || (int)(keys[i + 1] >> 32) != t) {
        if (ok) range[t].y = (int)(i + 1);
    }
}

// --------------------------------------------------------------- fast path
// Depth key: sign-flipped float bits (signed-int32 order).  Gaussians that
// emit nothing sort last.
__global__ void __launch_bounds__(256)
depth_key_kernel(int P, const float *__restrict__ depth, const int32_t *__restrict__ radius,
                 uint32_t *__restrict__ keys) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= P) return;
    keys[g] = radius[g] > 0 ? (__float_as_uint(depth[g]) ^ 0x80000000u) : 0xffffffffu;
}

// Tile count of each Gaussian, in depth order; counts Gaussians whose tiles[]
// entry disagrees with the rectangle (these need the reference layout).
__global__ void __launch_bounds__(256)
depth_order_count_kernel(int P, const uint32_t *__restrict__ order, const float2 *__restrict__ uv,
                         const int32_t *__restrict__ radius, const int32_t *__restrict__ tiles,
                         int gx, int gy, int32_t *__restrict__ cnt, int64_t *__restrict__ counts) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = false;
    if (j < P) {
        const int g = (int)order[j];
        int c = 0;
        if (radius[g] > 0) {
            int x0, y0, x1, y1;
            const float2 p = uv[g];
            tile_rect(p.x, p.y, radius[g], gx, gy, x0, y0, x1, y1);
            c = (x1 - x0) * (y1 - y0);
        }
        bad = c != tiles[g];
        cnt[j] = c;
    }
    const unsigned m = __ballot_sync(0xffffffffu, bad);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd((unsigned long long *)&counts[1], (unsigned long long)__popc(m));
}

// Emits the intersections of 32 depth-ordered Gaussians per warp; each
// Gaussian's run is written by all lanes (coalesced).
__global__ void __launch_bounds__(256)
emit_kernel(int P, const uint32_t *__restrict__ order, const int32_t *__restrict__ offs,
            const float2 *__restrict__ uv, const float *__restrict__ depth,
            const int32_t *__restrict__ radius, int gx, int gy, uint32_t *__restrict__ tkeys,
            uint32_t *__restrict__ tvals) {
    const int lane = threadIdx.x & 31;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    int g = -1, x0 = 0, y0 = 0, x1 = 0, y1 = 0, start = 0;
    bool neg = false;
    if (j < P) {
        g = (int)order[j];
        if (radius[g] > 0) {
            const float2 p = uv[g];
            tile_rect(p.x, p.y, radius[g], gx, gy, x0, y0, x1, y1);
            start = offs[j];
            neg = (__float_as_uint(depth[g]) >> 31) != 0;
        } else {
            x1 = x0;  // empty
        }
    }
    for (int s = 0; s < 32; ++s) {
        const int sg = __shfl_sync(0xffffffffu, g, s);
        const int sx0 = __shfl_sync(0xffffffffu, x0, s), sy0 = __shfl_sync(0xffffffffu, y0, s);
        const int sx1 = __shfl_sync(0xffffffffu, x1, s), sy1 = __shfl_sync(0xffffffffu, y1, s);
        const int sstart = __shfl_sync(0xffffffffu, start, s);
        const bool sneg = __shfl_sync(0xffffffffu, (int)neg, s) != 0;
        if (sg < 0) continue;
        const int w = sx1 - sx0;
        const int count = w * (sy1 - sy0);
        for (int k = lane; k < count; k += 32) {
            const int ty = sy0 + k / w, tx = sx0 + k % w;
            tkeys[sstart + k] = sneg ? 0u : (uint32_t)(ty * gx + tx + 1);
            tvals[sstart + k] = (uint32_t)sg;
        }
    }
}

// Ranges from tile keys (key 0 = no tile, key t + 1 = tile t).
__global__ void __launch_bounds__(256)
range_from_tilekey_kernel(int64_t I, const uint32_t *__restrict__ keys, int2 *__restrict__ range) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= I) return;
    const uint32_t k = keys[i];
    if (k == 0) return;
    const int t = (int)k - 1;
    if (i == 0 || keys[i - 1] != k) range[t].x = (int)i;
    if (i == I - 1 || keys[i + 1] != k) range[t].y = (int)(i + 1);
}

inline int bits_for(uint32_t maxval) {
    int b = 0;
    while (b < 32 && (maxval >> b) != 0) ++b;
    return b;
}

constexpr int kDepthPasses = 4;

// Prepare-step workspace.  `order` and `offs` come first and are read again
// by the finish step (which re-derives their addresses from P).
struct PrepareWs {
    uint32_t *order = nullptr;  // [P] Gaussian ids in depth order
    int32_t *offs = nullptr;    // [P] exclusive scan of tile counts, depth order
    int32_t *cnt = nullptr;     // [P]
    uint32_t *ka = nullptr, *kb = nullptr, *vt = nullptr;
    int64_t *scan_parts = nullptr;
    RadixBuffers rb{};
};

inline void prepare_carve(Workspace &w, int P, PrepareWs &ws) {
    ws.order = w.take<uint32_t>(P);
    ws.offs = w.take<int32_t>(P);
    ws.cnt = w.take<int32_t>(P);
    ws.ka = w.take<uint32_t>(P);
    ws.kb = w.take<uint32_t>(P);
    ws.vt = w.take<uint32_t>(P);
    ws.scan_parts = w.take<int64_t>((size_t)ceil_div(P, kScanTile) + 1);
    radix_take(w, P, kDepthPasses, ws.rb);
}

inline size_t prepare_bytes(int P) {
    WorkspaceSizer s;
    s.take<uint32_t>(P); s.take<int32_t>(P); s.take<int32_t>(P);
    s.take<uint32_t>(P); s.take<uint32_t>(P); s.take<uint32_t>(P);
    s.take<int64_t>((size_t)ceil_div(P, kScanTile) + 1);
    radix_size(s, P, kDepthPasses);
    return s.used;
}

inline int tile_key_passes(int W, int H) {
    const int ntiles = ceil_div(W, kTile) * ceil_div(H, kTile);
    const int bits = bits_for((uint32_t)ntiles);  // keys span [0, ntiles]
    return ceil_div(bits > 0 ? bits : 1, kRadixBits);
}

inline size_t finish_bytes(int64_t I, int W, int H) {
    WorkspaceSizer s;
    s.take<uint32_t>(I); s.take<uint32_t>(I); s.take<uint32_t>(I);
    radix_size(s, I, tile_key_passes(W, H));
    return s.used;
}

inline size_t radix_i64_bytes(int64_t n) {
    WorkspaceSizer s;
    s.take<uint64_t>(n);
    s.take<uint32_t>(n);
    radix_size(s, n, 8);
    return s.used;
}

}  // namespace msplat

using namespace msplat;

extern "C" int msplat_compute_gaussian_key(int P, const float *uv, const float *depth, int W,
                                           int H, const int32_t *radius,
                                           const int32_t *tiles_cumsum, int64_t num_intersects,
                                           int64_t *key, int32_t *idx, msplat_stream_t stream) {
    if (P < 0 || W <= 0 || H <= 0 || num_intersects < 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_gaussian_key: bad sizes");
    if (num_intersects > 0) {
        if (!key || !idx)
            return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_gaussian_key: null output");
        cudaMemsetAsync(key, 0, sizeof(int64_t) * num_intersects, stream);
        cudaMemsetAsync(idx, 0, sizeof(int32_t) * num_intersects, stream);
    }
    if (P == 0 || num_intersects == 0) return check_launch("compute_gaussian_key");
    if (!uv || !depth || !radius || !tiles_cumsum)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_gaussian_key: null pointer");
    const int gx = ceil_div(W, kTile), gy = ceil_div(H, kTile);
    gaussian_key_kernel<<<ceil_div(P, 256), 256, 0, stream>>>(P, (const float2 *)uv, depth, radius,
                                                              tiles_cumsum, gx, gy, num_intersects,
                                                              key, idx);
    return check_launch("compute_gaussian_key");
}

extern "C" int msplat_compute_tile_gaussian_range(int W, int H, int64_t num_intersects,
                                                  const int64_t *key_sorted, int32_t *tile_range,
                                                  msplat_stream_t stream) {
    if (W <= 0 || H <= 0 || num_intersects < 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_tile_gaussian_range: bad sizes");
    const int ntiles = ceil_div(W, kTile) * ceil_div(H, kTile);
    if (!tile_range)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_tile_gaussian_range: null output");
    cudaMemsetAsync(tile_range, 0, sizeof(int32_t) * 2 * ntiles, stream);
    if (num_intersects > 0) {
        if (!key_sorted)
            return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "compute_tile_gaussian_range: null keys");
        range_from_i64_kernel<<<(unsigned)ceil_div64(num_intersects, 256), 256, 0, stream>>>(
            num_intersects, key_sorted, ntiles, (int2 *)tile_range);
    }
    return check_launch("compute_tile_gaussian_range");
}

extern "C" size_t msplat_scan_workspace_size(int n) {
    WorkspaceSizer s;
    scan_size(s, n < 0 ? 0 : n);
    return s.used;
}

extern "C" int msplat_inclusive_scan_i32(int n, const int32_t *in, int32_t *out, int64_t *total,
                                         void *workspace, size_t workspace_bytes,
                                         msplat_stream_t stream) {
    if (n < 0) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "inclusive_scan_i32: n < 0");
    if (n > 0 && (!in || !out))
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "inclusive_scan_i32: null pointer");
    Workspace w(workspace, workspace_bytes);
    int64_t *parts = w.take<int64_t>((size_t)ceil_div(n, kScanTile) + 1);
    if (w.overflow)
        return set_error(MSPLAT_ERR_WORKSPACE, "inclusive_scan_i32: workspace of %zu bytes < %zu",
                         workspace_bytes, msplat_scan_workspace_size(n));
    return scan_i32(n, in, out, true, total, parts, stream);
}

extern "C" size_t msplat_radix_sort_i64_workspace_size(int64_t n) {
    return radix_i64_bytes(n < 0 ? 0 : n);
}

extern "C" int msplat_radix_sort_i64_pairs(int64_t n, const int64_t *keys_in, const int32_t *vals_in,
                                           int64_t *keys_out, int32_t *vals_out, int begin_bit,
                                           int end_bit, void *workspace, size_t workspace_bytes,
                                           msplat_stream_t stream) {
    if (n < 0 || begin_bit < 0 || end_bit > 64 || begin_bit > end_bit)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "radix_sort_i64_pairs: bad n or bit range");
    if (n == 0) return MSPLAT_OK;
    if (n > INT32_MAX) return set_error(MSPLAT_ERR_CAPACITY, "radix_sort_i64_pairs: n > 2^31 - 1");
    if (!keys_in || !keys_out || !vals_out)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "radix_sort_i64_pairs: null pointer");
    const int passes = ceil_div(end_bit - begin_bit, kRadixBits);
    if (passes == 0) {
        cudaMemcpyAsync(keys_out, keys_in, sizeof(int64_t) * n, cudaMemcpyDeviceToDevice, stream);
        return check_launch("radix_sort_i64_pairs");
    }
    Workspace w(workspace, workspace_bytes);
    uint64_t *kt = w.take<uint64_t>(n);
    uint32_t *vt = w.take<uint32_t>(n);
    RadixBuffers rb;
    if (!radix_take(w, n, passes, rb))
        return set_error(MSPLAT_ERR_WORKSPACE, "radix_sort_i64_pairs: workspace of %zu bytes < %zu",
                         workspace_bytes, msplat_radix_sort_i64_workspace_size(n));
    return radix_sort_pairs<uint64_t, true>(n, begin_bit, passes, (const uint64_t *)keys_in,
                                            (const uint32_t *)vals_in, (uint64_t *)keys_out,
                                            (uint32_t *)vals_out, kt, vt, rb, stream);
}

extern "C" size_t msplat_sort_prepare_workspace_size(int P) { return prepare_bytes(P < 0 ? 0 : P); }

extern "C" int msplat_sort_gaussian_prepare(int P, const float *depth, const int32_t *radius,
                                            const int32_t *tiles, const float *uv, int W, int H,
                                            int64_t *counts, void *workspace, size_t workspace_bytes,
                                            msplat_stream_t stream) {
    if (P < 0 || W <= 0 || H <= 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_prepare: bad sizes");
    if (!counts) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_prepare: null counts");
    cudaMemsetAsync(counts, 0, 2 * sizeof(int64_t), stream);
    if (P == 0) return check_launch("sort_gaussian_prepare");
    if (!depth || !radius || !tiles || !uv)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_prepare: null pointer");
    Workspace w(workspace, workspace_bytes);
    PrepareWs ws;
    prepare_carve(w, P, ws);
    if (w.overflow)
        return set_error(MSPLAT_ERR_WORKSPACE, "sort_gaussian_prepare: workspace of %zu bytes < %zu",
                         workspace_bytes, prepare_bytes(P));
    const int gx = ceil_div(W, kTile), gy = ceil_div(H, kTile);
    depth_key_kernel<<<ceil_div(P, 256), 256, 0, stream>>>(P, depth, radius, ws.ka);
    // Even pass count: the input keys may alias the output keys.
    int st = radix_sort_pairs<uint32_t, false>(P, 0, kDepthPasses, ws.ka, nullptr, ws.ka, ws.order,
                                               ws.kb, ws.vt, ws.rb, stream);
    if (st) return st;
    depth_order_count_kernel<<<ceil_div(P, 256), 256, 0, stream>>>(
        P, ws.order, (const float2 *)uv, radius, tiles, gx, gy, ws.cnt, counts);
    return scan_i32(P, ws.cnt, ws.offs, false, counts, ws.scan_parts, stream);
}

extern "C" size_t msplat_sort_finish_workspace_size(int P, int64_t num_intersects, int W, int H) {
    (void)P;
    if (W <= 0 || H <= 0 || num_intersects < 0) return 0;
    return finish_bytes(num_intersects, W, H);
}

extern "C" int msplat_sort_gaussian_finish(int P, const float *uv, const float *depth,
                                           const int32_t *radius, int W, int H,
                                           int64_t num_intersects, const void *prepare_workspace,
                                           int32_t *idx_sorted, int32_t *tile_range, void *workspace,
                                           size_t workspace_bytes, msplat_stream_t stream) {
    if (P < 0 || W <= 0 || H <= 0 || num_intersects < 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_finish: bad sizes");
    if (num_intersects > INT32_MAX)
        return set_error(MSPLAT_ERR_CAPACITY, "sort_gaussian_finish: %lld intersections exceed int32",
                         (long long)num_intersects);
    const int gx = ceil_div(W, kTile), gy = ceil_div(H, kTile), ntiles = gx * gy;
    if (!tile_range) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_finish: null tile_range");
    cudaMemsetAsync(tile_range, 0, sizeof(int32_t) * 2 * ntiles, stream);
    if (P == 0 || num_intersects == 0) return check_launch("sort_gaussian_finish");
    if (!uv || !depth || !radius || !prepare_workspace || !idx_sorted)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_finish: null pointer");
    Workspace pw(const_cast<void *>(prepare_workspace), prepare_bytes(P));
    PrepareWs prep;
    prepare_carve(pw, P, prep);
    const int64_t I = num_intersects;
    const int passes = tile_key_passes(W, H);
    Workspace w(workspace, workspace_bytes);
    uint32_t *ka = w.take<uint32_t>(I), *kb = w.take<uint32_t>(I), *vt = w.take<uint32_t>(I);
    RadixBuffers rb;
    radix_take(w, I, passes, rb);
    if (w.overflow)
        return set_error(MSPLAT_ERR_WORKSPACE, "sort_gaussian_finish: workspace of %zu bytes < %zu",
                         workspace_bytes, finish_bytes(I, W, H));
    // Even pass count: emit the ids straight into idx_sorted (input may alias
    // output); odd: emit into the temporary (input may alias tmp).
    uint32_t *out = (uint32_t *)idx_sorted;
    uint32_t *vemit = (passes % 2 == 0) ? out : vt;
    emit_kernel<<<ceil_div(P, 256), 256, 0, stream>>>(P, prep.order, prep.offs, (const float2 *)uv,
                                                      depth, radius, gx, gy, ka, vemit);
    int st = radix_sort_pairs<uint32_t, false>(I, 0, passes, ka, vemit, (passes % 2 == 0) ? ka : kb, out,
                                               (passes % 2 == 0) ? kb : ka, vt, rb, stream);
    if (st) return st;
    const uint32_t *sorted_keys = (passes % 2 == 0) ? ka : kb;
    range_from_tilekey_kernel<<<(unsigned)ceil_div64(I, 256), 256, 0, stream>>>(I, sorted_keys,
                                                                               (int2 *)tile_range);
    return check_launch("sort_gaussian_finish");
}

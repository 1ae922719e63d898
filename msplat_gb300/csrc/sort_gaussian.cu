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
// * fast path -- a stable sort by (tile, depth) equals a stable sort by
//   tile of a list already in depth order.  So the P Gaussians are sorted by
//   depth once (32-bit keys: the float bits with the sign flipped, i.e. the
//   reference's signed order; ties keep id order), their intersections are
//   emitted in that order with coalesced writes, and the I intersections are
//   stable-sorted by tile only: ceil(log2(tiles + 1)) bits, 2 passes at
//   1080p instead of 6-8 over 64-bit keys.  Negative-depth Gaussians, whose
//   sign-extended keys the reference sorts first and keeps out of every
//   range, get tile key 0 so they lead idx_sorted in depth order as there
//   (the reference writes their range out of bounds; we skip that write).
#include "cull.cuh"
#include "emit.cuh"
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

// Tile counts of the Gaussians in depth order, summed per block of 256
// (the block layout emit_kernel uses): bsum[block].  Also counts Gaussians
// whose tiles[] entry disagrees with their rectangle (those need the
// reference layout), the negative-depth emitters (they come first in depth
// order) and their intersections.
// With conic and opacity (the culled lists of the fused path) each
// rectangle is first shrunk by shrink_rect and, on images of at least
// kRowCutMinTiles tiles, each of its rows then cut to the columns the
// ellipse reaches there (row_span); negative-depth
// Gaussians (which no tile range includes) emit nothing; the rectangle and
// the reach are stored in depth order in rects[j] and reach[j] for
// emit_kernel, which evaluates the same spans.
__global__ void __launch_bounds__(256)
depth_order_count_kernel(int P, const uint32_t *__restrict__ order, const float2 *__restrict__ uv,
                         const float *__restrict__ depth, const int32_t *__restrict__ radius,
                         const int32_t *__restrict__ tiles, const float *__restrict__ conic,
                         const float *__restrict__ opacity, int gx, int gy, int64_t *__restrict__ bsum,
                         int64_t *__restrict__ counts, unsigned long long *__restrict__ neg,
                         short4 *__restrict__ rects, RowReach *__restrict__ reach) {
    __shared__ int64_t scratch[33];
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    bool bad = false, isneg = false;
    int c = 0;
    if (j < P) {
        const int g = (int)order[j];
        int x0 = 0, y0 = 0, x1 = 0, y1 = 0, cref = 0;
        if ((unsigned)g < (unsigned)P && radius[g] > 0) {  // (an id outside [0, P) is never read)
            const float2 p = uv[g];
            tile_rect(p.x, p.y, radius[g], gx, gy, x0, y0, x1, y1);
            cref = (x1 - x0) * (y1 - y0);
            // Sign-bit-set depths sort before all others (signed order).
            isneg = (__float_as_uint(depth[g]) >> 31) != 0;
            if (conic) {
                if (isneg) {
                    x1 = x0;
                    y1 = y0;
                } else {
                    const float ca = conic[3 * g], cb = conic[3 * g + 1], cc = conic[3 * g + 2], op = opacity[g];
                    shrink_rect(p.x, p.y, ca, cb, cc, op, x0, y0, x1, y1);
                    if (row_cut_enabled(gx, gy)) {
                        const RowReach rr = row_reach(p.x, p.y, ca, cb, cc, op, x0, y0, x1, y1);
                        reach[j] = rr;
                        c = row_span_count(rr, x0, y0, x1, y1);
                    } else {
                        c = (x1 - x0) * (y1 - y0);
                    }
                }
            }
            if (!conic || isneg) c = (x1 - x0) * (y1 - y0);
            if (isneg && c > 0) atomicAdd(neg + 1, (unsigned long long)c);
        }
        if (conic) rects[j] = make_short4((short)x0, (short)y0, (short)x1, (short)y1);
        bad = (unsigned)g < (unsigned)P && cref != tiles[g];
    }
    const unsigned mb = __ballot_sync(0xffffffffu, bad), mn = __ballot_sync(0xffffffffu, isneg);
    if ((threadIdx.x & 31) == 0) {
        if (mb) atomicAdd((unsigned long long *)&counts[1], (unsigned long long)__popc(mb));
        if (mn) atomicAdd(neg, (unsigned long long)__popc(mn));
    }
    int64_t total;
    block_exclusive_scan<int64_t>((int64_t)c, scratch, &total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// Exclusive scan of the nb block sums in place (one block), and the total:
// the number of intersections, written to counts[0].
__global__ void __launch_bounds__(1024)
block_offsets_kernel(int nb, int64_t *__restrict__ bsum, int64_t *__restrict__ counts) {
    __shared__ int64_t scratch[33];
    int64_t carry = 0;
    for (int c0 = 0; c0 < nb; c0 += blockDim.x) {
        const int i = c0 + threadIdx.x;
        const int64_t v = i < nb ? bsum[i] : 0;
        int64_t tot;
        const int64_t ex = block_exclusive_scan<int64_t>(v, scratch, &tot);
        if (i < nb) bsum[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) counts[0] = carry;
}

// Calls f(tile) for every tile of the rectangle of depth-ordered Gaussian j.
template <typename F>
__device__ __forceinline__ void for_rect_tiles(int g, const float2 *__restrict__ uv,
                                               const int32_t *__restrict__ radius, int gx, int gy, F &&f) {
    const int r = radius[g];
    if (r <= 0) return;
    int x0, y0, x1, y1;
    const float2 p = uv[g];
    tile_rect(p.x, p.y, r, gx, gy, x0, y0, x1, y1);
    for (int ty = y0; ty < y1; ++ty)
        for (int tx = x0; tx < x1; ++tx) f(ty * gx + tx);
}

// Emits the intersections of 256 depth-ordered Gaussians per block: each
// thread loads one Gaussian, then the block writes all their runs of
// (tile key, id) pairs together with coalesced stores (emit_block_runs).
// Tile key 0 marks negative-depth Gaussians, t + 1 tile t.
// A Gaussian's first slot is its block's base (boff, from the block sums)
// plus the exclusive scan of the tile counts within the block.
// With *culled set (by a culled prepare) the rectangles come from
// rects[j]; on images of at least kRowCutMinTiles tiles the reaches from
// reach[j], each row cut to its span (emit_block_rows), where `total` (or
// *total_dev when given, the device count) bounds the last block's slots.
__global__ void __launch_bounds__(256)
emit_kernel(int P, const uint32_t *__restrict__ order, const int64_t *__restrict__ boff,
            const float2 *__restrict__ uv, const float *__restrict__ depth,
            const int32_t *__restrict__ radius, const short4 *__restrict__ rects, const int *__restrict__ culled,
            const RowReach *__restrict__ reach, int gx, int gy, uint32_t *__restrict__ tkeys,
            uint32_t *__restrict__ tvals, int64_t cap, int64_t total, const int64_t *__restrict__ total_dev) {
    __shared__ union {
        EmitShared runs;
        EmitRowShared rows;
    } sm;
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    int g = -1, x0 = 0, y0 = 0, x1 = 0, y1 = 0;
    bool neg = false;
    if (*culled && row_cut_enabled(gx, gy)) {  // rows cut to the ellipse's reach (as the count kernel)
        RowReach rr{};
        if (j < P) {
            g = (int)order[j];
            const short4 r = rects[j];
            x0 = r.x;
            y0 = r.y;
            x1 = r.z;
            y1 = r.w;
            if (x0 < x1 && y0 < y1) rr = reach[j];
        }
        if (total_dev) total = min(total, *total_dev);
        const int64_t next = blockIdx.x + 1 < gridDim.x ? boff[blockIdx.x + 1] : total;
        emit_block_rows(sm.rows, boff[blockIdx.x], next - boff[blockIdx.x], j < P, rr, x0, y0, x1, y1, g, gx, tkeys,
                        tvals, cap);
        return;
    }
    if (j < P) {
        g = (int)order[j];
        if (*culled) {
            const short4 r = rects[j];
            x0 = r.x;
            y0 = r.y;
            x1 = r.z;
            y1 = r.w;
        } else if ((unsigned)g < (unsigned)P && radius[g] > 0) {
            const float2 p = uv[g];
            tile_rect(p.x, p.y, radius[g], gx, gy, x0, y0, x1, y1);
            neg = (__float_as_uint(depth[g]) >> 31) != 0;
        }
    }
    const int w = x1 - x0, n = w * (y1 - y0);
    // Offsets stay 64-bit: with a capacity-bounded finish the true count (and
    // so boff) may pass 2^31 while only the first `cap` slots exist.
    emit_block_runs(sm.runs, boff[blockIdx.x], n, g, x0, y0, w, neg, gx, tkeys, tvals, cap);
}

// Ranges from the sorted tile keys (key 0 = no tile, key t + 1 = tile t).
// Each thread reads 8 consecutive keys with two 16-byte loads (keys is
// 16-byte aligned) plus one neighbour on each side; a boundary between
// different keys writes the end of one tile's range and the start of the
// next.  0xffffffff (never a key) stands for "outside the array".
constexpr int kRangeKeys = 8;

__global__ void __launch_bounds__(256)
range_from_tilekey_kernel(int64_t I, const uint32_t *__restrict__ keys, int ntiles, int2 *__restrict__ range,
                          const int64_t *__restrict__ I_dev) {
    if (I_dev) I = min(I, *I_dev);  // the length is on the device; I is the capacity
    const int64_t i0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * kRangeKeys;
    if (i0 >= I) return;
    constexpr uint32_t kOut = 0xffffffffu;
    uint32_t k[kRangeKeys + 2];
    k[0] = i0 > 0 ? keys[i0 - 1] : kOut;
    if (i0 + kRangeKeys <= I) {
        const uint4 a = reinterpret_cast<const uint4 *>(keys + i0)[0];
        const uint4 b = reinterpret_cast<const uint4 *>(keys + i0)[1];
        k[1] = a.x; k[2] = a.y; k[3] = a.z; k[4] = a.w;
        k[5] = b.x; k[6] = b.y; k[7] = b.z; k[8] = b.w;
    } else {
#pragma unroll
        for (int u = 0; u < kRangeKeys; ++u) k[u + 1] = i0 + u < I ? keys[i0 + u] : kOut;
    }
    k[kRangeKeys + 1] = i0 + kRangeKeys < I ? keys[i0 + kRangeKeys] : kOut;
#pragma unroll
    for (int u = 1; u <= kRangeKeys; ++u) {
        const uint32_t key = k[u];
        if (key == 0 || key > (uint32_t)ntiles) continue;  // (kOut too)
        const int64_t i = i0 + u - 1;
        if (k[u - 1] != key) range[key - 1].x = (int)i;
        if (k[u + 1] != key) range[key - 1].y = (int)(i + 1);
    }
}
inline int bits_for(uint32_t maxval) {
    int b = 0;
    while (b < 32 && (maxval >> b) != 0) ++b;
    return b;
}

constexpr int kDepthPasses = 4;

// Prepare-step workspace.  `order`, `offs`, `cnt` and the negative-depth
// counters come first and are read again by the finish step (which
// re-derives their addresses from P).
struct PrepareWs {
    uint32_t *order = nullptr;  // [P] Gaussian ids in depth order
    int64_t *bsum = nullptr;    // [P/256] tile counts per block of 256 in depth order, then their scan
    unsigned long long *neg = nullptr;  // [0] negative emitters, [1] their intersections
    short4 *rects = nullptr;    // [P] rectangles in depth order (culled prepare)
    RowReach *reach = nullptr;  // [P] per-row reach parameters in depth order (culled prepare)
    int *culled = nullptr;      // [1] nonzero after a culled prepare
    uint32_t *ka = nullptr, *kb = nullptr, *vt = nullptr;
    RadixBuffers rb{};
};

template <typename WS>
inline void prepare_carve(WS &w, int P, PrepareWs &ws) {
    ws.order = w.template take<uint32_t>(P);
    ws.bsum = w.template take<int64_t>((size_t)ceil_div(P, 256));
    ws.neg = w.template take<unsigned long long>(2);
    ws.rects = w.template take<short4>(P);
    ws.reach = w.template take<RowReach>(P);
    ws.culled = w.template take<int>(1);
    ws.ka = w.template take<uint32_t>(P);
    ws.kb = w.template take<uint32_t>(P);
    ws.vt = w.template take<uint32_t>(P);
    radix_carve(w, sort_tiles(P), 1, kDepthPasses, ws.rb);
}

struct SizeOnly {
    WorkspaceSizer s;
    template <typename T> T *take(size_t n) { s.take<T>(n); return nullptr; }
};

inline size_t prepare_bytes(int P) {
    SizeOnly z;
    PrepareWs ws;
    prepare_carve(z, P, ws);
    return z.s.used;
}

inline int tile_key_passes(int W, int H) {
    const int ntiles = ceil_div(W, kTile) * ceil_div(H, kTile);
    const int bits = bits_for((uint32_t)ntiles);  // keys span [0, ntiles]
    return ceil_div(bits > 0 ? bits : 1, kRadixBits);
}

struct FinishWs {
    uint32_t *ka = nullptr, *kb = nullptr, *vt = nullptr;
    RadixBuffers rb{};
};

template <typename WS>
inline void finish_carve(WS &w, int64_t I, int passes, FinishWs &f) {
    f.ka = w.template take<uint32_t>(I);
    f.kb = w.template take<uint32_t>(I);
    f.vt = w.template take<uint32_t>(I);
    radix_carve(w, sort_tiles(I), 1, passes, f.rb);
}

inline size_t finish_bytes(int64_t I, int W, int H) {
    SizeOnly z;
    FinishWs f;
    finish_carve(z, I, tile_key_passes(W, H), f);
    return z.s.used;
}

template <typename WS>
inline void radix_i64_carve(WS &w, int64_t n, int passes, uint64_t *&kt, uint32_t *&vt, RadixBuffers &rb) {
    kt = w.template take<uint64_t>(n);
    vt = w.template take<uint32_t>(n);
    radix_carve(w, sort_tiles(n), 1, passes, rb);
}

inline size_t radix_i64_bytes(int64_t n) {
    SizeOnly z;
    uint64_t *kt;
    uint32_t *vt;
    RadixBuffers rb;
    radix_i64_carve(z, n, 8, kt, vt, rb);
    return z.s.used;
}

}  // namespace msplat

namespace msplat {
static int g_sort_onesweep = 0;  // three launches per pass: measured faster on the tile lists (see the header)
bool sort_onesweep_enabled() { return g_sort_onesweep != 0; }
cudaError_t sort_wait_error_single(int reset, int *value, cudaStream_t stream) {
    return sort_wait_error_read(reset, value, stream);
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
    launch(gaussian_key_kernel, ceil_div(P, 256), 256, 0, stream, P, (const float2 *)uv, depth, radius,
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
        launch(range_from_i64_kernel, (unsigned)ceil_div64(num_intersects, 256), 256, 0, stream,
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

// ---------------------------------------------------- allocation-free scan
// Scratch of msplat_inclusive_scan_i32_noalloc: the partial sums of a scan of
// up to MSPLAT_SCAN_NOALLOC_MAX_N elements, one int64 per 4096-element tile
// plus one (131 KB).  Host code cannot use the symbol as a device address;
// noalloc_scan_parts() looks the address up.
constexpr int kNoAllocScanParts = MSPLAT_SCAN_NOALLOC_MAX_N / kScanTile + 1;
static __device__ __align__(256) int64_t g_noalloc_scan_parts[kNoAllocScanParts];

// Device address of g_noalloc_scan_parts in the current context, looked up
// on every call (no allocation; a cached address would go stale when a
// device reset reloads the module).
static int64_t *noalloc_scan_parts(cudaError_t *err) {
    void *p = nullptr;
    *err = cudaGetSymbolAddress(&p, g_noalloc_scan_parts);
    return *err == cudaSuccess ? static_cast<int64_t *>(p) : nullptr;
}

extern "C" int msplat_inclusive_scan_i32_noalloc(int n, const int32_t *in, int32_t *out, int64_t *total,
                                                 msplat_stream_t stream) {
    if (n < 0) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "inclusive_scan_i32_noalloc: n < 0");
    if (n > MSPLAT_SCAN_NOALLOC_MAX_N)
        return set_error(MSPLAT_ERR_CAPACITY,
                         "inclusive_scan_i32_noalloc: n = %d exceeds the maximum of %d elements of its "
                         "built-in scratch; use msplat_inclusive_scan_i32 with a workspace",
                         n, MSPLAT_SCAN_NOALLOC_MAX_N);
    if (n > 0 && (!in || !out))
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "inclusive_scan_i32_noalloc: null pointer");
    cudaError_t err = cudaSuccess;
    int64_t *parts = noalloc_scan_parts(&err);
    if (!parts)
        return set_error(MSPLAT_ERR_LAUNCH, "inclusive_scan_i32_noalloc: device address of the scratch: %s",
                         cudaGetErrorString(err));
    // Every partial sum is written by scan_reduce_kernel before it is read,
    // so the shared scratch needs no clearing between calls.
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
    uint64_t *kt;
    uint32_t *vt;
    RadixBuffers rb;
    radix_i64_carve(w, n, 8, kt, vt, rb);  // sized for 8 passes, as the size query
    if (w.overflow)
        return set_error(MSPLAT_ERR_WORKSPACE, "radix_sort_i64_pairs: workspace of %zu bytes < %zu",
                         workspace_bytes, msplat_radix_sort_i64_workspace_size(n));
    return radix_sort_pairs<uint64_t, true>(n, begin_bit, passes, (const uint64_t *)keys_in,
                                            (const uint32_t *)vals_in, (uint64_t *)keys_out,
                                            (uint32_t *)vals_out, kt, vt, rb, stream);
}

extern "C" size_t msplat_sort_prepare_workspace_size(int P, int W, int H) {
    (void)W; (void)H;
    return prepare_bytes(P < 0 ? 0 : P);
}

static int prepare_impl(int P, const float *depth, const int32_t *radius, const int32_t *tiles, const float *uv,
                        const float *conic, const float *opacity, int W, int H, int64_t *counts, void *workspace,
                        size_t workspace_bytes, cudaStream_t stream) {
    if (P < 0 || W <= 0 || H <= 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_prepare: bad sizes");
    if (conic && (ceil_div(W, kTile) > 32767 || ceil_div(H, kTile) > 32767))  // rects hold int16 tile indices
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_prepare_culled: grid of %d x %d tiles too large",
                         ceil_div(W, kTile), ceil_div(H, kTile));
    if (!counts) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_prepare: null counts");
    Workspace w(workspace, workspace_bytes);
    PrepareWs ws;
    prepare_carve(w, P, ws);
    if (w.overflow)
        return set_error(MSPLAT_ERR_WORKSPACE, "sort_gaussian_prepare: workspace of %zu bytes < %zu",
                         workspace_bytes, prepare_bytes(P));
    cudaMemsetAsync(counts, 0, 2 * sizeof(int64_t), stream);
    cudaMemsetAsync(ws.neg, 0, 2 * sizeof(unsigned long long), stream);
    cudaMemsetAsync(ws.culled, conic ? 0xff : 0, sizeof(int), stream);
    if (P == 0) return check_launch("sort_gaussian_prepare");
    if (!depth || !radius || !tiles || !uv)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_prepare: null pointer");
    const int gx = ceil_div(W, kTile), gy = ceil_div(H, kTile);
    launch(depth_key_kernel, ceil_div(P, 256), 256, 0, stream, P, depth, radius, ws.ka);
    // Even pass count: the input keys may alias the output keys.
    int st = radix_sort_pairs<uint32_t, false>(P, 0, kDepthPasses, ws.ka, nullptr, ws.ka, ws.order,
                                               ws.kb, ws.vt, ws.rb, stream);
    if (st) return st;
    const int nb = ceil_div(P, 256);
    launch(depth_order_count_kernel, nb, 256, 0, stream,
        P, ws.order, (const float2 *)uv, depth, radius, tiles, conic, opacity, gx, gy, ws.bsum, counts, ws.neg,
        ws.rects, ws.reach);
    launch(block_offsets_kernel, 1, 1024, 0, stream, nb, ws.bsum, counts);
    return check_launch("sort_gaussian_prepare");
}

extern "C" int msplat_sort_gaussian_prepare(int P, const float *depth, const int32_t *radius,
                                            const int32_t *tiles, const float *uv, int W, int H,
                                            int64_t *counts, void *workspace, size_t workspace_bytes,
                                            msplat_stream_t stream) {
    return prepare_impl(P, depth, radius, tiles, uv, nullptr, nullptr, W, H, counts, workspace, workspace_bytes,
                        stream);
}

extern "C" int msplat_sort_gaussian_prepare_culled(int P, const float *depth, const int32_t *radius,
                                                   const int32_t *tiles, const float *uv, const float *conic,
                                                   const float *opacity, int W, int H, int64_t *counts,
                                                   void *workspace, size_t workspace_bytes,
                                                   msplat_stream_t stream) {
    if (P > 0 && (!conic || !opacity))
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_prepare_culled: null conic / opacity");
    return prepare_impl(P, depth, radius, tiles, uv, conic, opacity, W, H, counts, workspace, workspace_bytes,
                        stream);
}

extern "C" size_t msplat_sort_finish_workspace_size(int P, int64_t num_intersects, int W, int H) {
    (void)P;
    if (W <= 0 || H <= 0 || num_intersects < 0) return 0;
    return finish_bytes(num_intersects, W, H);
}

// Emit, two tile-key passes and ranges.  I is the intersection count, or
// with I_dev the capacity of the buffers and I_dev the device-side count
// (entries past the capacity are dropped).
static int finish_impl(int P, const float *uv, const float *depth, const int32_t *radius, int W, int H, int64_t I,
                       const int64_t *I_dev, const void *prepare_workspace, int32_t *idx_sorted,
                       int32_t *tile_range, void *workspace, size_t workspace_bytes, cudaStream_t stream) {
    if (P < 0 || W <= 0 || H <= 0 || I < 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_finish: bad sizes");
    if (I > INT32_MAX)
        return set_error(MSPLAT_ERR_CAPACITY, "sort_gaussian_finish: %lld intersections exceed int32", (long long)I);
    const int gx = ceil_div(W, kTile), gy = ceil_div(H, kTile), nt = gx * gy;
    if (!tile_range) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_finish: null tile_range");
    cudaMemsetAsync(tile_range, 0, sizeof(int32_t) * 2 * nt, stream);
    if (P == 0 || I == 0) return check_launch("sort_gaussian_finish");
    if (!uv || !depth || !radius || !prepare_workspace || !idx_sorted)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_finish: null pointer");
    if (((uintptr_t)idx_sorted & 15) != 0)  // the emit writes it with 16-byte stores
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_finish: idx_sorted is not 16-byte aligned");
    Workspace pw(const_cast<void *>(prepare_workspace), prepare_bytes(P));
    PrepareWs prep;
    prepare_carve(pw, P, prep);
    const int passes = tile_key_passes(W, H);
    Workspace w(workspace, workspace_bytes);
    FinishWs f;
    finish_carve(w, I, passes, f);
    if (w.overflow)
        return set_error(MSPLAT_ERR_WORKSPACE, "sort_gaussian_finish: workspace of %zu bytes < %zu",
                         workspace_bytes, finish_bytes(I, W, H));
    // Even pass count: emit the ids straight into idx_sorted (the input may
    // alias the output); odd: into the temporary (the input may alias tmp).
    uint32_t *out = (uint32_t *)idx_sorted;
    const bool even = passes % 2 == 0;
    uint32_t *vemit = even ? out : f.vt;
    launch(emit_kernel, ceil_div(P, 256), 256, 0, stream, P, prep.order, prep.bsum, (const float2 *)uv, depth,
           radius, (const short4 *)prep.rects, (const int *)prep.culled, (const RowReach *)prep.reach, gx, gy, f.ka,
           vemit, I, I, I_dev);
    uint32_t *kout = even ? f.ka : f.kb;
    // the last pass meets only the digits of keys up to ntiles (5 bits of 8 at 1920 x 1080)
    const int last_bits = max(1, bits_for((uint32_t)nt)) - kRadixBits * (passes - 1);
    int st = radix_sort_pairs<uint32_t, false>(I, 0, passes, f.ka, vemit, kout, out, even ? f.kb : f.ka, f.vt,
                                               f.rb, stream, I_dev, last_bits);
    if (st) return st;
    launch(range_from_tilekey_kernel, (unsigned)ceil_div64(ceil_div64(I, kRangeKeys), 256), 256, 0, stream, I, kout,
           nt, (int2 *)tile_range, I_dev);
    return check_launch("sort_gaussian_finish");
}

// status = 1 when the results of a capacity-bounded finish are not valid:
// more intersections than the capacity, or tiles[] entries that disagree
// with the rectangles (those need the reference-layout sort).
__global__ void capacity_status_kernel(const int64_t *__restrict__ counts, int64_t cap, int32_t *__restrict__ status) {
    status[0] = (counts[0] > cap || counts[1] != 0) ? 1 : 0;
}

extern "C" int msplat_sort_gaussian_finish(int P, const float *uv, const float *depth,
                                           const int32_t *radius, int W, int H,
                                           int64_t num_intersects, const void *prepare_workspace,
                                           int32_t *idx_sorted, int32_t *tile_range, void *workspace,
                                           size_t workspace_bytes, msplat_stream_t stream) {
    return finish_impl(P, uv, depth, radius, W, H, num_intersects, nullptr, prepare_workspace, idx_sorted,
                       tile_range, workspace, workspace_bytes, stream);
}

extern "C" int msplat_sort_gaussian_finish_capacity(int P, const float *uv, const float *depth,
                                                    const int32_t *radius, int W, int H, int64_t capacity,
                                                    const int64_t *counts, const void *prepare_workspace,
                                                    int32_t *idx_sorted, int32_t *tile_range, int32_t *status,
                                                    void *workspace, size_t workspace_bytes,
                                                    msplat_stream_t stream) {
    if (!counts || !status)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_finish_capacity: null counts / status");
    if (capacity < 0) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "sort_gaussian_finish_capacity: capacity < 0");
    launch(capacity_status_kernel, 1, 1, 0, stream, counts, capacity, status);
    return finish_impl(P, uv, depth, radius, W, H, capacity, counts, prepare_workspace, idx_sorted, tile_range,
                       workspace, workspace_bytes, stream);
}

extern "C" int msplat_set_sort_onesweep(int on) {
    g_sort_onesweep = on ? 1 : 0;
    return MSPLAT_OK;
}

// Multi-camera tile sort in one key space: the intersections of every
// camera of a batch ordered by (camera, tile, depth) with one set of
// launches.  No counterpart in the reference, which sorts one camera per
// call (msplat/sort_gaussian.py:8-54, called from msplat/__init__.py:70-93).
//
// Per camera the order is the single-camera fast path's (and so the
// reference's order restricted to the culled lists): Gaussians sorted by
// depth (stable, ties by id), intersections emitted in that order, then
// stably sorted by tile.  Batched:
//   prepare  depth keys and culled rectangles of every camera's Gaussians
//            in one array of padded segments (one per camera), one
//            segmented 4-pass radix sort, the rectangles and tile counts
//            gathered into depth order, block offsets scanned per camera
//            (one block per camera), and the camera segments of the
//            intersection list (each padded to a sort tile) -- all on the
//            device;
//   finish   emit every camera's (local tile + 1, Gaussian) pairs into its
//            segment, one segmented radix sort by local tile (2 passes at
//            1080p), and the tile ranges in the global tile numbering.
// The finish takes a capacity (the padded list length it may use) and the
// counts from device memory, so a batch needs at most one host read (the
// padded length) and none with a caller-given capacity.
#include <cstring>

#include "batch_plan.cuh"
#include "cull.cuh"
#include "emit.cuh"
#include "radix_sort.cuh"

namespace msplat {

constexpr int kBatchDepthPasses = 4;
constexpr int kBlocksPerSortTile = kSortTile / 256;

// Depth keys of every camera's Gaussians in its padded segment (sign-flipped
// float bits; Gaussians that emit nothing sort last), their culled
// rectangles, per-row reaches and kept-tile counts in the same layout (as
// the single-camera culled prepare: negative depths emit nothing,
// rectangles shrunk by shrink_rect, each row cut to row_span).  Rows are
// read in order here, so the count after the depth sort gathers one
// 16-byte record per Gaussian instead of its projected values.
struct BatchRect {
    short4 rect;
    int count;  // tiles the per-row reach keeps
    int pad;
};

__global__ void __launch_bounds__(256)
batch_key_rect_kernel(BatchPlanView pv, int64_t n, const float2 *__restrict__ uv, const float *__restrict__ depth,
                      const int32_t *__restrict__ radius, const float *__restrict__ conic,
                      const float *__restrict__ opacity, uint32_t *__restrict__ keys, BatchRect *__restrict__ rects,
                      RowReach *__restrict__ reach) {
    const int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= n) return;
    const int b = upper_index(pv.dtile_start, pv.B, pos / kSortTile);
    const BatchCam &c = pv.cams[b];
    const int64_t j = pos - (int64_t)pv.dtile_start[b] * kSortTile;
    if (j >= c.P) return;  // padding: never read by the segmented sort or the count
    const int64_t q = c.row_off + j;
    const int rad = radius[q];
    const float d = depth[q];
    keys[pos] = rad > 0 ? (__float_as_uint(d) ^ 0x80000000u) : 0xffffffffu;
    int x0 = 0, y0 = 0, x1 = 0, y1 = 0, cnt = 0;
    if (rad > 0 && (__float_as_uint(d) >> 31) == 0) {
        const float2 p = uv[q];
        const float ca = conic[3 * q], cb = conic[3 * q + 1], cc = conic[3 * q + 2], op = opacity[c.op_off + j];
        tile_rect(p.x, p.y, rad, c.gx, c.gy, x0, y0, x1, y1);
        shrink_rect(p.x, p.y, ca, cb, cc, op, x0, y0, x1, y1);
        if (x0 < x1 && y0 < y1) {
            if (row_cut_enabled(c.gx, c.gy)) {
                const RowReach rr = row_reach(p.x, p.y, ca, cb, cc, op, x0, y0, x1, y1);
                reach[pos] = rr;
                cnt = row_span_count(rr, x0, y0, x1, y1);
            } else {
                cnt = (x1 - x0) * (y1 - y0);
            }
        }
    }
    rects[pos] = BatchRect{make_short4((short)x0, (short)y0, (short)x1, (short)y1), cnt, 0};
}

// The culled rectangles and kept-tile counts of every camera's Gaussians in
// depth order (gathered from the position layout of
// batch_key_rect_kernel); the sum per block of 256 (blocks never straddle
// cameras: segments are padded to sort tiles of 12 blocks).
__global__ void __launch_bounds__(256)
batch_count_kernel(BatchPlanView pv, const uint32_t *__restrict__ order, const BatchRect *__restrict__ rect_at,
                   short4 *__restrict__ rects, int64_t *__restrict__ bsum) {
    __shared__ int64_t scratch[33];
    const int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int b = upper_index(pv.dtile_start, pv.B, (int64_t)blockIdx.x / kBlocksPerSortTile);
    const BatchCam &c = pv.cams[b];
    const int64_t s0 = (int64_t)pv.dtile_start[b] * kSortTile;
    BatchRect r{make_short4(0, 0, 0, 0), 0, 0};
    if (pos - s0 < c.P) {
        const uint32_t g = order[pos];
        if (g < (uint32_t)c.P) r = rect_at[s0 + g];  // (an id outside the camera's rows is never read)
    }
    rects[pos] = r.rect;
    int64_t total;
    block_exclusive_scan<int64_t>((int64_t)r.count, scratch, &total);
    if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// One block per camera: exclusive scan of its block sums in place and its
// intersection count.
__global__ void __launch_bounds__(1024)
batch_block_offsets_kernel(BatchPlanView pv, int64_t *__restrict__ bsum, int64_t *__restrict__ cam_count) {
    __shared__ int64_t scratch[33];
    const int b = blockIdx.x;
    const int64_t k0 = (int64_t)pv.dtile_start[b] * kBlocksPerSortTile;
    const int64_t k1 = (int64_t)pv.dtile_start[b + 1] * kBlocksPerSortTile;
    int64_t carry = 0;
    for (int64_t c0 = k0; c0 < k1; c0 += blockDim.x) {
        const int64_t i = c0 + threadIdx.x;
        const int64_t v = i < k1 ? bsum[i] : 0;
        int64_t tot;
        const int64_t ex = block_exclusive_scan<int64_t>(v, scratch, &tot);
        if (i < k1) bsum[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) cam_count[b] = carry;
}

// The camera segments of the intersection list (sort tiles, padded) and the
// counts the caller reads: counts[0] = intersections, counts[1] = padded
// length (the capacity a finish needs), counts[2 + b] = camera b's.
__global__ void __launch_bounds__(256)
batch_layout_kernel(int B, const int64_t *__restrict__ cam_count, int32_t *__restrict__ fin_start,
                    int64_t *__restrict__ counts) {
    if (threadIdx.x != 0) return;
    int64_t tiles = 0, total = 0;
    for (int b = 0; b < B; ++b) {
        fin_start[b] = (int32_t)min(tiles, (int64_t)INT32_MAX);
        tiles += ceil_div64(cam_count[b], kSortTile);
        total += cam_count[b];
        counts[2 + b] = cam_count[b];
    }
    fin_start[B] = (int32_t)min(tiles, (int64_t)INT32_MAX);
    counts[0] = total;
    counts[1] = tiles * kSortTile;
}

// The finish's segments clipped to a capacity of ntiles sort tiles (only
// ever smaller when the capacity is exceeded, and then status = 1).
__global__ void __launch_bounds__(256)
batch_finish_segs_kernel(int B, int ntiles, const int32_t *__restrict__ fin_start,
                         const int64_t *__restrict__ cam_count, int32_t *__restrict__ seg_start,
                         int64_t *__restrict__ seg_count, int32_t *__restrict__ status) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b <= B) seg_start[b] = min(fin_start[b], ntiles);
    if (b < B) {
        const int64_t room = (int64_t)(ntiles - min(fin_start[b], ntiles)) * kSortTile;
        seg_count[b] = max((int64_t)0, min(cam_count[b], room));
    }
    if (b == 0 && status) status[0] = fin_start[B] > ntiles ? 1 : 0;
}

// Emits each camera's (local tile + 1, Gaussian id) pairs into its segment,
// in depth order, as the culled emit_kernel: on cameras of at least
// kRowCutMinTiles tiles each rectangle's rows cut to their spans
// (emit_block_rows, on the reach batch_key_rect_kernel recorded), whole
// rectangles otherwise (emit_block_runs); nothing at or past the capacity
// `cap`, nor past the slots the count gave the block.
__global__ void __launch_bounds__(256)
batch_emit_kernel(BatchPlanView pv, const uint32_t *__restrict__ order, const short4 *__restrict__ rects,
                  const RowReach *__restrict__ reach_at, const int64_t *__restrict__ boff,
                  const int64_t *__restrict__ cam_count, const int32_t *__restrict__ seg_start,
                  uint32_t *__restrict__ tkeys, uint32_t *__restrict__ tvals, int64_t cap) {
    __shared__ union {
        EmitShared runs;
        EmitRowShared rows;
    } sm;
    const int64_t pos = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int b = upper_index(pv.dtile_start, pv.B, (int64_t)blockIdx.x / kBlocksPerSortTile);
    const BatchCam &c = pv.cams[b];
    const int64_t s0 = (int64_t)pv.dtile_start[b] * kSortTile;
    const int64_t j = pos - s0;
    const bool cut = row_cut_enabled(c.gx, c.gy);  // the same for the whole block (one camera)
    int g = 0;
    short4 r = make_short4(0, 0, 0, 0);
    RowReach rr{};
    if (j < c.P) {
        g = (int)order[pos];
        r = rects[pos];
        if (cut && r.x < r.z && r.y < r.w) rr = reach_at[s0 + g];  // (a non-empty rectangle has a valid id)
    }
    if (!cut) {
        const int w = r.z - r.x, n = w * (r.w - r.y);
        emit_block_runs(sm.runs, (int64_t)seg_start[b] * kSortTile + boff[blockIdx.x], n, g, r.x, r.y, w, false,
                        c.gx, tkeys, tvals, cap);
        return;
    }
    // the block's slots: up to the next block of the camera, or its count
    const int64_t last_block = (int64_t)pv.dtile_start[b + 1] * kBlocksPerSortTile - 1;
    const int64_t next = (int64_t)blockIdx.x < last_block ? boff[blockIdx.x + 1] : cam_count[b];
    emit_block_rows(sm.rows, (int64_t)seg_start[b] * kSortTile + boff[blockIdx.x], next - boff[blockIdx.x], j < c.P, rr,
                    r.x, r.y, r.z, r.w, g, c.gx, tkeys, tvals, cap);
}

// Tile ranges in the global tile numbering from the sorted segments: each
// thread reads 8 keys of one camera's segment (segments start on sort
// tiles, so the 8 never straddle two) with a neighbour on each side; a
// neighbour outside the segment's items counts as "outside".
__global__ void __launch_bounds__(256)
batch_range_kernel(BatchPlanView pv, int ntiles, const int32_t *__restrict__ seg_start,
                   const int64_t *__restrict__ seg_count, const uint32_t *__restrict__ keys,
                   int2 *__restrict__ range) {
    constexpr int K = 8;
    const int64_t i0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * K;
    if (i0 >= (int64_t)ntiles * kSortTile) return;
    const int st = (int)(i0 / kSortTile);
    if (st >= seg_start[pv.B]) return;
    const int b = upper_index(seg_start, pv.B, st);
    const int64_t s0 = (int64_t)seg_start[b] * kSortTile, s1 = s0 + seg_count[b];
    if (i0 >= s1) return;
    constexpr uint32_t kOut = 0xffffffffu;
    uint32_t k[K + 2];
#pragma unroll
    for (int u = -1; u <= K; ++u) {
        const int64_t i = i0 + u;
        k[u + 1] = (i >= s0 && i < s1) ? keys[i] : kOut;
    }
    const int toff = pv.cams[b].tile_off;
    const uint32_t nkeys = (uint32_t)(pv.cams[b].gx * pv.cams[b].gy);  // keys of the camera: [1, nkeys]
#pragma unroll
    for (int u = 1; u <= K; ++u) {
        const uint32_t key = k[u];
        if (key == 0 || key > nkeys) continue;  // (kOut too)
        const int64_t i = i0 + u - 1;
        if (k[u - 1] != key) range[toff + key - 1].x = (int)i;
        if (k[u + 1] != key) range[toff + key - 1].y = (int)(i + 1);
    }
}

struct BatchPrepareWs {
    uint32_t *ka, *kb, *vt, *order;
    short4 *rects;
    BatchRect *rect_at;
    RowReach *reach_at;
    int64_t *bsum, *cam_count;
    int32_t *fin_start;
    RadixBuffers rb;
};

template <typename WS>
inline void batch_prepare_carve(WS &w, int B, int64_t dn, BatchPrepareWs &ws) {
    ws.ka = w.template take<uint32_t>(dn);
    ws.kb = w.template take<uint32_t>(dn);
    ws.vt = w.template take<uint32_t>(dn);
    ws.order = w.template take<uint32_t>(dn);
    ws.rects = w.template take<short4>(dn);
    ws.rect_at = w.template take<BatchRect>(dn);
    ws.reach_at = w.template take<RowReach>(dn);
    ws.bsum = w.template take<int64_t>((size_t)(dn / 256));
    ws.cam_count = w.template take<int64_t>(B);
    ws.fin_start = w.template take<int32_t>(B + 1);
    radix_carve(w, dn / kSortTile, B, kBatchDepthPasses, ws.rb);
}

struct BatchFinishWs {
    uint32_t *ka, *kb, *vt;
    RadixBuffers rb;
    int32_t *seg_start;
    int64_t *seg_count;
};

template <typename WS>
inline void batch_finish_carve(WS &w, int B, int64_t cap, int passes, BatchFinishWs &f) {
    f.ka = w.template take<uint32_t>(cap);
    f.kb = w.template take<uint32_t>(cap);
    f.vt = w.template take<uint32_t>(cap);
    radix_carve(w, cap / kSortTile, B, passes, f.rb);
    f.seg_start = w.template take<int32_t>(B + 1);
    f.seg_count = w.template take<int64_t>(B);
}

struct SizeOnlyB {
    WorkspaceSizer s;
    template <typename T> T *take(size_t n) { s.take<T>(n); return nullptr; }
};

inline int batch_tile_passes(int max_tiles) {
    int bits = 0;
    while (bits < 32 && ((uint32_t)max_tiles >> bits) != 0) ++bits;  // keys span [1, max_tiles]
    return ceil_div(bits > 0 ? bits : 1, kRadixBits);
}

}  // namespace msplat

namespace msplat {
cudaError_t sort_wait_error_batch(int reset, int *value, cudaStream_t stream) {
    return sort_wait_error_read(reset, value, stream);
}
}  // namespace msplat

using namespace msplat;

extern "C" size_t msplat_batch_plan_bytes(int B) { return B > 0 ? batch_plan_bytes(B) : 0; }

extern "C" int msplat_batch_plan(int B, const int32_t *dims, const int32_t *npoints, const int64_t *opacity_offset,
                                 void *plan, size_t plan_bytes, int64_t *sizes) {
    if (B <= 0 || !dims || !npoints || !plan || !sizes)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_plan: B = %d or a null pointer", B);
    if (plan_bytes < batch_plan_bytes(B))
        return set_error(MSPLAT_ERR_WORKSPACE, "batch_plan: %zu bytes < %zu", plan_bytes, batch_plan_bytes(B));
    char *p = static_cast<char *>(plan);
    memset(p, 0, batch_plan_bytes(B));
    BatchCam *cams = reinterpret_cast<BatchCam *>(p);
    int32_t *dstart = reinterpret_cast<int32_t *>(p + batch_plan_off_dtile(B));
    int64_t *dcount = reinterpret_cast<int64_t *>(p + batch_plan_off_dcount(B));
    int32_t *tstart = reinterpret_cast<int32_t *>(p + batch_plan_off_tiles(B));
    int64_t rows = 0, pix = 0, dt = 0, tiles = 0;
    int max_tiles = 1;
    for (int b = 0; b < B; ++b) {
        const int W = dims[2 * b], H = dims[2 * b + 1], P = npoints[b];
        if (W <= 0 || H <= 0 || P < 0)
            return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_plan: camera %d has W=%d H=%d P=%d", b, W, H, P);
        BatchCam &c = cams[b];
        c.W = W;
        c.H = H;
        c.gx = ceil_div(W, kTile);
        c.gy = ceil_div(H, kTile);
        if (c.gx > 32767 || c.gy > 32767)
            return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_plan: camera %d grid too large", b);
        c.P = P;
        c.tile_off = (int32_t)tiles;
        c.dtile = (int32_t)dt;
        c.row_off = rows;
        c.op_off = opacity_offset ? opacity_offset[b] : 0;
        c.pix_off = pix;
        dstart[b] = (int32_t)dt;
        dcount[b] = P;
        tstart[b] = (int32_t)tiles;
        const int nt = c.gx * c.gy;
        max_tiles = max(max_tiles, nt);
        tiles += nt;
        rows += P;
        pix += (int64_t)W * H;
        dt += ceil_div64(P, kSortTile);
        if (tiles > INT32_MAX || dt > INT32_MAX / kSortTile)
            return set_error(MSPLAT_ERR_CAPACITY, "batch_plan: batch too large");
    }
    dstart[B] = (int32_t)dt;
    tstart[B] = (int32_t)tiles;
    sizes[0] = tiles;                       // total tiles (tile_range rows)
    sizes[1] = rows;                        // total per-camera Gaussian rows
    sizes[2] = pix;                         // total pixels
    sizes[3] = dt * kSortTile;              // padded depth-key items
    sizes[4] = batch_tile_passes(max_tiles);  // tile-key passes of the finish
    return MSPLAT_OK;
}

extern "C" size_t msplat_batch_sort_prepare_workspace_size(int B, int64_t depth_items) {
    if (B <= 0 || depth_items < 0) return 0;
    SizeOnlyB z;
    BatchPrepareWs ws;
    batch_prepare_carve(z, B, depth_items, ws);
    return z.s.used;
}

extern "C" int msplat_batch_sort_prepare(const void *plan, int B, int64_t depth_items, const float *uv,
                                         const float *depth, const int32_t *radius, const float *conic,
                                         const float *opacity, int64_t *counts, void *workspace,
                                         size_t workspace_bytes, msplat_stream_t stream) {
    if (B <= 0 || depth_items < 0 || depth_items % kSortTile != 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_sort_prepare: B = %d, depth items %lld", B,
                         (long long)depth_items);
    if (!plan || !counts) return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_sort_prepare: null plan / counts");
    Workspace w(workspace, workspace_bytes);
    BatchPrepareWs ws;
    batch_prepare_carve(w, B, depth_items, ws);
    if (w.overflow)
        return set_error(MSPLAT_ERR_WORKSPACE, "batch_sort_prepare: workspace of %zu bytes < %zu", workspace_bytes,
                         msplat_batch_sort_prepare_workspace_size(B, depth_items));
    const BatchPlanView pv = batch_plan_view(plan, B);
    if (depth_items == 0) {
        cudaMemsetAsync(ws.cam_count, 0, sizeof(int64_t) * B, stream);
        launch(batch_layout_kernel, 1, 32, 0, stream, B, (const int64_t *)ws.cam_count, ws.fin_start, counts);
        return check_launch("batch_sort_prepare");
    }
    if (!uv || !depth || !radius || !conic || !opacity)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_sort_prepare: null pointer");
    const int dtiles = (int)(depth_items / kSortTile);
    launch(batch_key_rect_kernel, (unsigned)ceil_div64(depth_items, 256), 256, 0, stream, pv, depth_items,
           (const float2 *)uv, depth, radius, conic, opacity, ws.ka, ws.rect_at, ws.reach_at);
    SortSegs segs;
    segs.tile_start = pv.dtile_start;
    segs.count = pv.dcount;
    segs.nseg = B;
    // 4 passes (even): ka -> kb -> ka ... the values land in order
    int st = radix_sort_segmented<uint32_t>(dtiles, segs, 0, kBatchDepthPasses, ws.ka, nullptr, ws.ka, ws.order,
                                            ws.kb, ws.vt, ws.rb, stream);
    if (st) return st;
    launch(batch_count_kernel, (unsigned)(depth_items / 256), 256, 0, stream, pv, (const uint32_t *)ws.order,
           (const BatchRect *)ws.rect_at, ws.rects, ws.bsum);
    launch(batch_block_offsets_kernel, B, 1024, 0, stream, pv, ws.bsum, ws.cam_count);
    launch(batch_layout_kernel, 1, 32, 0, stream, B, (const int64_t *)ws.cam_count, ws.fin_start, counts);
    return check_launch("batch_sort_prepare");
}

extern "C" size_t msplat_batch_sort_finish_workspace_size(int B, int64_t capacity, int passes) {
    if (B <= 0 || capacity < 0 || passes <= 0) return 0;
    SizeOnlyB z;
    BatchFinishWs f;
    batch_finish_carve(z, B, ceil_div64(capacity, kSortTile) * kSortTile, passes, f);
    return z.s.used;
}

static int batch_sort_finish(const void *plan, int B, int64_t depth_items, int total_tiles, int passes,
                             int last_pass_bits, int64_t capacity, const void *prepare_workspace,
                             int32_t *idx_sorted, int32_t *tile_range, int32_t *status, void *workspace,
                             size_t workspace_bytes, cudaStream_t stream) {
    if (B <= 0 || depth_items < 0 || depth_items % kSortTile != 0 || total_tiles < 0 || passes <= 0 ||
        passes > 4 || capacity < 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_sort_finish: bad sizes");
    if (capacity % kSortTile != 0)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_sort_finish: capacity %lld is not a multiple of %d",
                         (long long)capacity, kSortTile);
    if (capacity > INT32_MAX)
        return set_error(MSPLAT_ERR_CAPACITY, "batch_sort_finish: capacity %lld exceeds int32",
                         (long long)capacity);
    if (!plan || !prepare_workspace || !tile_range || (capacity > 0 && !idx_sorted))
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_sort_finish: null pointer");
    if (((uintptr_t)idx_sorted & 15) != 0)  // the emit writes it with 16-byte stores
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_sort_finish: idx_sorted is not 16-byte aligned");
    Workspace pw(const_cast<void *>(prepare_workspace), msplat_batch_sort_prepare_workspace_size(B, depth_items));
    BatchPrepareWs prep;
    batch_prepare_carve(pw, B, depth_items, prep);
    Workspace w(workspace, workspace_bytes);
    BatchFinishWs f;
    batch_finish_carve(w, B, capacity, passes, f);
    if (w.overflow)
        return set_error(MSPLAT_ERR_WORKSPACE, "batch_sort_finish: workspace of %zu bytes < %zu", workspace_bytes,
                         msplat_batch_sort_finish_workspace_size(B, capacity, passes));
    const BatchPlanView pv = batch_plan_view(plan, B);
    const int ntiles = (int)(capacity / kSortTile);
    cudaMemsetAsync(tile_range, 0, sizeof(int32_t) * 2 * (size_t)total_tiles, stream);
    launch(batch_finish_segs_kernel, ceil_div(B + 1, 256), 256, 0, stream, B, ntiles,
           (const int32_t *)prep.fin_start, (const int64_t *)prep.cam_count, f.seg_start, f.seg_count, status);
    if (capacity == 0 || depth_items == 0) return check_launch("batch_sort_finish");
    // Even pass count: emit the ids straight into idx_sorted; odd: into the
    // temporary (as the single-camera finish).
    uint32_t *out = (uint32_t *)idx_sorted;
    const bool even = passes % 2 == 0;
    uint32_t *vemit = even ? out : f.vt;
    launch(batch_emit_kernel, (unsigned)(depth_items / 256), 256, 0, stream, pv, (const uint32_t *)prep.order,
           (const short4 *)prep.rects, (const RowReach *)prep.reach_at, (const int64_t *)prep.bsum,
           (const int64_t *)prep.cam_count, (const int32_t *)f.seg_start, f.ka, vemit, capacity);
    SortSegs segs;
    segs.tile_start = f.seg_start;
    segs.count = f.seg_count;
    segs.nseg = B;
    uint32_t *kout = even ? f.ka : f.kb;
    int st = radix_sort_segmented<uint32_t>(ntiles, segs, 0, passes, f.ka, vemit, kout, out, even ? f.kb : f.ka,
                                            f.vt, f.rb, stream, last_pass_bits);
    if (st) return st;
    launch(batch_range_kernel, (unsigned)ceil_div64(capacity / 8, 256), 256, 0, stream, pv, ntiles,
           (const int32_t *)f.seg_start, (const int64_t *)f.seg_count, (const uint32_t *)kout, (int2 *)tile_range);
    return check_launch("batch_sort_finish");
}

extern "C" int msplat_batch_sort_finish(const void *plan, int B, int64_t depth_items, int total_tiles, int passes,
                                        int64_t capacity, const void *prepare_workspace, int32_t *idx_sorted,
                                        int32_t *tile_range, int32_t *status, void *workspace,
                                        size_t workspace_bytes, msplat_stream_t stream) {
    return batch_sort_finish(plan, B, depth_items, total_tiles, passes, kRadixBits, capacity, prepare_workspace,
                             idx_sorted, tile_range, status, workspace, workspace_bytes, stream);
}

extern "C" int msplat_batch_sort_finish_bits(const void *plan, int B, int64_t depth_items, int total_tiles,
                                             int passes, int last_pass_bits, int64_t capacity,
                                             const void *prepare_workspace, int32_t *idx_sorted,
                                             int32_t *tile_range, int32_t *status, void *workspace,
                                             size_t workspace_bytes, msplat_stream_t stream) {
    if (last_pass_bits < 1 || last_pass_bits > kRadixBits)
        return set_error(MSPLAT_ERR_INVALID_ARGUMENT, "batch_sort_finish_bits: last_pass_bits = %d not in 1..8",
                         last_pass_bits);
    return batch_sort_finish(plan, B, depth_items, total_tiles, passes, last_pass_bits, capacity, prepare_workspace,
                             idx_sorted, tile_range, status, workspace, workspace_bytes, stream);
}

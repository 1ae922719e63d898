// LSD radix sort of (key, uint32 value) pairs and int32 scans, written for
// sm_103a without library calls.
//
// One 8-bit pass = three launches with no device-side waiting:
//   upsweep   per-tile digit histogram (per-warp shared atomics), stored
//             digit-major [256][tiles]
//   row scan  one block per digit: exclusive scan of its row (the start of
//             each (digit, tile) bucket among the digit's items) and the
//             digit's total
//   downsweep adds the exclusive scan of the 256 totals (the start of each
//             digit), re-reads the tile, ranks each item among equal digits with a
//             warp-level multisplit (stable: items are ranked in index
//             order), reorders the tile in shared memory and writes each
//             digit run contiguously (coalesced).
// Tiles are 3072 items (256 threads x 12).
#pragma once

#include "block_scan.cuh"

namespace msplat {

constexpr int kRadixBits = 8;
constexpr int kRadix = 1 << kRadixBits;
constexpr int kSortThreads = 256;
#ifndef MSPLAT_SORT_ITEMS
#define MSPLAT_SORT_ITEMS 12
#endif
constexpr int kSortItems = MSPLAT_SORT_ITEMS;
constexpr int kSortTile = kSortThreads * kSortItems;
constexpr int kSortWarps = kSortThreads / 32;

template <typename K>
__device__ __forceinline__ K sign_bit() { return K(1) << (sizeof(K) * 8 - 1); }

template <typename K>
__device__ __forceinline__ uint32_t digit_of(K k, int shift) {
    return (uint32_t)(k >> shift) & (kRadix - 1);
}

inline int sort_tiles(int64_t n) { return (int)ceil_div64(n, kSortTile); }

// Segments of a segmented sort: segment s holds count[s] items starting at
// item tile_start[s] * kSortTile (segments start on sort-tile boundaries,
// the gap after a segment's last item is padding that is neither read nor
// written).  Each segment is sorted on its own, in place of the same
// layout: the sorted items of segment s land in the same positions.  Both
// arrays live in device memory (the counts may come from a kernel), so a
// segmented sort needs no host read.
struct SortSegs {
    const int32_t *tile_start = nullptr;  // [nseg + 1]
    const int64_t *count = nullptr;       // [nseg]
    int nseg = 0;
};

// The segment holding sort tile t, or -1 past the last segment.
__device__ __forceinline__ int seg_of_tile(const SortSegs &sg, int t) {
    if (t >= sg.tile_start[sg.nseg]) return -1;
    int lo = 0, hi = sg.nseg - 1;  // last s with tile_start[s] <= t
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (sg.tile_start[mid] <= t) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Items of sort tile t inside its segment (0 past the last segment).
__device__ __forceinline__ int seg_tile_items(const SortSegs &sg, int t, int &seg) {
    seg = seg_of_tile(sg, t);
    if (seg < 0) return 0;
    const int64_t left = sg.count[seg] - (int64_t)(t - sg.tile_start[seg]) * kSortTile;
    return (int)max((int64_t)0, min((int64_t)kSortTile, left));
}

// Lanes of `valid` holding the same 8-bit digit as this lane, from eight
// ballots (much cheaper than __match_any_sync, whose throughput limits a
// ranking loop).  Every lane of the warp must call it.
__device__ __forceinline__ unsigned digit_peers(uint32_t d, unsigned valid) {
    unsigned peers = valid;
#pragma unroll
    for (int b = 0; b < kRadixBits; ++b) {
        const bool bit = (d >> b) & 1u;
        const unsigned bb = __ballot_sync(0xffffffffu, bit);
        peers &= bit ? bb : ~bb;
    }
    return peers;
}

// ---------------------------------------------------------------- upsweep
// All of a thread's keys are loaded before any counting so that the loads
// are in flight together; counts go to per-warp shared histograms with plain
// shared atomics (cheaper than aggregating equal digits first).
template <typename K, bool FLIP, bool SEG = false>
__global__ void __launch_bounds__(kSortThreads)
radix_upsweep_kernel(const K *__restrict__ keys, int64_t n, int shift, int ntiles,
                     uint32_t *__restrict__ hist, const int64_t *__restrict__ n_dev, SortSegs segs = {}) {
    __shared__ uint32_t cnt[kSortWarps][kRadix];
    if (SEG) {
        // items of this tile within its segment, as a length relative to
        // the tile's first item
        int sg;
        n = (int64_t)blockIdx.x * kSortTile + seg_tile_items(segs, blockIdx.x, sg);
    } else if (n_dev) {
        n = min(n, *n_dev);  // the length is on the device; n is the capacity
    }
    for (int i = threadIdx.x; i < kSortWarps * kRadix; i += kSortThreads) (&cnt[0][0])[i] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t base = (int64_t)blockIdx.x * kSortTile + warp * (32 * kSortItems) + lane;
    uint32_t dig[kSortItems];
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int64_t idx = base + r * 32;
        K k = idx < n ? __ldcs(keys + idx) : K(0);
        if (FLIP) k ^= sign_bit<K>();
        dig[r] = idx < n ? digit_of(k, shift) : 0xffffffffu;
    }
#pragma unroll
    for (int r = 0; r < kSortItems; ++r)
        if (dig[r] != 0xffffffffu) atomicAdd(&cnt[warp][dig[r]], 1u);
    __syncthreads();
    uint32_t c = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) c += cnt[w][threadIdx.x];
    hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = c;
}

// --------------------------------------------------------------- row scan
// Block d: exclusive scan of row d of hist in place, and the row's total.
// (A total per digit written once replaces atomics from every upsweep tile
// onto 256 addresses, which serialised when the digits were diverse.)
// Segmented (grid.y = segment s): the row's part [tile_start[s],
// tile_start[s + 1]) is scanned, and the total goes to totals[s][d].
static __global__ void __launch_bounds__(1024)
radix_rowscan_kernel(uint32_t *__restrict__ hist, uint32_t *__restrict__ totals, int ntiles,
                     SortSegs segs = {}) {
    __shared__ uint32_t scratch[33];
    const int d = blockIdx.x;
    uint32_t carry = 0;
    int t0 = 0, t1 = ntiles;
    if (segs.nseg) {
        t0 = segs.tile_start[blockIdx.y];
        t1 = segs.tile_start[blockIdx.y + 1];
        totals += (size_t)blockIdx.y * kRadix;
    }
    uint32_t *row = hist + (size_t)d * ntiles;
    for (int c0 = t0; c0 < t1; c0 += blockDim.x) {
        const int i = c0 + threadIdx.x;
        const uint32_t v = i < t1 ? row[i] : 0u;
        uint32_t tot;
        const uint32_t ex = block_exclusive_scan<uint32_t>(v, scratch, &tot);
        if (i < t1) row[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0) totals[d] = carry;
}

// Segmented row scan, one warp per (digit, segment): the segment's part of
// the digit's row scanned in place (exclusive) and its total to
// totals[s][d].  Any number of segments at the cost of their tiles.
static __global__ void __launch_bounds__(256)
radix_rowscan_warp_kernel(uint32_t *__restrict__ hist, uint32_t *__restrict__ totals, int ntiles, SortSegs segs) {
    const int gw = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (gw >= kRadix * segs.nseg) return;  // whole warps
    const int s = gw / kRadix, d = gw - s * kRadix;
    const int t0 = segs.tile_start[s], t1 = segs.tile_start[s + 1];
    uint32_t *row = hist + (size_t)d * ntiles;
    uint32_t carry = 0;
    for (int c0 = t0; c0 < t1; c0 += 32) {
        const int i = c0 + lane;
        const uint32_t v = i < t1 ? row[i] : 0u;
        const uint32_t inc = warp_inclusive_scan(v);
        if (i < t1) row[i] = carry + inc - v;
        carry += __shfl_sync(0xffffffffu, inc, 31);
    }
    if (lane == 0) totals[(size_t)s * kRadix + d] = carry;
}

// -------------------------------------------------------------- downsweep
inline size_t radix_downsweep_smem(size_t key_bytes) {
    return kSortTile * (key_bytes + 4) + (size_t)(kSortWarps * kRadix + 2 * kRadix) * 4;
}

// vals_in == nullptr means "value = input index".  FLIP_IN / FLIP_OUT xor
// the key's sign bit on load / store (signed-integer order).
// 32-bit keys: capped at 64 registers for 4 blocks per SM (no spill); the
// 64-bit keys of the reference-layout sort would spill there and keep 3.
template <typename K, bool FLIP_IN, bool FLIP_OUT, bool SEG = false>
__global__ void __launch_bounds__(kSortThreads, sizeof(K) == 4 ? 4 : 3)
radix_downsweep_kernel(const K *__restrict__ kin, const uint32_t *__restrict__ vin,
                       K *__restrict__ kout, uint32_t *__restrict__ vout, int64_t n, int shift,
                       int ntiles, const uint32_t *__restrict__ hist, const uint32_t *__restrict__ totals,
                       const int64_t *__restrict__ n_dev, SortSegs segs = {}) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    K *skeys = reinterpret_cast<K *>(sm_raw);
    uint32_t *svals = reinterpret_cast<uint32_t *>(skeys + kSortTile);
    uint32_t *whist = svals + kSortTile;            // [warps][radix]
    uint32_t *lstart = whist + kSortWarps * kRadix;  // [radix]
    uint32_t *gstart = lstart + kRadix;              // [radix]
    __shared__ uint32_t scan_scratch[33];

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int64_t base = (int64_t)blockIdx.x * kSortTile;
    int tile_n, sg = 0;
    int64_t out_base = 0;  // first item of the segment in the arrays
    if (SEG) {
        tile_n = seg_tile_items(segs, blockIdx.x, sg);
        if (sg < 0) return;  // past the last segment: nothing to move (uniform over the block)
        totals += (size_t)sg * kRadix;
        out_base = (int64_t)segs.tile_start[sg] * kSortTile;
    } else {
        if (n_dev) n = min(n, *n_dev);
        tile_n = (int)min((int64_t)kSortTile, n - base);  // <= 0 past a device-side length
    }
    for (int i = tid; i < kSortWarps * kRadix; i += kSortThreads) whist[i] = 0;
    // start of this tile's bucket of digit tid: the digit's start (scan of
    // the totals of the smaller digits) + the tile's offset within the digit
    const uint32_t dtot = totals[tid];
    const uint32_t dbase = block_exclusive_scan<uint32_t>(dtot, scan_scratch, nullptr);
    gstart[tid] = dbase + hist[(size_t)tid * ntiles + blockIdx.x];
    // A digit that every key of the sort (segment) shares makes the pass the
    // identity (stable): the tile is copied straight through.
    const int64_t n_all = SEG ? segs.count[sg] : n;
    if (__syncthreads_or(n_all > 0 && (int64_t)dtot == n_all)) {
        for (int i = tid; i < tile_n; i += kSortThreads) {
            K k = __ldcs(kin + base + i);
            if (FLIP_IN != FLIP_OUT) k ^= sign_bit<K>();
            if (kout) kout[base + i] = k;
            vout[base + i] = vin ? __ldcs(vin + base + i) : (uint32_t)(base + i - out_base);
        }
        return;
    }

    K key[kSortItems];
    uint32_t val[kSortItems];
    uint32_t rank[kSortItems];
    uint32_t *my_hist = whist + warp * kRadix;
    // Issue every load of the tile before ranking (the ranking loop's warp
    // barriers would otherwise serialise them).
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int li = warp * (32 * kSortItems) + r * 32 + lane;
        const bool valid = li < tile_n;
        K k = K(0);
        uint32_t v = 0;
        if (valid) {
            k = __ldcs(kin + base + li);
            if (FLIP_IN) k ^= sign_bit<K>();
            v = vin ? __ldcs(vin + base + li) : (uint32_t)(base + li - out_base);  // index within the segment
        }
        key[r] = k;
        val[r] = v;
    }
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int li = warp * (32 * kSortItems) + r * 32 + lane;
        const bool valid = li < tile_n;
        const K k = key[r];
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        const uint32_t d = digit_of(k, shift);
        const unsigned peers = digit_peers(d, vmask);
        uint32_t b0 = 0;
        if (valid) b0 = my_hist[d];
        __syncwarp();
        if (valid) {
            rank[r] = b0 + __popc(peers & ((1u << lane) - 1u));
            if (lane == 31 - __clz(peers)) my_hist[d] = b0 + __popc(peers);
        }
        __syncwarp();
    }
    __syncthreads();
    // Per digit (thread = digit): exclusive over warps, then over digits.
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        const uint32_t c = whist[w * kRadix + tid];
        whist[w * kRadix + tid] = tot;
        tot += c;
    }
    const uint32_t ex = block_exclusive_scan<uint32_t>(tot, scan_scratch, nullptr);
    lstart[tid] = ex;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int li = warp * (32 * kSortItems) + r * 32 + lane;
        if (li < tile_n) {
            const uint32_t d = digit_of(key[r], shift);
            const uint32_t pos = lstart[d] + my_hist[d] + rank[r];
            skeys[pos] = key[r];
            svals[pos] = val[r];
        }
    }
    __syncthreads();
    for (int i = tid; i < tile_n; i += kSortThreads) {
        K k = skeys[i];
        const uint32_t d = digit_of(k, shift);
        const size_t o = (size_t)out_base + (size_t)gstart[d] + (size_t)(i - (int)lstart[d]);
        if (FLIP_OUT) k ^= sign_bit<K>();
        if (kout) kout[o] = k;
        vout[o] = svals[i];
    }
}

// Workspace of one sort of n items over `passes` digits.
struct RadixBuffers {
    uint32_t *hist;    // [radix][tiles]
    uint32_t *totals;  // [passes][radix]
};

inline void radix_size(WorkspaceSizer &s, int64_t n, int passes) {
    s.take<uint32_t>((size_t)kRadix * sort_tiles(n));
    s.take<uint32_t>((size_t)kRadix * passes);
}

inline bool radix_take(Workspace &w, int64_t n, int passes, RadixBuffers &b) {
    b.hist = w.take<uint32_t>((size_t)kRadix * sort_tiles(n));
    b.totals = w.take<uint32_t>((size_t)kRadix * passes);
    return !w.overflow;
}

// Stable sort of n (key, value) pairs by key bits [begin_bit, begin_bit +
// 8 * passes).  Pass p reads `src` and writes `dst`; the chain is
//   in -> out -> tmp -> out ...   (odd pass count)
//   in -> tmp -> out -> tmp -> out (even pass count)
// so the result always lands in (kout, vout) and `in` is only read.
// Aliasing allowed: for an even pass count `in` may alias `out`, for an odd
// count `in` may alias `tmp`.  vin == nullptr means value = index.  kout may
// not be null.  FLIP: keys are signed integers (sign bit flipped on the
// first load and restored on the last store).
template <typename K, bool FLIP>
int radix_sort_pairs(int64_t n, int begin_bit, int passes, const K *kin, const uint32_t *vin,
                     K *kout, uint32_t *vout, K *ktmp, uint32_t *vtmp, const RadixBuffers &b,
                     cudaStream_t stream, const int64_t *n_dev = nullptr) {
    if (n <= 0 || passes <= 0) return MSPLAT_OK;
    const int nt = sort_tiles(n);
    const size_t smem = radix_downsweep_smem(sizeof(K));
    const K *ksrc = kin;
    const uint32_t *vsrc = vin;
    for (int p = 0; p < passes; ++p) {
        const int shift = begin_bit + p * kRadixBits;
        const bool to_out = ((passes - 1 - p) & 1) == 0;
        K *kdst = to_out ? kout : ktmp;
        uint32_t *vdst = to_out ? vout : vtmp;
        uint32_t *tot = b.totals + p * kRadix;
        const bool first = p == 0, last = p == passes - 1;
        if (FLIP && first)
            launch(radix_upsweep_kernel<K, true>, nt, kSortThreads, 0, stream, ksrc, n, shift, nt, b.hist, n_dev,
                   SortSegs{});
        else
            launch(radix_upsweep_kernel<K, false>, nt, kSortThreads, 0, stream, ksrc, n, shift, nt, b.hist, n_dev,
                   SortSegs{});
        launch(radix_rowscan_kernel, kRadix, 1024, 0, stream, b.hist, tot, nt, SortSegs{});
#define MSPLAT_DOWNSWEEP(FI, FO)                                                                                \
    do {                                                                                                        \
        auto kern = radix_downsweep_kernel<K, FI, FO>;                                                          \
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                     \
        launch(kern, nt, kSortThreads, smem, stream, ksrc, vsrc, kdst, vdst, n, shift, nt, b.hist, tot, n_dev,    \
               SortSegs{});                                                                             \
    } while (0)
        if (FLIP && first && last) MSPLAT_DOWNSWEEP(true, true);
        else if (FLIP && first) MSPLAT_DOWNSWEEP(true, false);
        else if (FLIP && last) MSPLAT_DOWNSWEEP(false, true);
        else MSPLAT_DOWNSWEEP(false, false);
#undef MSPLAT_DOWNSWEEP
        ksrc = kdst;
        vsrc = vdst;
    }
    return check_launch("radix_sort_pairs");
}

// Segmented stable sort of unsigned keys (see SortSegs): every segment's
// items sorted by key bits [begin_bit, begin_bit + 8 * passes) in place of
// the same layout, with the pass chain of radix_sort_pairs.  ntiles = the
// sort tiles the launches cover (at least segs.tile_start[nseg]); hist
// [radix][ntiles], totals [passes][nseg][radix].  vin == nullptr means value
// = index within the segment.
template <typename K>
int radix_sort_segmented(int ntiles, const SortSegs &segs, int begin_bit, int passes, const K *kin,
                         const uint32_t *vin, K *kout, uint32_t *vout, K *ktmp, uint32_t *vtmp, uint32_t *hist,
                         uint32_t *totals, cudaStream_t stream) {
    if (ntiles <= 0 || passes <= 0 || segs.nseg <= 0) return MSPLAT_OK;
    const size_t smem = radix_downsweep_smem(sizeof(K));
    const K *ksrc = kin;
    const uint32_t *vsrc = vin;
    auto down = radix_downsweep_kernel<K, false, false, true>;
    cudaFuncSetAttribute(down, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    for (int p = 0; p < passes; ++p) {
        const int shift = begin_bit + p * kRadixBits;
        const bool to_out = ((passes - 1 - p) & 1) == 0;
        K *kdst = to_out ? kout : ktmp;
        uint32_t *vdst = to_out ? vout : vtmp;
        uint32_t *tot = totals + (size_t)p * segs.nseg * kRadix;
        launch(radix_upsweep_kernel<K, false, true>, ntiles, kSortThreads, 0, stream, ksrc, (int64_t)0, shift,
               ntiles, hist, (const int64_t *)nullptr, segs);
        launch(radix_rowscan_warp_kernel, (unsigned)ceil_div64((int64_t)kRadix * segs.nseg, 8), 256, 0, stream,
               hist, tot, ntiles, segs);
        launch(down, ntiles, kSortThreads, smem, stream, ksrc, vsrc, kdst, vdst, (int64_t)0, shift, ntiles, hist,
               (const uint32_t *)tot, (const int64_t *)nullptr, segs);
        ksrc = kdst;
        vsrc = vdst;
    }
    return check_launch("radix_sort_segmented");
}

// ------------------------------------------------------------------- scan
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;

static __global__ void __launch_bounds__(kScanThreads)
scan_reduce_kernel(const int32_t *__restrict__ in, int n, int64_t *__restrict__ partials) {
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    int64_t s = 0;
    for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
        const int64_t idx = base + i;
        if (idx < n) s += in[idx];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ int64_t ws[kScanThreads / 32];
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        int64_t t = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) t += ws[w];
        partials[blockIdx.x] = t;
    }
}

// One block: exclusive scan of the tile sums (in place), total -> *total.
static __global__ void __launch_bounds__(1024)
scan_partials_kernel(int64_t *__restrict__ partials, int nparts, int64_t *__restrict__ total) {
    __shared__ int64_t scratch[33];
    int64_t carry = 0;
    for (int c0 = 0; c0 < nparts; c0 += blockDim.x) {
        const int i = c0 + threadIdx.x;
        const int64_t v = i < nparts ? partials[i] : 0;
        int64_t tot;
        const int64_t ex = block_exclusive_scan<int64_t>(v, scratch, &tot);
        if (i < nparts) partials[i] = carry + ex;
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

// Rescans each tile with its carry-in; writes inclusive or exclusive sums.
// Items are blocked per thread (16 consecutive) for a thread-local prefix.
static __global__ void __launch_bounds__(kScanThreads)
scan_apply_kernel(const int32_t *__restrict__ in, int n, const int64_t *__restrict__ partials,
                  int32_t *__restrict__ out, bool inclusive) {
    __shared__ int64_t scratch[33];
    __shared__ int32_t tile[kScanTile];
    const int64_t base = (int64_t)blockIdx.x * kScanTile;
    for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
        const int64_t idx = base + i;
        tile[i] = idx < n ? in[idx] : 0;
    }
    __syncthreads();
    int64_t local = 0;
    const int t0 = threadIdx.x * kScanItems;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) local += tile[t0 + k];
    const int64_t ex = block_exclusive_scan<int64_t>(local, scratch, nullptr);
    int64_t run = partials[blockIdx.x] + ex;
    int32_t res[kScanItems];
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        const int32_t v = tile[t0 + k];
        res[k] = (int32_t)(inclusive ? run + v : run);
        run += v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) tile[t0 + k] = res[k];
    __syncthreads();
    for (int i = threadIdx.x; i < kScanTile; i += kScanThreads) {
        const int64_t idx = base + i;
        if (idx < n) out[idx] = tile[i];
    }
}

inline void scan_size(WorkspaceSizer &s, int n) { s.take<int64_t>((size_t)ceil_div(n, kScanTile) + 1); }

inline int scan_i32(int n, const int32_t *in, int32_t *out, bool inclusive, int64_t *total,
                    int64_t *partials, cudaStream_t stream) {
    if (n <= 0) {
        if (total) cudaMemsetAsync(total, 0, sizeof(int64_t), stream);
        return check_launch("scan");
    }
    const int nb = ceil_div(n, kScanTile);
    launch(scan_reduce_kernel, nb, kScanThreads, 0, stream, in, n, partials);
    launch(scan_partials_kernel, 1, 1024, 0, stream, partials, nb, total);
    launch(scan_apply_kernel, nb, kScanThreads, 0, stream, in, n, partials, out, inclusive);
    return check_launch("scan");
}

}  // namespace msplat

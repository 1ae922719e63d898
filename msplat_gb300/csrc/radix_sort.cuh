// LSD radix sort of (key, uint32 value) pairs and int32 scans, written for
// sm_103a without library calls.
//
// Two implementations of an 8-bit pass, with identical results:
//
// Three launches per pass (the default): upsweep (per-tile digit
// histogram, stored digit-major [256][tiles]), row scan (one block per
// digit: exclusive scan of its row and the digit's total), downsweep
// (re-reads the tile, ranks each item among equal digits with a warp-level
// multisplit -- stable: items are ranked in index order -- reorders the
// tile in shared memory and writes each digit run contiguously).
//
// One kernel per pass (msplat_set_sort_onesweep): a histogram kernel reads
// the keys once and counts the digits of every pass (per segment); then
// each pass is one onesweep kernel.  Its blocks take sort tiles in order
// from an atomic counter, rank and reorder them as the downsweep does,
// publish the tile's count of every digit and find each digit's count in
// all earlier tiles by decoupled look-back over the published words (a
// tile's predecessors were taken by blocks that already run, so every wait
// ends; each is also bounded, see below).  Measured slower on GB300 for
// the tile lists (its kernel spills more at the same 64-register cap, and
// small sorts wait along long look-back chains), so it is not the default.
//
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

// Lanes of `valid` holding the same digit as this lane, from one ballot
// per significant digit bit (much cheaper than __match_any_sync, whose
// throughput limits a ranking loop).  `dbits` (<= 8, the same in every
// lane): only digit bits below it can be set in any key of the pass (the
// others are zero in every key and need no ballot).  Every lane of the
// warp must call it.
__device__ __forceinline__ unsigned digit_peers(uint32_t d, unsigned valid, int dbits = kRadixBits) {
    unsigned peers = valid;
#pragma unroll
    for (int b = 0; b < kRadixBits; ++b) {
        if (b < dbits) {
            const bool bit = (d >> b) & 1u;
            const unsigned bb = __ballot_sync(0xffffffffu, bit);
            peers &= bit ? bb : ~bb;
        }
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
                     uint32_t *__restrict__ hist, const int64_t *__restrict__ n_dev, int nd, SortSegs segs = {}) {
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
    if ((int)threadIdx.x < nd) hist[(size_t)threadIdx.x * ntiles + blockIdx.x] = c;  // (digits >= nd: none)
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
radix_rowscan_warp_kernel(uint32_t *__restrict__ hist, uint32_t *__restrict__ totals, int ntiles, int nd,
                          SortSegs segs) {
    const int gw = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (gw >= nd * segs.nseg) return;  // whole warps
    const int s = gw / nd, d = gw - s * nd;
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
// DB: the digit bits any key of the pass can have (the last pass of a sort
// whose keys are known to stay below 2^(shift + DB)); the ranking takes one
// ballot per such bit.
template <typename K, bool FLIP_IN, bool FLIP_OUT, bool SEG = false, int DB = kRadixBits>
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
    // (digits from 2^DB on occur in no key of the pass: no count, no row)
    const bool used = tid < (1 << DB);
    const uint32_t dtot = used ? totals[tid] : 0u;
    const uint32_t dbase = block_exclusive_scan<uint32_t>(dtot, scan_scratch, nullptr);
    gstart[tid] = dbase + (used ? hist[(size_t)tid * ntiles + blockIdx.x] : 0u);
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
        const unsigned peers = digit_peers(d, vmask, DB);
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

// ------------------------------------------------------------- onesweep
// Status word of a (tile, digit) in a pass's look-back array: a flag in the
// top two bits (0: not yet published), the count below.
constexpr unsigned long long kLbAggregate = 1ull << 62;  // the digit's count in this tile
constexpr unsigned long long kLbInclusive = 2ull << 62;  // ... in this tile and every earlier one of its segment
constexpr unsigned long long kLbCount = (1ull << 62) - 1;
constexpr int kHistTilesPerBlock = 16;  // sort tiles counted per block of the histogram kernel
constexpr int kLbWindow = 8;            // earlier tiles' words a look-back step reads at once
#ifndef MSPLAT_LB_BACKOFF_NS
#define MSPLAT_LB_BACKOFF_NS 256
#endif
constexpr unsigned kLbBackoffNs = MSPLAT_LB_BACKOFF_NS;  // sleep after a poll that found a word unpublished

// Set when a look-back wait of a onesweep pass gave up (see
// radix_onesweep_kernel); read and cleared through sort_wait_error.
static __device__ int g_sort_wait_error;

// Polls a look-back wait makes before it gives up (process-wide, shared
// with the blend's ring; set by msplat_set_wait_limit).
int wait_limit_polls();
// Whether the passes run as one kernel each (default) or as three launches
// (process-wide; msplat_set_sort_onesweep).
bool sort_onesweep_enabled();

__device__ __forceinline__ void st_relaxed_u64(unsigned long long *p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}

// Digit counts of every pass, per segment: totals[(p * nseg + s) * 256 + d]
// += the items of segment s whose digit in pass p is d (totals cleared by
// the caller).  Each block counts kHistTilesPerBlock consecutive sort tiles
// in per-warp shared histograms and adds them to the totals once per
// segment it covers.  Also clears the first pass's look-back words of its
// tiles and (block 0) the passes' tile counters.
template <typename K, bool FLIP, bool SEG>
__global__ void __launch_bounds__(kSortThreads)
radix_hist_kernel(const K *__restrict__ keys, int64_t n, int begin_bit, int passes, int ntiles,
                  uint32_t *__restrict__ totals, unsigned long long *__restrict__ status0, int *__restrict__ counters,
                  const int64_t *__restrict__ n_dev, SortSegs segs) {
    extern __shared__ uint32_t hcnt[];  // [warps][passes][radix]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int nseg = SEG ? segs.nseg : 1;
    if (!SEG && n_dev) n = min(n, *n_dev);
    if (blockIdx.x == 0 && tid < passes) counters[tid] = 0;
    const int t0 = blockIdx.x * kHistTilesPerBlock, t1 = min(ntiles, t0 + kHistTilesPerBlock);
    for (int64_t i = (int64_t)t0 * kRadix + tid; i < (int64_t)t1 * kRadix; i += kSortThreads) status0[i] = 0ull;
    const int hsize = kSortWarps * passes * kRadix;
    for (int i = tid; i < hsize; i += kSortThreads) hcnt[i] = 0u;
    __syncthreads();
    auto flush = [&](int sg) {
        __syncthreads();
        for (int p = 0; p < passes; ++p) {
            uint32_t c = 0;
#pragma unroll
            for (int w = 0; w < kSortWarps; ++w) {
                uint32_t &h = hcnt[(w * passes + p) * kRadix + tid];
                c += h;
                h = 0u;
            }
            if (c) atomicAdd(&totals[((size_t)p * nseg + sg) * kRadix + tid], c);
        }
        __syncthreads();
    };
    int cur = -1;  // the segment being counted (the same in every thread)
    for (int t = t0; t < t1; ++t) {
        int sg = 0, items;
        if (SEG) items = seg_tile_items(segs, t, sg);
        else items = (int)max((int64_t)0, min((int64_t)kSortTile, n - (int64_t)t * kSortTile));
        if (sg != cur) {
            if (cur >= 0) flush(cur);
            cur = sg;
        }
        if (sg < 0 || items <= 0) continue;
        const int64_t base = (int64_t)t * kSortTile;
        K k[kSortItems];
#pragma unroll
        for (int r = 0; r < kSortItems; ++r) {
            const int li = warp * (32 * kSortItems) + r * 32 + lane;
            k[r] = li < items ? __ldcs(keys + base + li) : K(0);
            if (FLIP) k[r] ^= sign_bit<K>();
        }
        for (int p = 0; p < passes; ++p) {
            uint32_t *h = hcnt + (warp * passes + p) * kRadix;
#pragma unroll
            for (int r = 0; r < kSortItems; ++r) {
                const int li = warp * (32 * kSortItems) + r * 32 + lane;
                if (li < items) atomicAdd(&h[digit_of(k[r], begin_bit + p * kRadixBits)], 1u);
            }
        }
    }
    if (cur >= 0) flush(cur);
}

inline size_t radix_hist_smem(int passes) { return (size_t)kSortWarps * passes * kRadix * sizeof(uint32_t); }

// One 8-bit pass in one kernel.  `totals` = this pass's digit counts of the
// block's segment ([nseg][radix]), `status` = this pass's look-back words
// ([tiles][radix], cleared), `status_next` = the next pass's (cleared here,
// row by row, for the tiles this pass covers; null after the last pass),
// `counter` = this pass's tile counter (zero).  A tile's items, ranks and
// output positions are those of radix_downsweep_kernel.
//
// Look-back (thread = digit d): the block publishes its count of d as an
// aggregate as soon as it is known, then walks back over the earlier tiles
// of its segment adding their published counts until it meets an inclusive
// one, and publishes its own inclusive count.  The walk gives up once it
// has polled wait_limit times without finding a word published (a limit of
// 0: before the first poll): it sets g_sort_wait_error and counts the rest
// as zero, so the kernel always finishes, with output positions that are
// wrong but in bounds (every count it adds is a true count of an earlier
// tile), and the host reports MSPLAT_ERR_TIMEOUT.
#ifndef MSPLAT_ONESWEEP_TRIM
#define MSPLAT_ONESWEEP_TRIM 1  // rank with one ballot per digit bit present in the segment's pass
#endif
#ifndef MSPLAT_ONESWEEP_MIN_BLOCKS
#define MSPLAT_ONESWEEP_MIN_BLOCKS 4  // resident onesweep blocks per SM asked of the compiler (32-bit keys)
#endif
template <typename K, bool FLIP_IN, bool FLIP_OUT, bool SEG>
__global__ void __launch_bounds__(kSortThreads, sizeof(K) == 4 ? MSPLAT_ONESWEEP_MIN_BLOCKS : 3)
radix_onesweep_kernel(const K *__restrict__ kin, const uint32_t *__restrict__ vin, K *__restrict__ kout,
                      uint32_t *__restrict__ vout, int64_t n, int shift,
                      const uint32_t *__restrict__ totals, unsigned long long *__restrict__ status,
                      unsigned long long *__restrict__ status_next, int *__restrict__ counter,
                      const int64_t *__restrict__ n_dev, SortSegs segs, int wait_limit) {
    extern __shared__ __align__(16) unsigned char sm_raw[];
    K *skeys = reinterpret_cast<K *>(sm_raw);
    uint32_t *svals = reinterpret_cast<uint32_t *>(skeys + kSortTile);
    uint32_t *whist = svals + kSortTile;             // [warps][radix]
    uint32_t *lstart = whist + kSortWarps * kRadix;  // [radix]
    uint32_t *gofs = lstart + kRadix;                // [radix]
    __shared__ uint32_t scan_scratch[33];
    __shared__ int s_tile;
    __shared__ unsigned s_digits;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    if (tid == 0) {
        s_tile = atomicAdd(counter, 1);
        s_digits = 0u;
    }
    __syncthreads();
    const int tile = s_tile;
    const int64_t base = (int64_t)tile * kSortTile;
    if (status_next) status_next[(size_t)tile * kRadix + tid] = 0ull;
    int tile_n, sg = 0, first = 0;
    int64_t out_base = 0;  // first item of the segment in the arrays
    if (SEG) {
        tile_n = seg_tile_items(segs, tile, sg);
        if (sg < 0) return;  // past the last segment: nothing to move
        totals += (size_t)sg * kRadix;
        first = segs.tile_start[sg];
        out_base = (int64_t)first * kSortTile;
    } else {
        if (n_dev) n = min(n, *n_dev);
        tile_n = (int)max((int64_t)0, min((int64_t)kSortTile, n - base));
    }
    // Empty tiles come after every non-empty one of their segment, so no
    // tile that looks back ever reaches one.
    if (tile_n <= 0) return;
    for (int i = tid; i < kSortWarps * kRadix; i += kSortThreads) whist[i] = 0;
    const uint32_t dtot = totals[tid];
    // The digit bits any key of the segment has set in this pass: those of
    // the OR of the digits present (the largest digit's bits).
    if (dtot) atomicOr(&s_digits, (unsigned)tid);
    const uint32_t dbase = block_exclusive_scan<uint32_t>(dtot, scan_scratch, nullptr);
#if MSPLAT_ONESWEEP_TRIM
    const int dbits = 32 - __clz((int)s_digits);
#else
    const int dbits = kRadixBits;
#endif
    // A digit that every key of the segment shares makes the pass the
    // identity (stable): every tile of the segment copies itself through.
    const int64_t n_all = SEG ? segs.count[sg] : n;
    if (__syncthreads_or(n_all > 0 && (int64_t)dtot == n_all)) {
        for (int i = tid; i < tile_n; i += kSortThreads) {
            K k = __ldcs(kin + base + i);
            if (FLIP_IN != FLIP_OUT) k ^= sign_bit<K>();
            kout[base + i] = k;
            vout[base + i] = vin ? __ldcs(vin + base + i) : (uint32_t)(base + i - out_base);
        }
        return;
    }

    K key[kSortItems];
    uint32_t val[kSortItems];
    uint32_t rank[kSortItems];
    uint32_t *my_hist = whist + warp * kRadix;
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int li = warp * (32 * kSortItems) + r * 32 + lane;
        const bool valid = li < tile_n;
        K k = K(0);
        uint32_t v = 0;
        if (valid) {
            k = __ldcs(kin + base + li);
            if (FLIP_IN) k ^= sign_bit<K>();
            v = vin ? __ldcs(vin + base + li) : (uint32_t)(base + li - out_base);
        }
        key[r] = k;
        val[r] = v;
    }
#pragma unroll
    for (int r = 0; r < kSortItems; ++r) {
        const int li = warp * (32 * kSortItems) + r * 32 + lane;
        const bool valid = li < tile_n;
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        const uint32_t d = digit_of(key[r], shift);
        const unsigned peers = digit_peers(d, vmask, dbits);
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
    uint32_t tot = 0;
#pragma unroll
    for (int w = 0; w < kSortWarps; ++w) {
        const uint32_t c = whist[w * kRadix + tid];
        whist[w * kRadix + tid] = tot;
        tot += c;
    }
    // publish this tile's count of digit tid before anything else
    unsigned long long *mine = status + (size_t)tile * kRadix + tid;
    st_relaxed_u64(mine, (tile == first ? kLbInclusive : kLbAggregate) | (unsigned long long)tot);
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
    // count of digit tid in the segment's earlier tiles: the walk reads
    // kLbWindow earlier words at a time (independent loads), adds them from
    // the nearest back while they are aggregates, and stops at the first
    // inclusive one; a word not yet published ends the window there and
    // the walk polls again from it
    uint32_t before = 0;
    if (tile != first) {
        int polls = 0;
        for (int t = tile - 1;;) {
            if (polls >= wait_limit) {
                atomicExch(&g_sort_wait_error, 1);
                break;
            }
            unsigned long long w[kLbWindow];
#pragma unroll
            for (int k = 0; k < kLbWindow; ++k)
                w[k] = t - k >= first ? ld_relaxed_u64(status + (size_t)(t - k) * kRadix + tid) : 0ull;
            int used = 0;
            bool done = false, blocked = false;
#pragma unroll
            for (int k = 0; k < kLbWindow; ++k) {
                if (done || blocked) continue;
                const unsigned long long f = w[k] & ~kLbCount;
                if (t - k < first || f == 0ull) {  // (the segment's first tile publishes an inclusive word)
                    blocked = true;
                    continue;
                }
                before += (uint32_t)(w[k] & kLbCount);
                ++used;
                done = f == kLbInclusive;
            }
            if (done) break;
            t -= used;
            if (blocked) {
                ++polls;
                __nanosleep(kLbBackoffNs);
            }
        }
        st_relaxed_u64(mine, kLbInclusive | (unsigned long long)(before + tot));
    }
    // output position of the tile's i-th reordered item with digit d:
    // out_base + gofs[d] + i (uint32 arithmetic; the sum is below 2^31)
    gofs[tid] = dbase + before - ex;
    __syncthreads();
    for (int i = tid; i < tile_n; i += kSortThreads) {
        K k = skeys[i];
        const uint32_t d = digit_of(k, shift);
        const size_t o = (size_t)out_base + (size_t)(uint32_t)(gofs[d] + (uint32_t)i);
        if (FLIP_OUT) k ^= sign_bit<K>();
        kout[o] = k;
        vout[o] = svals[i];
    }
}

inline size_t radix_onesweep_smem(size_t key_bytes) {
    return kSortTile * (key_bytes + 4) + (size_t)(kSortWarps * kRadix + 2 * kRadix) * 4;
}

// Reads (after synchronising `stream`) this translation unit's look-back
// error word, clearing it when reset != 0.
static inline cudaError_t sort_wait_error_read(int reset, int *value, cudaStream_t stream) {
    int h = 0;
    cudaError_t e = cudaMemcpyFromSymbolAsync(&h, g_sort_wait_error, sizeof(int), 0, cudaMemcpyDeviceToHost, stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e == cudaSuccess && reset && h) {
        const int zero = 0;
        e = cudaMemcpyToSymbolAsync(g_sort_wait_error, &zero, sizeof(int), 0, cudaMemcpyHostToDevice, stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    }
    *value = h;
    return e;
}

// Workspace of a sort over `ntiles` sort tiles, `nseg` segments (1 when
// not segmented) and `passes` digits.  The three-launch passes use the
// first quarter of the look-back words' bytes as their digit-major
// histogram.
struct RadixBuffers {
    uint32_t *hist = nullptr;                // [radix][tiles]           (three launches per pass)
    unsigned long long *status = nullptr;    // [2][tiles][radix]        (one kernel per pass)
    uint32_t *totals = nullptr;              // [passes][nseg][radix]
    int *counters = nullptr;                 // [passes]
};

template <typename WS>
inline void radix_carve(WS &w, int64_t ntiles, int nseg, int passes, RadixBuffers &b) {
    b.status = w.template take<unsigned long long>((size_t)2 * kRadix * ntiles);
    b.hist = reinterpret_cast<uint32_t *>(b.status);
    b.totals = w.template take<uint32_t>((size_t)kRadix * passes * nseg);
    b.counters = w.template take<int>((size_t)passes);
}

// The one-kernel passes of a sort (segmented when segs.nseg > 0): the
// histogram of every pass, then one onesweep launch per pass along the
// pass chain of radix_sort_pairs.  ntiles = the sort tiles the launches
// cover.  Graph-capturable (a memset and launches only).
template <typename K, bool FLIP>
int radix_onesweep_passes(int ntiles, int64_t n, const int64_t *n_dev, const SortSegs &segs, int begin_bit,
                          int passes, const K *kin, const uint32_t *vin, K *kout, uint32_t *vout,
                          K *ktmp, uint32_t *vtmp, const RadixBuffers &b, cudaStream_t stream) {
    const bool seg = segs.nseg > 0;
    const int nseg = seg ? segs.nseg : 1;
    cudaMemsetAsync(b.totals, 0, sizeof(uint32_t) * kRadix * passes * nseg, stream);
    const size_t hsm = radix_hist_smem(passes);
    const unsigned hblocks = (unsigned)ceil_div(ntiles, kHistTilesPerBlock);
    auto hist = seg ? radix_hist_kernel<K, FLIP, true> : radix_hist_kernel<K, FLIP, false>;
    if (hsm > 48 * 1024) cudaFuncSetAttribute(hist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)hsm);
    launch(hist, hblocks, kSortThreads, hsm, stream, kin, n, begin_bit, passes, ntiles, b.totals, b.status,
           b.counters, n_dev, segs);
    const size_t smem = radix_onesweep_smem(sizeof(K));
    const int limit = wait_limit_polls();
    const K *ksrc = kin;
    const uint32_t *vsrc = vin;
    for (int p = 0; p < passes; ++p) {
        const int shift = begin_bit + p * kRadixBits;
        const bool to_out = ((passes - 1 - p) & 1) == 0;
        K *kdst = to_out ? kout : ktmp;
        uint32_t *vdst = to_out ? vout : vtmp;
        const bool first = p == 0, last = p == passes - 1;
        unsigned long long *st = b.status + (size_t)(p & 1) * kRadix * ntiles;
        unsigned long long *st_next = last ? nullptr : b.status + (size_t)((p + 1) & 1) * kRadix * ntiles;
        const uint32_t *tot = b.totals + (size_t)p * nseg * kRadix;
#define MSPLAT_ONESWEEP(FI, FO, SG)                                                                             \
    do {                                                                                                        \
        auto kern = radix_onesweep_kernel<K, FI, FO, SG>;                                                       \
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                     \
        launch(kern, ntiles, kSortThreads, smem, stream, ksrc, vsrc, kdst, vdst, n, shift, tot, st, st_next,    \
               b.counters + p, n_dev, segs, limit);                                                             \
    } while (0)
        if (seg) MSPLAT_ONESWEEP(false, false, true);
        else if (FLIP && first && last) MSPLAT_ONESWEEP(true, true, false);
        else if (FLIP && first) MSPLAT_ONESWEEP(true, false, false);
        else if (FLIP && last) MSPLAT_ONESWEEP(false, true, false);
        else MSPLAT_ONESWEEP(false, false, false);
#undef MSPLAT_ONESWEEP
        ksrc = kdst;
        vsrc = vdst;
    }
    return check_launch("radix_onesweep_passes");
}

// Stable sort of n (key, value) pairs by key bits [begin_bit, begin_bit +
// 8 * passes).  Pass p
// reads `src` and writes `dst`; the chain is
//   in -> out -> tmp -> out ...   (odd pass count)
//   in -> tmp -> out -> tmp -> out (even pass count)
// so the result always lands in (kout, vout) and `in` is only read.
// Aliasing allowed: for an even pass count `in` may alias `out`, for an odd
// count `in` may alias `tmp`.  vin == nullptr means value = index.  kout may
// not be null.  FLIP: keys are signed integers (sign bit flipped on the
// first load and restored on the last store).  n_dev: the length is on the
// device (n is then the capacity the buffers hold).
template <typename K, bool FLIP>
int radix_sort_pairs(int64_t n, int begin_bit, int passes, const K *kin, const uint32_t *vin,
                     K *kout, uint32_t *vout, K *ktmp, uint32_t *vtmp, const RadixBuffers &b,
                     cudaStream_t stream, const int64_t *n_dev = nullptr, int last_bits = kRadixBits) {
    if (n <= 0 || passes <= 0) return MSPLAT_OK;
    const int nt = sort_tiles(n);
    if (sort_onesweep_enabled())
        return radix_onesweep_passes<K, FLIP>(nt, n, n_dev, SortSegs{}, begin_bit, passes, kin, vin, kout, vout,
                                              ktmp, vtmp, b, stream);
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
        // digits the pass can meet; the ranking is specialised for 5-7 bits (fewer round up to 5)
        int dbits = last ? last_bits : kRadixBits;
        if (FLIP || dbits < 1 || dbits > kRadixBits) dbits = kRadixBits;
        else if (dbits < 5) dbits = 5;
        const int nd = 1 << dbits;
        if (FLIP && first)
            launch(radix_upsweep_kernel<K, true>, nt, kSortThreads, 0, stream, ksrc, n, shift, nt, b.hist, n_dev, nd,
                   SortSegs{});
        else
            launch(radix_upsweep_kernel<K, false>, nt, kSortThreads, 0, stream, ksrc, n, shift, nt, b.hist, n_dev, nd,
                   SortSegs{});
        launch(radix_rowscan_kernel, nd, 1024, 0, stream, b.hist, tot, nt, SortSegs{});
#define MSPLAT_DOWNSWEEP(FI, FO, DBV)                                                                           \
    do {                                                                                                        \
        auto kern = radix_downsweep_kernel<K, FI, FO, false, DBV>;                                              \
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                     \
        launch(kern, nt, kSortThreads, smem, stream, ksrc, vsrc, kdst, vdst, n, shift, nt, b.hist, tot, n_dev,    \
               SortSegs{});                                                                                     \
    } while (0)
        if (FLIP && first && last) MSPLAT_DOWNSWEEP(true, true, kRadixBits);
        else if (FLIP && first) MSPLAT_DOWNSWEEP(true, false, kRadixBits);
        else if (FLIP && last) MSPLAT_DOWNSWEEP(false, true, kRadixBits);
        else if (dbits == 5) MSPLAT_DOWNSWEEP(false, false, 5);
        else if (dbits == 6) MSPLAT_DOWNSWEEP(false, false, 6);
        else if (dbits == 7) MSPLAT_DOWNSWEEP(false, false, 7);
        else MSPLAT_DOWNSWEEP(false, false, kRadixBits);
#undef MSPLAT_DOWNSWEEP
        ksrc = kdst;
        vsrc = vdst;
    }
    return check_launch("radix_sort_pairs");
}

// Segmented stable sort of unsigned keys (see SortSegs): every segment's
// items sorted by key bits [begin_bit, begin_bit + 8 * passes) in place of
// the same layout, with the pass chain of radix_sort_pairs.  ntiles = the
// sort tiles the launches cover (at least segs.tile_start[nseg]); the
// buffers are carved by radix_carve(ntiles, segs.nseg, passes).  vin ==
// nullptr means value = index within the segment.
template <typename K>
int radix_sort_segmented(int ntiles, const SortSegs &segs, int begin_bit, int passes, const K *kin,
                         const uint32_t *vin, K *kout, uint32_t *vout, K *ktmp, uint32_t *vtmp,
                         const RadixBuffers &b, cudaStream_t stream, int last_bits = kRadixBits) {
    if (ntiles <= 0 || passes <= 0 || segs.nseg <= 0) return MSPLAT_OK;
    if (sort_onesweep_enabled())
        return radix_onesweep_passes<K, false>(ntiles, 0, nullptr, segs, begin_bit, passes, kin, vin, kout, vout,
                                               ktmp, vtmp, b, stream);
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
        uint32_t *tot = b.totals + (size_t)p * segs.nseg * kRadix;
        // digits the pass can meet (as radix_sort_pairs: 5-7 bits specialised, fewer round up to 5)
        int dbits = p == passes - 1 ? last_bits : kRadixBits;
        if (dbits < 1 || dbits > kRadixBits) dbits = kRadixBits;
        else if (dbits < 5) dbits = 5;
        const int nd = 1 << dbits;
        launch(radix_upsweep_kernel<K, false, true>, ntiles, kSortThreads, 0, stream, ksrc, (int64_t)0, shift,
               ntiles, b.hist, (const int64_t *)nullptr, nd, segs);
        launch(radix_rowscan_warp_kernel, (unsigned)ceil_div64((int64_t)nd * segs.nseg, 8), 256, 0, stream,
               b.hist, tot, ntiles, nd, segs);
#define MSPLAT_SEG_DOWN(DBV)                                                                                    \
    do {                                                                                                        \
        auto kd = radix_downsweep_kernel<K, false, false, true, DBV>;                                           \
        cudaFuncSetAttribute(kd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                       \
        launch(kd, ntiles, kSortThreads, smem, stream, ksrc, vsrc, kdst, vdst, (int64_t)0, shift, ntiles, b.hist, \
               (const uint32_t *)tot, (const int64_t *)nullptr, segs);                                          \
    } while (0)
        if (dbits == 5) MSPLAT_SEG_DOWN(5);
        else if (dbits == 6) MSPLAT_SEG_DOWN(6);
        else if (dbits == 7) MSPLAT_SEG_DOWN(7);
        else launch(down, ntiles, kSortThreads, smem, stream, ksrc, vsrc, kdst, vdst, (int64_t)0, shift, ntiles,
                    b.hist, (const uint32_t *)tot, (const int64_t *)nullptr, segs);
#undef MSPLAT_SEG_DOWN
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

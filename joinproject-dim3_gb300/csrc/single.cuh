// single.cuh -- single-pass join-project: each row is expanded once.
//
// Every first insertion of a z (hash set or tile bitmap, as in expand.cuh)
// appends its z value -- loaded beside the z id, coalesced -- to the warp's
// own shared-memory staging buffer.  When the buffer would overflow, and at
// the end of the row, the warp reserves that many output slots with one
// atomicAdd on a global cursor and writes (x value, z value) pairs
// coalesced.  No second expansion, no gather through id2z, no cross-warp
// synchronisation for emission.  The output is dense and exact; pairs of one
// x come in chunks of up to kStage pairs, in unspecified order.  A
// reservation ending past the caller's capacity writes nothing; the cursor
// still ends at the exact total, which the host reports as the size needed.
#pragma once
#include "common.cuh"
#include "expand.cuh"

namespace dim3g {

#ifndef DIM3G_STAGE
#define DIM3G_STAGE 512
#endif
constexpr uint32_t kStage = DIM3G_STAGE;  // staged z values per warp (2 KB)

struct Reserve {
    unsigned long long* cursor;
    unsigned long long cap;
};

struct StageSink {
    static constexpr bool kValues = true;
    uint32_t* stage;  // this warp's buffer of `cap` entries
    uint2* out;
    Reserve rs;
    uint32_t xv;
    uint32_t n = 0;        // staged entries (warp-uniform)
    uint32_t cap = kStage;  // at least 32 * kUnroll

    __device__ __forceinline__ void flush() {
        if (n == 0) return;
        unsigned long long base = 0;
        if (lane_id() == 0) base = atomicAdd(rs.cursor, (unsigned long long)n);
        base = __shfl_sync(0xffffffffu, base, 0);
        __syncwarp();
        if (base + n <= rs.cap)
            for (uint32_t i = lane_id(); i < n; i += 32) st_stream(&out[base + i], make_uint2(xv, stage[i]));
        __syncwarp();
        n = 0;
    }

    template <uint32_t N>
    __device__ __forceinline__ void take(const uint32_t (&b)[N], const uint32_t (&v)[N]) {
        uint32_t tot = 0;
#pragma unroll
        for (uint32_t u = 0; u < N; u++) tot += __popc(b[u]);
        if (tot == 0) return;
        if (n + tot > cap) flush();
        const uint32_t lt = lanemask_lt();
        uint32_t pos = n;
#pragma unroll
        for (uint32_t u = 0; u < N; u++) {
            if (b[u] & (1u << lane_id())) stage[pos + __popc(b[u] & lt)] = v[u];
            pos += __popc(b[u]);
        }
        n += tot;
    }
};

// As StageSink, but staging (x value, z value) pairs, so a warp keeps one
// buffer across the many small rows it takes and reserves output once per
// kStage pairs instead of once per row (millions of rows of a few pairs
// each would otherwise serialise on the cursor).  The owner sets xv per row
// and flushes when it changes cursor and at the end.
struct PairStageSink {
    static constexpr bool kValues = true;
    uint2* stage;  // this warp's buffer of `cap` pairs
    uint2* out;
    Reserve rs;
    uint32_t xv;
    uint32_t cap;  // staged pairs the buffer holds (at least 32 * kUnroll)
    uint32_t n = 0;

    __device__ __forceinline__ void flush() {
        if (n == 0) return;
        unsigned long long base = 0;
        if (lane_id() == 0) base = atomicAdd(rs.cursor, (unsigned long long)n);
        base = __shfl_sync(0xffffffffu, base, 0);
        __syncwarp();
        if (base + n <= rs.cap)
            for (uint32_t i = lane_id(); i < n; i += 32) st_stream(&out[base + i], stage[i]);
        __syncwarp();
        n = 0;
    }

    template <uint32_t N>
    __device__ __forceinline__ void take(const uint32_t (&b)[N], const uint32_t (&v)[N]) {
        uint32_t tot = 0;
#pragma unroll
        for (uint32_t u = 0; u < N; u++) tot += __popc(b[u]);
        if (tot == 0) return;
        if (n + tot > cap) flush();
        const uint32_t lt = lanemask_lt();
        uint32_t pos = n;
#pragma unroll
        for (uint32_t u = 0; u < N; u++) {
            if (b[u] & (1u << lane_id())) stage[pos + __popc(b[u] & lt)] = make_uint2(xv, v[u]);
            pos += __popc(b[u]);
        }
        n += tot;
    }
};

// Summary sink: no pairs written; each lane sums pair hashes and counts of
// its first insertions, committed to the row's A-tile at the end of the row.
struct HashSink {
    static constexpr bool kValues = true;
    uint32_t xv = 0;
    unsigned long long h = 0, n = 0;
    template <uint32_t N>
    __device__ __forceinline__ void take(const uint32_t (&b)[N], const uint32_t (&v)[N]) {
#pragma unroll
        for (uint32_t u = 0; u < N; u++)
            if (b[u] & (1u << lane_id())) {
                h += pair_hash(xv, v[u]);
                n++;
            }
    }
    __device__ __forceinline__ void commit(const SumAcc& acc) {
        acc.commit(xv, n, n, h);
        h = n = 0;
    }
};

#ifndef DIM3G_BLOCK_DYN_PIECE
#define DIM3G_BLOCK_DYN_PIECE 0
#endif
// block-class rows: candidates a warp takes at a time from a shared counter
// (0: equal static shares)
constexpr uint32_t kBlockDynPiece = DIM3G_BLOCK_DYN_PIECE;
// CTA width of the two smaller-set block launches (block_split)
#ifndef DIM3G_BLOCK_SPLIT_THREADS
#define DIM3G_BLOCK_SPLIT_THREADS 256
#endif
constexpr uint32_t kBlockSplitThreads = DIM3G_BLOCK_SPLIT_THREADS;

// ---- row bodies (shared by the one-join kernels below and the many-query
// kernels of batch.cuh)

// Class 1: the calling warp expands row x with its own 2^warp_lg-word table
// (hash set, or a whole-domain bitmap when use_row_bitmap) into the warp's
// pair sink, which stays open across the warp's rows.
template <class Sink>
__device__ __forceinline__ void single_warp_row(const RowCtx& c, uint32_t x, uint32_t* tab, Sink& sink,
                                                uint32_t warp_lg) {
    const uint32_t lane = lane_id();
    const uint32_t u = c.ucap[x];
    const bool bm = use_row_bitmap(c.m, u, warp_lg);
    uint32_t lg = ceil_log2(2 * u);
    lg = lg < 5 ? 5 : (lg > warp_lg ? warp_lg : lg);
    const uint32_t nclr = bm ? row_bitmap_words(c.m) : (1u << lg);
    const uint32_t fill = bm ? 0u : kEmpty32;
    for (uint32_t s = lane; s < nclr; s += 32) tab[s] = fill;
    __syncwarp();
    sink.xv = c.id2x[x];
    if (bm) {
        TileBitmap set{tab, 0};
        warp_expand(c, c.JR_R[x], c.JR_R[x + 1], 0, 0, 0, c.T, set, sink);
    } else {
        HashSet set{tab, lg, c.err};
        warp_expand(c, c.JR_R[x], c.JR_R[x + 1], 0, 0, 0, c.T, set, sink);
    }
    __syncwarp();
}

// Row look-ahead for the bitmap class.  A CTA row starts with a chain of
// dependent global round trips -- the row counter's atomic, the row id, the
// row's header (x value, distinct bound, R bounds) -- before its own staging
// loads, with the whole CTA waiting.  With RowAhead, thread 0 walks that
// chain for the NEXT row once this row's first tile has started (the other
// warps take its share through the tile's dynamic pieces) and leaves the
// header in shared memory, read by every thread after the row's closing
// barrier.  (Block-class rows are too short for it: their static shares
// would wait on thread 0, and dynamic pieces cost them more than the chain.)
struct RowHead {
    uint32_t ri, xv, u, e0, e1;  // ri >= the row count: no row
};
struct NoAhead {
    __device__ __forceinline__ void run() {}
};
// Where the look-ahead reads from, set once per CTA (shared memory, so the
// row loop holds no registers for it).
struct AheadSrc {
    const uint32_t* rows;
    uint32_t* counter;
    const uint32_t* id2x;
    const uint32_t* ucap;
    const uint32_t* JR_R;
    uint32_t nrows;
};
static __shared__ AheadSrc s_ahead_src;
struct RowAhead {
    RowHead* dst;
    __device__ __forceinline__ void run() {
        if (threadIdx.x != 0) return;
        const AheadSrc& a = s_ahead_src;
        RowHead h{atomicAdd(a.counter, 1u), 0u, 0u, 0u, 0u};
        if (h.ri < a.nrows) {
            const uint32_t x = a.rows[h.ri];
            h.xv = a.id2x[x];
            h.u = a.ucap[x];
            h.e0 = a.JR_R[x];
            h.e1 = a.JR_R[x + 1];
        }
        *dst = h;
    }
};
// Thread 0: the look-ahead's source and the first row's header (s_head[0]);
// followed by a barrier in the caller.
__device__ __forceinline__ void ahead_start(const RowCtx& c, const uint32_t* rows, uint32_t* counter, uint32_t nrows,
                                            RowHead* s_head) {
    if (threadIdx.x != 0) return;
    s_ahead_src = AheadSrc{rows, counter, c.id2x, c.ucap, c.JR_R, nrows};
    RowAhead{s_head}.run();
}

// Class 2: the whole CTA expands row x; a 2^block_lg-word table (hash set or
// whole-domain bitmap) at smem, into each warp's sink (the caller sets its
// x value and flushes it).  Called by all threads after a barrier that
// follows the previous row; the caller's next call comes after another
// barrier (the last warps may still be expanding when this returns).
template <class Sink, class Ahead>
__device__ __forceinline__ void block_row(const RowCtx& c, uint32_t u, uint32_t e0, uint32_t e1, uint32_t* smem,
                                          Sink& sink, uint32_t block_lg, CtaChunks* cc, Ahead& ah) {
    const uint32_t wib = threadIdx.x >> 5;
    const uint32_t nw_lg = 31 - __clz(blockDim.x >> 5);
    const bool bm = use_row_bitmap(c.m, u, block_lg);
    uint32_t lg = ceil_log2(2 * u);
    lg = lg < 5 ? 5 : (lg > block_lg ? block_lg : lg);
    const uint32_t fill = bm ? 0u : kEmpty32;
    const uint32_t n4 = (bm ? row_bitmap_words(c.m) : (1u << lg)) / 4;
    uint4* t4 = reinterpret_cast<uint4*>(smem);
    for (uint32_t s = threadIdx.x; s < n4; s += blockDim.x) t4[s] = make_uint4(fill, fill, fill, fill);
    const uint32_t ne = e1 - e0;
    if (c.cta_rr == 3 && ne <= kRowBlk) {
        // balanced walk of one staging block: the table's clearing and the
        // staging share one barrier; the caller's next-row barrier ends it
        const uint64_t pol = l2_keep_policy();
        const uint32_t nw = blockDim.x >> 5;
        balanced_stage(c, e0, ne, 0, c.T, cc, pol, wib, nw);
        uint32_t* dyn = nullptr;
        if (kBlockDynPiece) {
            if (threadIdx.x == 0) cc->n = 0;
            dyn = &cc->n;
        }
        __syncthreads();
        ah.run();
        if (bm) {
            TileBitmap set{smem, 0};
            balanced_expand(c, ne, set, sink, cc->st.seg.s0, cc->st.seg.incl, cc->ctot, pol, wib, nw, dyn,
                            kBlockDynPiece);
        } else {
            HashSet set{smem, lg, c.err};
            balanced_expand(c, ne, set, sink, cc->st.seg.s0, cc->st.seg.incl, cc->ctot, pol, wib, nw, dyn,
                            kBlockDynPiece);
        }
        return;
    }
    __syncthreads();
    ah.run();
    if (bm) {
        TileBitmap set{smem, 0};
        cta_expand(c, e0, e1, wib, nw_lg, 0, c.T, set, sink, cc);
    } else {
        HashSet set{smem, lg, c.err};
        cta_expand(c, e0, e1, wib, nw_lg, 0, c.T, set, sink, cc);
    }
}

template <class Sink>
__device__ __forceinline__ void single_block_row(const RowCtx& c, uint32_t x, uint32_t* smem, Sink& sink,
                                                 uint32_t block_lg, CtaChunks* cc) {
    NoAhead na;
    block_row(c, c.ucap[x], c.JR_R[x], c.JR_R[x + 1], smem, sink, block_lg, cc, na);
}

// Classes 3/4 with the balanced walk for a row of at most kRowBlk entries
// whose S row bounds over all z tiles fit the staging table: the bounds
// (T + 1 per entry) are read once for the row, so each tile's chunks come
// from shared memory -- no global round trip and two barriers per tile.
#ifndef DIM3G_DYN_PIECE
#define DIM3G_DYN_PIECE 256
#endif
constexpr uint32_t kDynPiece = DIM3G_DYN_PIECE;  // candidates a warp takes at a time (staged bitmap rows)

// With kTilePrefetch each S segment is prefetched into L2 by one bulk
// prefetch a tile ahead (the first tile's while the row is staged).
#ifndef DIM3G_TILE_PREFETCH
#define DIM3G_TILE_PREFETCH 1
#endif
constexpr bool kTilePrefetch = DIM3G_TILE_PREFETCH != 0;

template <class Sink, class Ahead>
__device__ __forceinline__ void bitmap_row_staged(const RowCtx& c, uint32_t e0, uint32_t ne, uint32_t* bm,
                                                  Sink& sink, CtaChunks* cc, Ahead& ah) {
    const uint32_t lane = lane_id(), wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const uint32_t T = c.T, TB = T + 1, nch = (ne + 31) >> 5;
    const uint64_t pol = l2_keep_policy();
    uint32_t* bnd = cc->st.bnd;
    for (uint32_t i = threadIdx.x; i < ne; i += blockDim.x) {
        const uint32_t y = ld_keep(&c.IC_R[e0 + i], pol);
        const uint64_t r = (uint64_t)y * T;
        for (uint32_t k = 0; k <= T; k++) bnd[i * TB + k] = ld_keep(&c.JR_S[r + k], pol);
        if (kTilePrefetch && c.ISV) l2_prefetch(c.ISV + bnd[i * TB], c.ISV + bnd[i * TB + 1], pol);
    }
    for (uint32_t t = 0; t < T; t++) {
        const uint32_t lo = t * c.tile_width;
        const uint32_t width = min(c.tile_width, c.m - lo);
        const uint32_t words4 = (((width + 31) >> 5) + 3) >> 2;
        uint4* b4 = reinterpret_cast<uint4*>(bm);
        for (uint32_t w = threadIdx.x; w < words4; w += blockDim.x) b4[w] = make_uint4(0, 0, 0, 0);
        if (t == 0) __syncthreads();  // the staged bounds
        if (kTilePrefetch && t + 1 < T && c.ISV) {
            // the next tile's segments into L2 while this tile expands (its
            // candidate loads then hit L2 instead of waiting on DRAM)
            for (uint32_t i = threadIdx.x; i < ne; i += blockDim.x)
                l2_prefetch(c.ISV + bnd[i * TB + t + 1], c.ISV + bnd[i * TB + t + 2], pol);
        }
        for (uint32_t k = wib; k < nch; k += nw) {
            const uint32_t i = k * 32 + lane;
            const uint32_t len = i < ne ? bnd[i * TB + t + 1] - bnd[i * TB + t] : 0u;
            const uint32_t inc = warp_incl_scan(len);
            if (__any_sync(0xffffffffu, inc < len)) raise_error(c.err, kErrCountRange);  // 32-bit prefix wrapped
            if (lane == 31) cc->ctot[k] = inc;
        }
        if (threadIdx.x == 0) cc->n = 0;  // the tile's piece counter
        __syncthreads();  // the tile's bitmap cleared, its chunk totals written
        if (t == 0) ah.run();
        const uint32_t v = lane < nch ? cc->ctot[lane] : 0u;
        const uint32_t inc = warp_incl_scan(v);
        if (__any_sync(0xffffffffu, inc < v)) raise_error(c.err, kErrCountRange);
        const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
        TileBitmap set{bm, lo};
        // pieces of kDynPiece candidates taken from a shared counter: a warp
        // slowed by short segments takes fewer, so the tile's barrier waits
        // on at most one piece
        for (;;) {
            uint32_t p0 = 0;
            if (lane == 0) p0 = atomicAdd(&cc->n, kDynPiece);
            p0 = __shfl_sync(0xffffffffu, p0, 0);
            if (p0 >= total) break;
            const uint32_t p1 = min(p0 + kDynPiece, total);
            for (uint32_t k = __popc(__ballot_sync(0xffffffffu, lane < nch && inc <= p0)); k < nch; k++) {
                const uint32_t cin = __shfl_sync(0xffffffffu, inc, k), ctot = __shfl_sync(0xffffffffu, v, k);
                const uint32_t cex = cin - ctot;
                if (cex >= p1) break;
                if (ctot == 0) continue;
                const uint32_t i = k * 32 + lane;
                Chunk ch;
                ch.s0 = i < ne ? bnd[i * TB + t] : 0u;
                ch.len = i < ne ? bnd[i * TB + t + 1] - ch.s0 : 0u;
                ch.incl = warp_incl_scan(ch.len);
                ch.excl = ch.incl - ch.len;
                ch.total = ctot;
                const uint32_t plo = p0 > cex ? p0 - cex : 0u, phi = p1 < cin ? p1 - cex : ctot;
                expand_piece(c, ch, plo, phi, set, sink, pol);
            }
        }
        __syncthreads();  // every insert into this tile done before the next clear
    }
    if (T == 0) ah.run();
    if (threadIdx.x == 0) cc->n = 0;  // the round-robin walk's deferred-chunk count starts at 0
}

// Classes 3/4: the whole CTA expands row x one z tile at a time into a
// bitmap at bm (words rounded up to uint4, at least 32), into each warp's
// sink (the caller sets its x value and flushes it once for the row).
template <class Sink, class Ahead>
__device__ __forceinline__ void bitmap_row(const RowCtx& c, uint32_t e0, uint32_t e1, uint32_t* bm, Sink& sink,
                                           CtaChunks* cc, Ahead& ah) {
    const uint32_t wib = threadIdx.x >> 5;
    const uint32_t nw_lg = 31 - __clz(blockDim.x >> 5);
    const uint32_t ne = e1 - e0;
    if (c.cta_rr == 3 && ne <= kRowBlk && (uint64_t)ne * (c.T + 1) <= 2 * kRowBlk) {
        bitmap_row_staged(c, e0, ne, bm, sink, cc, ah);
        return;
    }
    for (uint32_t t = 0; t < c.T; t++) {
        const uint32_t lo = t * c.tile_width;
        const uint32_t width = min(c.tile_width, c.m - lo);
        const uint32_t words4 = (((width + 31) >> 5) + 3) >> 2;
        uint4* b4 = reinterpret_cast<uint4*>(bm);
        for (uint32_t w = threadIdx.x; w < words4; w += blockDim.x) b4[w] = make_uint4(0, 0, 0, 0);
        __syncthreads();
        if (t == 0) ah.run();
        TileBitmap set{bm, lo};
        cta_expand(c, e0, e1, wib, nw_lg, t, t + 1, set, sink, cc);
        __syncthreads();
    }
    if (c.T == 0) ah.run();  // (every look-ahead runs once a row)
}

template <class Sink>
__device__ __forceinline__ void single_bitmap_row(const RowCtx& c, uint32_t x, uint32_t* bm, Sink& sink,
                                                  CtaChunks* cc) {
    NoAhead na;
    bitmap_row(c, c.JR_R[x], c.JR_R[x + 1], bm, sink, cc, na);
}

// ---- one join

// Shared memory per warp of the warp classes: 2^warp_lg table words, then
// `stage` staged pairs.
__host__ __device__ constexpr size_t warp_row_words(uint32_t warp_lg, uint32_t stage) {
    return ((size_t)1 << warp_lg) + 2 * (size_t)stage;
}

// Classes 1 and 5 (tiny): one warp per row.
static __global__ void __launch_bounds__(256) k_single_warp(RowCtx c, Reserve rs, const uint32_t* __restrict__ rows,
                                                            const unsigned long long* __restrict__ nrows_p,
                                                            uint32_t warp_lg, uint32_t stage) {
    extern __shared__ uint32_t smem[];
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5;
    uint32_t* tab = smem + (size_t)wib * warp_row_words(warp_lg, stage);
    PairStageSink sink{reinterpret_cast<uint2*>(tab + (1u << warp_lg)), c.out, rs, 0, stage};
    const uint32_t nrows = (uint32_t)*nrows_p;
    for (uint32_t ri = blockIdx.x * nw + wib; ri < nrows; ri += gridDim.x * nw)
        single_warp_row(c, rows[ri], tab, sink, warp_lg);
    sink.flush();
}

// Class 2: one CTA per row; 2^block_lg table words, then one staging buffer
// per warp.
// Rows rows[skip0 + skip1 + i], i < *nrows_p (skips: device counts, either
// may be null), taken through row counter c.next_row[ctr].
static __global__ void __launch_bounds__(1024) k_single_block(RowCtx c, Reserve rs, const uint32_t* __restrict__ rows,
                                                              const unsigned long long* __restrict__ nrows_p,
                                                              uint32_t block_lg, const unsigned long long* skip0,
                                                              const unsigned long long* skip1, uint32_t ctr) {
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t s_row;
    __shared__ CtaChunks s_cc;
    if (threadIdx.x == 0) s_cc.n = 0;
    uint32_t* stage = smem + (1u << block_lg) + (threadIdx.x >> 5) * kStage;
    const uint32_t nrows = (uint32_t)*nrows_p;
    rows += (skip0 ? *skip0 : 0ull) + (skip1 ? *skip1 : 0ull);
    for (uint32_t ri = cta_next_row(&c.next_row[ctr], &s_row); ri < nrows; ri = cta_next_row(&c.next_row[ctr], &s_row)) {
        const uint32_t x = rows[ri];
        StageSink sink{stage, c.out, rs, c.id2x[x]};
        single_block_row(c, x, smem, sink, block_lg, &s_cc);
        sink.flush();
    }
}

// Classes 3/4: one CTA per row; a bitmap of bitmap_words, then one staging
// buffer per warp.  DIM3G_BM_THREADS threads a CTA for tiles of up to 2^19
// z ids (1024 for wider tiles).
#ifndef DIM3G_BM_THREADS
#define DIM3G_BM_THREADS 512
#endif
#ifndef DIM3G_BM_BOUNDS
#define DIM3G_BM_BOUNDS 1024
#endif
#ifndef DIM3G_BM_MINB
#define DIM3G_BM_MINB 1
#endif
static __global__ void __launch_bounds__(DIM3G_BM_BOUNDS, DIM3G_BM_MINB) k_single_bitmap(RowCtx c, Reserve rs, const uint32_t* __restrict__ rows,
                                                               const unsigned long long* __restrict__ n3,
                                                               const unsigned long long* __restrict__ n4,
                                                               uint32_t bitmap_words) {
    extern __shared__ uint32_t bm[];
    __shared__ uint32_t s_row;
    __shared__ CtaChunks s_cc;
    if (threadIdx.x == 0) s_cc.n = 0;
    uint32_t* stage = bm + bitmap_words + (threadIdx.x >> 5) * kStage;
    const uint32_t nrows = (uint32_t)(*n3 + *n4);
    __shared__ RowHead s_head[2];
    ahead_start(c, rows, &c.next_row[3], nrows, s_head);
    __syncthreads();
    for (uint32_t k = 0;; k ^= 1) {
        const RowHead h = s_head[k];
        if (h.ri >= nrows) break;
        RowAhead ah{&s_head[k ^ 1]};
        StageSink sink{stage, c.out, rs, h.xv};
        bitmap_row(c, h.e0, h.e1, bm, sink, &s_cc, ah);
        sink.flush();
        __syncthreads();  // the next row's header is in s_head[k ^ 1]
    }
}

// ---- summaries (no pairs written): the same row bodies into hash sinks

static __global__ void __launch_bounds__(256) k_sum_warp(RowCtx c, SumAcc acc, const uint32_t* __restrict__ rows,
                                                         const unsigned long long* __restrict__ nrows_p,
                                                         uint32_t warp_lg) {
    extern __shared__ uint32_t smem[];
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5;
    uint32_t* tab = smem + ((size_t)wib << warp_lg);
    const uint32_t nrows = (uint32_t)*nrows_p;
    HashSink sink;
    for (uint32_t ri = blockIdx.x * nw + wib; ri < nrows; ri += gridDim.x * nw) {
        single_warp_row(c, rows[ri], tab, sink, warp_lg);
        sink.commit(acc);
    }
}

static __global__ void __launch_bounds__(1024) k_sum_block(RowCtx c, SumAcc acc, const uint32_t* __restrict__ rows,
                                                           const unsigned long long* __restrict__ nrows_p,
                                                           uint32_t block_lg) {
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t s_row;
    __shared__ CtaChunks s_cc;
    if (threadIdx.x == 0) s_cc.n = 0;
    const uint32_t nrows = (uint32_t)*nrows_p;
    for (uint32_t ri = cta_next_row(&c.next_row[2], &s_row); ri < nrows; ri = cta_next_row(&c.next_row[2], &s_row)) {
        const uint32_t x = rows[ri];
        HashSink sink;
        sink.xv = c.id2x[x];
        single_block_row(c, x, smem, sink, block_lg, &s_cc);
        sink.commit(acc);
    }
}

static __global__ void __launch_bounds__(1024) k_sum_bitmap(RowCtx c, SumAcc acc, const uint32_t* __restrict__ rows,
                                                            const unsigned long long* __restrict__ n3,
                                                            const unsigned long long* __restrict__ n4) {
    extern __shared__ uint32_t bm[];
    __shared__ uint32_t s_row;
    __shared__ CtaChunks s_cc;
    if (threadIdx.x == 0) s_cc.n = 0;
    const uint32_t nrows = (uint32_t)(*n3 + *n4);
    for (uint32_t ri = cta_next_row(&c.next_row[3], &s_row); ri < nrows; ri = cta_next_row(&c.next_row[3], &s_row)) {
        const uint32_t x = rows[ri];
        HashSink sink;
        sink.xv = c.id2x[x];
        single_bitmap_row(c, x, bm, sink, &s_cc);
        sink.commit(acc);
    }
}

}  // namespace dim3g

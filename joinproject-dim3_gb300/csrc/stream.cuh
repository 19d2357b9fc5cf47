// stream.cuh -- the bitmap-class rows (classes 3/4) of the single-pass
// join-project with their candidates streamed into shared memory by TMA.
//
// The sparse expansion of Hybrid_solution (dim3.hpp:952-973) for the heavy
// rows: for an x row and one z tile, every z of S row y in that tile for
// every y of R row x, deduplicated in a shared-memory bitmap of the tile.
// The warp-per-lane form (single.cuh) spends most of its instructions
// finding each candidate's S segment and waits on dependent global loads.
// Here the CTA is split by role:
//   producer (warp 0)  takes rows from the class's dynamic counter, reads the
//                      row's S segment bounds for one tile 32 entries at a
//                      time, and copies the segments' (z id, z value) pairs
//                      into a ring of stages in shared memory: one
//                      cp.async.bulk of the segment's 16-byte-aligned
//                      superset (completion counted on the stage's mbarrier);
//                      a valid mask per stage marks the segment's own slots.
//                      A segment longer than kStreamPiece is cut into pieces
//                      at aligned points.
//   consumers          every consumer warp takes an equal slice of each
//                      stage: test-and-set of the tile bitmap from shared
//                      memory, first insertions staged per warp and written
//                      out as (x value, z value) pairs (StageSink).
// A stage's header names its row and tile and marks the last stage of a
// tile; after it the consumers meet on an mbarrier, clear the bitmap, and
// meet again.  The producer never waits on the bitmap, so it runs ahead by
// the ring's depth.  Every wait is bounded (kStreamWaitNs); one that runs out
// raises kErrStreamTimeout, stops every role of the CTA, and the producer
// waits (bounded) for its copies in flight before the CTA exits.
#pragma once
#include "common.cuh"
#include "dense.cuh"
#include "expand.cuh"
#include "single.cuh"

namespace dim3g {

#ifndef DIM3G_STREAM_CONSUMERS
#define DIM3G_STREAM_CONSUMERS 8
#endif
#ifndef DIM3G_STREAM_STAGES
#define DIM3G_STREAM_STAGES 4
#endif
constexpr uint32_t kStreamConsumers = DIM3G_STREAM_CONSUMERS;
constexpr uint32_t kStreamThreads = 32 * (kStreamConsumers + 1);
constexpr uint32_t kStreamStages = DIM3G_STREAM_STAGES;
constexpr uint32_t kStreamCap = 128 * kStreamConsumers;  // slots per stage: 128 per consumer warp (4 steps of 32)
static_assert(kStreamCap / kStreamConsumers == 32 * kUnroll, "a consumer's slice is one group of loads");
constexpr uint32_t kStreamPiece = 496;  // longest piece of a segment placed at once (+ 6 alignment slots <= cap / 2)
constexpr uint32_t kStreamStageVals = 256;  // staged z values per consumer warp
constexpr unsigned long long kStreamWaitNs = 2000000000ull;

enum StreamFlag : uint32_t { kStreamTileEnd = 1u, kStreamDone = 2u };

struct StreamHdr {
    uint32_t n;      // slots used (a multiple of 4)
    uint32_t x;      // row id
    uint32_t lo;     // the tile's first z id
    uint32_t flags;  // StreamFlag
};

// Dynamic shared memory of the kernel: the tile bitmap (bm_words, a
// multiple of 4) then the fixed part below.
struct StreamSmem {
    uint2 zv[kStreamStages][kStreamCap];  // (z id, z value) per slot
    uint32_t stage[kStreamConsumers][kStreamStageVals];
    uint32_t mask[kStreamStages][kStreamCap / 32];  // valid slots of each stage
    StreamHdr hdr[kStreamStages];
    unsigned long long full[kStreamStages], empty[kStreamStages];
    unsigned long long tdone, tclear;  // consumers: tile finished, bitmap cleared
    uint32_t abort;
};
__host__ __device__ constexpr size_t stream_smem_bytes(uint32_t bm_words) {
    return (size_t)bm_words * 4 + sizeof(StreamSmem);
}

__device__ __forceinline__ void mbar_expect_only(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Bulk copy of `bytes` (a multiple of 16) from global to shared memory, both
// 16-byte aligned, completing on mbarrier `bar`; kept in L2 (the S rows are
// read by many x rows).
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar, uint64_t pol) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;"
        ::"r"(dst), "l"(src), "r"(bytes), "r"(bar), "l"(pol)
        : "memory");
}
__device__ __forceinline__ bool stream_wait(uint32_t bar, uint32_t parity, volatile uint32_t* abort) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try(bar, parity)) {
        if (*abort) return false;
        if (global_ns() - t0 > kStreamWaitNs) return false;
    }
    return true;
}

// The producer: rows, tiles, 32-entry chunks of the row, segment pieces
// placed in lane order into the open stage.  Every piece is copied from the
// (z id, z value) pairs as its 16-byte-aligned superset [a & ~1, (b + 1) & ~1)
// -- at most one element of a neighbouring segment on either side, which the
// stage's valid mask leaves out -- so the producer never waits on segment
// data, only on the bounds.
__device__ __forceinline__ void stream_produce(const RowCtx& c, StreamSmem& sm, const uint32_t* __restrict__ rows,
                                               uint32_t nrows, uint32_t* s_row) {
    const uint32_t lane = lane_id();
    const uint64_t pol = l2_keep_policy();
    volatile uint32_t* abort = &sm.abort;
    uint32_t s = 0, ph = 0;    // the stage to fill next and its phase parity
    uint32_t fill = 0;         // slots used in the open stage (a multiple of 2)
    bool open = false;
    uint32_t closed = 0;       // stages closed since the start
    bool bad = false;

    auto acquire = [&]() -> bool {
        if (!stream_wait(smem_addr(&sm.empty[s]), ph ^ 1, abort)) return false;
        for (uint32_t w = lane; w < kStreamCap / 32; w += 32) sm.mask[s][w] = 0;
        fill = 0;
        open = true;
        return true;
    };
    // Publishes the open stage (header, valid mask) and arrives on its full
    // barrier; the copies complete it.
    auto close = [&](uint32_t x, uint32_t lo, uint32_t flags) {
        if (lane == 0) sm.hdr[s] = StreamHdr{fill, x, lo, flags};
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(&sm.full[s]));
        open = false;
        closed++;
        if (++s == kStreamStages) {
            s = 0;
            ph ^= 1;
        }
    };

    for (;;) {
        if (lane == 0) *s_row = atomicAdd(&c.next_row[3], 1u);
        __syncwarp();
        const uint32_t ri = *s_row;
        __syncwarp();
        if (ri >= nrows || bad) break;
        const uint32_t x = rows[ri];
        const uint32_t e0 = c.JR_R[x], e1 = c.JR_R[x + 1];
        // the row's first 32 join values, kept across its tiles
        const uint32_t y0 = e0 + lane < e1 ? ld_keep(&c.IC_R[e0 + lane], pol) : 0u;
        for (uint32_t t = 0; t < c.T && !bad; t++) {
            const uint32_t lo = t * c.tile_width;
            for (uint32_t eb = e0; eb < e1 && !bad; eb += 32) {
                const uint32_t e = eb + lane;
                uint32_t g0 = 0, g1 = 0;
                if (e < e1) {
                    const uint32_t y = eb == e0 ? y0 : ld_keep(&c.IC_R[e], pol);
                    const uint64_t r = (uint64_t)y * c.T + t;
                    g0 = ld_keep(&c.JR_S[r], pol);
                    g1 = ld_keep(&c.JR_S[r + 1], pol);
                }
                uint32_t a = g0;  // next element of this lane's segment to place
                while (__any_sync(0xffffffffu, a < g1)) {
                    if (!open && !acquire()) {
                        bad = true;
                        break;
                    }
                    // this lane's next piece [a, b): the segment's end, or an
                    // aligned point kStreamPiece or fewer elements on
                    uint32_t b = g1;
                    if (g1 - a > kStreamPiece) b = (a + kStreamPiece) & ~1u;
                    const uint32_t A0 = a & ~1u, A1 = (b + 1) & ~1u;
                    const uint32_t need = a < g1 ? A1 - A0 : 0u;
                    const uint32_t incl = warp_incl_scan(need), excl = incl - need;
                    const uint32_t room = kStreamCap - fill;
                    const uint32_t fits = __ballot_sync(0xffffffffu, !need || incl <= room);
                    const uint32_t placed = fits == 0xffffffffu ? 32u : __ffs(~fits) - 1;  // lanes [0, placed)
                    if (need && lane < placed) {
                        const uint32_t p = fill + excl;  // slot of element A0
                        const uint32_t full = smem_addr(&sm.full[s]);
                        mbar_expect_only(full, 8 * need);
                        bulk_g2s(smem_addr(&sm.zv[s][p]), &c.ISV[A0], 8 * need, full, pol);
                        // valid slots [p + a - A0, p + b - A0)
                        const uint32_t v0 = p + (a - A0), v1 = p + (b - A0);
                        for (uint32_t w = v0 >> 5; w <= (v1 - 1) >> 5; w++) {
                            const uint32_t lo_b = w * 32 > v0 ? 0u : v0 - w * 32;
                            const uint32_t hi_b = w * 32 + 32 < v1 ? 32u : v1 - w * 32;
                            const uint32_t bits = (hi_b == 32 ? 0xFFFFFFFFu : ((1u << hi_b) - 1u)) & ~((1u << lo_b) - 1u);
                            atomicOr(&sm.mask[s][w], bits);
                        }
                        a = b;
                    }
                    // slots taken by the placed lanes
                    const uint32_t used = placed ? __shfl_sync(0xffffffffu, incl, placed - 1) : 0u;
                    fill += used;
                    // a lane left over: the stage is as full as it gets
                    if (placed < 32 && __shfl_sync(0xffffffffu, need, placed)) close(x, lo, 0);
                }
            }
            if (bad) break;
            // end of the tile: close the open stage, or an empty one, marked
            if (!open && !acquire()) {
                bad = true;
                break;
            }
            close(x, lo, kStreamTileEnd);
        }
        if (bad) break;
    }
    if (!bad) {
        if (!open && !acquire()) bad = true;
        if (!bad) close(0, 0, kStreamDone);
    }
    if (bad) {
        if (lane == 0) {
            raise_error(c.err, kErrStreamTimeout);
            *abort = 1;
        }
        // an open stage may have copies in flight: close it, then wait
        // (bounded) for every stage closed within the ring's depth to
        // complete, so no copy lands after the CTA exits
        if (open) close(0, 0, kStreamDone);
        uint32_t ss = s, pp = ph;
        for (uint32_t k = 0; k < kStreamStages && k < closed; k++) {
            if (ss == 0) {
                ss = kStreamStages;
                pp ^= 1;
            }
            ss--;
            const unsigned long long t0 = global_ns();
            while (!mbar_try(smem_addr(&sm.full[ss]), pp) && global_ns() - t0 < kStreamWaitNs) {
            }
        }
    }
}

// The consumers (warps 1..kStreamConsumers).
__device__ __forceinline__ void stream_consume(const RowCtx& c, const Reserve& rs, StreamSmem& sm, uint32_t* bm,
                                               uint32_t bm_words) {
    const uint32_t lane = lane_id(), cw = (threadIdx.x >> 5) - 1;
    volatile uint32_t* abort = &sm.abort;
    StageSink sink{sm.stage[cw], c.out, rs, 0};
    sink.cap = kStreamStageVals;
    uint32_t cur_x = 0xFFFFFFFFu;
    uint32_t s = 0, ph = 0, tph = 0;
    bool bad = false;
    auto meet = [&](unsigned long long* bar) -> bool {
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(bar));
        return stream_wait(smem_addr(bar), tph, abort);
    };
    for (;;) {
        if (!stream_wait(smem_addr(&sm.full[s]), ph, abort)) {
            bad = true;
            break;
        }
        const StreamHdr h = sm.hdr[s];
        if (h.flags & kStreamDone) break;
        if (h.x != cur_x && h.n) {
            sink.flush();
            cur_x = h.x;
            sink.xv = c.id2x[h.x];
        }
        const uint2* zvs = sm.zv[s];
        const uint32_t base = cw * (kStreamCap / kStreamConsumers);
        if (base < h.n) {
            uint32_t z[kUnroll], v[kUnroll], b[kUnroll];
#pragma unroll
            for (uint32_t u = 0; u < kUnroll; u++) {
                const uint32_t i = base + u * 32 + lane;
                const bool in = i < h.n && ((sm.mask[s][(base >> 5) + u] >> lane) & 1u);
                const uint2 p = in ? zvs[i] : make_uint2(kEmpty32, 0u);
                z[u] = p.x;
                v[u] = p.y;
            }
            TileBitmap set{bm, h.lo};
#pragma unroll
            for (uint32_t u = 0; u < kUnroll; u++) b[u] = __ballot_sync(0xffffffffu, set.insert(z[u], z[u] != kEmpty32));
            sink.take(b, v);
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(&sm.empty[s]));
        if (++s == kStreamStages) {
            s = 0;
            ph ^= 1;
        }
        if (h.flags & kStreamTileEnd) {
            // every consumer done with the tile, then the bitmap cleared
            if (!meet(&sm.tdone)) {
                bad = true;
                break;
            }
            uint4* b4 = reinterpret_cast<uint4*>(bm);
            for (uint32_t w = cw * 32 + lane; w < bm_words / 4; w += kStreamConsumers * 32)
                b4[w] = make_uint4(0, 0, 0, 0);
            if (!meet(&sm.tclear)) {
                bad = true;
                break;
            }
            tph ^= 1;
        }
    }
    if (bad && lane == 0) {
        raise_error(c.err, kErrStreamTimeout);
        *abort = 1;
    }
    sink.flush();
}

// Classes 3/4 of the single pass: rows list_m[0 .. *n3 + *n4) (class 4
// first), bm_words-word tile bitmap (whole uint4s, >= 32).
static __global__ void __launch_bounds__(kStreamThreads) k_stream_bitmap(RowCtx c, Reserve rs,
                                                                         const uint32_t* __restrict__ rows,
                                                                         const unsigned long long* __restrict__ n3,
                                                                         const unsigned long long* __restrict__ n4,
                                                                         uint32_t bm_words) {
    extern __shared__ __align__(128) uint32_t stream_raw[];
    uint32_t* bm = stream_raw;
    StreamSmem& sm = *reinterpret_cast<StreamSmem*>(stream_raw + bm_words);
    __shared__ uint32_t s_row;
    const uint32_t nrows = (uint32_t)(*n3 + *n4);
    if (threadIdx.x == 0) {
        for (uint32_t k = 0; k < kStreamStages; k++) {
            mbar_init(smem_addr(&sm.full[k]), 1);
            mbar_init(smem_addr(&sm.empty[k]), kStreamConsumers);
        }
        mbar_init(smem_addr(&sm.tdone), kStreamConsumers);
        mbar_init(smem_addr(&sm.tclear), kStreamConsumers);
        sm.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    // the first tile's bitmap, cleared by everyone before the roles split
    uint4* b4 = reinterpret_cast<uint4*>(bm);
    for (uint32_t w = threadIdx.x; w < bm_words / 4; w += blockDim.x) b4[w] = make_uint4(0, 0, 0, 0);
    __syncthreads();
    if (threadIdx.x < 32)
        stream_produce(c, sm, rows, nrows, &s_row);
    else
        stream_consume(c, rs, sm, bm, bm_words);
}

}  // namespace dim3g

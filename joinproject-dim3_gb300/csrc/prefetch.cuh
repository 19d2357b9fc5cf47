// prefetch.cuh -- the block-class rows (class 2) of the single-pass
// join-project with their metadata fetched ahead by a producer warp.
//
// A block-class row is small (a few join values, a few thousand candidates,
// a shared-memory hash set of up to 2^block_lg slots), so with one CTA per
// row most of a row's time is the chain of dependent global loads before its
// first candidate: the row counter, the row id, the row's bounds, its join
// values, their S row bounds.  Here warp 0 runs that chain ahead of the
// others: it claims kPfBatch rows at a time, issues the loads of all of them
// together (one round trip per step of the chain for the whole batch), and
// writes each row -- id, x value, bound on distinct outputs, and for rows of
// at most kPfEntries join values their S segments and chunk totals -- into a
// ring of kPfSlots slots (mbarriers full / empty).  The other warps take rows
// from the ring in order: clear the hash set (or bitmap), meet, expand with
// the balanced walk of expand.cuh, meet, release the slot.  A row with more
// join values is staged by the expanding warps themselves.  Every wait is
// bounded (kStreamWaitNs); one that runs out raises kErrStreamTimeout and
// stops every role of the CTA.
#pragma once
#include "common.cuh"
#include "dense.cuh"
#include "expand.cuh"
#include "single.cuh"
#include "stream.cuh"

namespace dim3g {

constexpr uint32_t kPfWorkers = 15;                 // expanding warps
constexpr uint32_t kPfThreads = 32 * (kPfWorkers + 1);
constexpr uint32_t kPfSlots = 8;
constexpr uint32_t kPfBatch = 4;                    // rows claimed and fetched together
constexpr uint32_t kPfEntries = 64;                 // join values a slot stages (two chunks)

enum PfFlag : uint32_t { kPfSelfStage = 1u, kPfDone = 2u };

struct PfRow {
    uint32_t x, xv, u, e0, ne, flags;
    uint32_t s0[kPfEntries], len[kPfEntries], ctot[kPfEntries / 32];
};
struct PfSmem {
    PfRow row[kPfSlots];
    unsigned long long full[kPfSlots], empty[kPfSlots];
    unsigned long long ready, done;  // workers: set cleared and row staged; row expanded
    uint32_t abort;
};

// Warp 0: rows into the ring, kPfBatch at a time.
__device__ __forceinline__ void pf_produce(const RowCtx& c, PfSmem& sm, const uint32_t* __restrict__ rows,
                                           uint32_t nrows, uint32_t* counter) {
    const uint32_t lane = lane_id();
    const uint64_t pol = l2_keep_policy();
    volatile uint32_t* abort = &sm.abort;
    uint32_t s = 0, ph = 0;
    bool bad = false;
    auto acquire = [&]() -> bool { return stream_wait(smem_addr(&sm.empty[s]), ph ^ 1, abort); };
    auto publish = [&]() {
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(&sm.full[s]));
        if (++s == kPfSlots) {
            s = 0;
            ph ^= 1;
        }
    };
    for (;;) {
        uint32_t ri0 = 0;
        if (lane == 0) ri0 = atomicAdd(counter, kPfBatch);
        ri0 = __shfl_sync(0xffffffffu, ri0, 0);
        if (ri0 >= nrows) break;
        const uint32_t nb = min(kPfBatch, nrows - ri0);
        // the batch's rows (lane j < nb holds row j)
        uint32_t x = 0, e0 = 0, e1 = 0, u = 0, xv = 0;
        if (lane < nb) {
            x = rows[ri0 + lane];
            e0 = c.JR_R[x];
            e1 = c.JR_R[x + 1];
            u = c.ucap[x];
            xv = c.id2x[x];
        }
        // join values of the rows short enough to stage: entry k of row j at
        // lane k % 32, register j * 2 + k / 32
        uint32_t y[kPfBatch * 2], g0[kPfBatch * 2], g1[kPfBatch * 2];
#pragma unroll
        for (uint32_t j = 0; j < kPfBatch; j++) {
            const uint32_t je0 = __shfl_sync(0xffffffffu, e0, j), jne = __shfl_sync(0xffffffffu, e1 - e0, j);
            const bool staged = j < nb && jne <= kPfEntries;
#pragma unroll
            for (uint32_t h = 0; h < 2; h++) {
                const uint32_t k = h * 32 + lane;
                y[j * 2 + h] = staged && k < jne ? ld_keep(&c.IC_R[je0 + k], pol) : 0xFFFFFFFFu;
            }
        }
#pragma unroll
        for (uint32_t q = 0; q < kPfBatch * 2; q++) {
            g0[q] = g1[q] = 0;
            if (y[q] != 0xFFFFFFFFu) {
                const uint64_t r = (uint64_t)y[q] * c.T;
                g0[q] = ld_keep(&c.JR_S[r], pol);
                g1[q] = ld_keep(&c.JR_S[r + c.T], pol);
            }
        }
#pragma unroll
        for (uint32_t j = 0; j < kPfBatch; j++) {
            if (j >= nb) break;
            if (!acquire()) {
                bad = true;
                break;
            }
            PfRow& pr = sm.row[s];
            const uint32_t jne = __shfl_sync(0xffffffffu, e1 - e0, j);
            const uint32_t jx = __shfl_sync(0xffffffffu, x, j), jxv = __shfl_sync(0xffffffffu, xv, j),
                           ju = __shfl_sync(0xffffffffu, u, j), je0 = __shfl_sync(0xffffffffu, e0, j);
            if (lane == 0) {
                pr.x = jx;
                pr.xv = jxv;
                pr.u = ju;
                pr.e0 = je0;
                pr.ne = jne;
                pr.flags = jne <= kPfEntries ? 0u : kPfSelfStage;
            }
            if (jne <= kPfEntries) {
#pragma unroll
                for (uint32_t h = 0; h < 2; h++) {
                    const uint32_t len = g1[j * 2 + h] - g0[j * 2 + h];
                    pr.s0[h * 32 + lane] = g0[j * 2 + h];
                    pr.len[h * 32 + lane] = len;
                    const uint32_t inc = warp_incl_scan(len);
                    if (__any_sync(0xffffffffu, inc < len)) raise_error(c.err, kErrCountRange);
                    if (lane == 31) pr.ctot[h] = inc;
                }
            }
            publish();
        }
        if (bad) break;
    }
    if (!bad) {
        if (acquire()) {
            if (lane == 0) sm.row[s].flags = kPfDone;
            publish();
        } else {
            bad = true;
        }
    }
    if (bad && lane == 0) {
        raise_error(c.err, kErrStreamTimeout);
        *abort = 1;
    }
}

// Warps 1..kPfWorkers: rows from the ring, expanded into each warp's sink.
template <class Sink>
__device__ __forceinline__ void pf_work(const RowCtx& c, PfSmem& sm, uint32_t* tab, uint32_t block_lg, Sink& sink,
                                        CtaChunks* cc) {
    const uint32_t lane = lane_id(), wi = (threadIdx.x >> 5) - 1, tw = threadIdx.x - 32, ntw = 32 * kPfWorkers;
    const uint64_t pol = l2_keep_policy();
    volatile uint32_t* abort = &sm.abort;
    uint32_t s = 0, ph = 0, mph = 0;
    bool bad = false;
    auto meet = [&](unsigned long long* bar) -> bool {
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_addr(bar));
        return stream_wait(smem_addr(bar), mph, abort);
    };
    for (;;) {
        if (!stream_wait(smem_addr(&sm.full[s]), ph, abort)) {
            bad = true;
            break;
        }
        const PfRow& pr = sm.row[s];
        const uint32_t flags = pr.flags;
        if (flags & kPfDone) break;
        const uint32_t u = pr.u, e0 = pr.e0, ne = pr.ne;
        sink.xv = pr.xv;
        const bool bm = use_row_bitmap(c.m, u, block_lg);
        uint32_t lg = ceil_log2(2 * u);
        lg = lg < 5 ? 5 : (lg > block_lg ? block_lg : lg);
        const uint32_t fill = bm ? 0u : kEmpty32;
        const uint32_t n4 = (bm ? row_bitmap_words(c.m) : (1u << lg)) / 4;
        uint4* t4 = reinterpret_cast<uint4*>(tab);
        for (uint32_t i = tw; i < n4; i += ntw) t4[i] = make_uint4(fill, fill, fill, fill);
        const uint32_t* s0a = pr.s0;
        const uint32_t* lena = pr.len;
        const uint32_t* ctota = pr.ctot;
        uint32_t blk = ne;  // entries expanded in this pass
        if (flags & kPfSelfStage) {
            blk = min(ne, kRowBlk);
            balanced_stage(c, e0, blk, 0, c.T, cc, pol, wi, kPfWorkers);
            s0a = cc->st.seg.s0;
            lena = cc->st.seg.incl;
            ctota = cc->ctot;
        }
        if (!meet(&sm.ready)) {
            bad = true;
            break;
        }
        for (uint32_t eb = e0;;) {
            if (bm) {
                TileBitmap set{tab, 0};
                balanced_expand(c, blk, set, sink, s0a, lena, ctota, pol, wi, kPfWorkers);
            } else {
                HashSet set{tab, lg, c.err};
                balanced_expand(c, blk, set, sink, s0a, lena, ctota, pol, wi, kPfWorkers);
            }
            if (!meet(&sm.done)) {
                bad = true;
                break;
            }
            mph ^= 1;
            eb += blk;
            if (eb >= e0 + ne) break;
            // a row of more than kRowBlk join values: its next block
            blk = min(e0 + ne - eb, kRowBlk);
            balanced_stage(c, eb, blk, 0, c.T, cc, pol, wi, kPfWorkers);
            if (!meet(&sm.ready)) {
                bad = true;
                break;
            }
        }
        if (bad) break;
        if (tw == 0) mbar_arrive(smem_addr(&sm.empty[s]));
        if (++s == kPfSlots) {
            s = 0;
            ph ^= 1;
        }
        sink.flush();
    }
    if (bad && lane == 0) {
        raise_error(c.err, kErrStreamTimeout);
        *abort = 1;
    }
    sink.flush();
}

// Class 2 of the single pass with prefetched rows: 2^block_lg table words,
// then one kStage staging buffer per expanding warp.
static __global__ void __launch_bounds__(kPfThreads) k_single_block_pf(RowCtx c, Reserve rs,
                                                                       const uint32_t* __restrict__ rows,
                                                                       const unsigned long long* __restrict__ nrows_p,
                                                                       uint32_t block_lg) {
    extern __shared__ __align__(16) uint32_t pf_raw[];
    __shared__ PfSmem sm;
    __shared__ CtaChunks s_cc;
    const uint32_t nrows = (uint32_t)*nrows_p;
    if (threadIdx.x == 0) {
        for (uint32_t k = 0; k < kPfSlots; k++) {
            mbar_init(smem_addr(&sm.full[k]), 1);
            mbar_init(smem_addr(&sm.empty[k]), 1);
        }
        mbar_init(smem_addr(&sm.ready), kPfWorkers);
        mbar_init(smem_addr(&sm.done), kPfWorkers);
        sm.abort = 0;
        s_cc.n = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        pf_produce(c, sm, rows, nrows, &c.next_row[2]);
    } else {
        uint32_t* stage = pf_raw + (1u << block_lg) + ((threadIdx.x >> 5) - 1) * kStage;
        StageSink sink{stage, c.out, rs, 0};
        pf_work(c, sm, pf_raw, block_lg, sink, &s_cc);
    }
}

}  // namespace dim3g

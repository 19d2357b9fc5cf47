// aggregate.cuh -- COUNT(*) GROUP BY (x, z): the write pass of the
// join-aggregate (SpmmAggregate with a COUNT plug-in, dim3.hpp:1271-1310).
//
// The count pass is the join-project count pass (distinct z per row).  The
// write pass expands each row again with a per-z counter -- a shared-memory
// hash map (z -> count) for classes 1 and 2, a shared-memory counter array
// over one z tile for classes 3/4 -- and then emits every (x, z, count) of
// the row at off[x] + a row-local slot.  Counts are exact: each expansion
// candidate is one joining (R tuple, S tuple) pair.
#pragma once
#include "common.cuh"
#include "expand.cuh"

namespace dim3g {

struct AggOut {
    unsigned long long* cnt;  // one count per output pair
    SumAcc sum;               // sum.tiles set: summaries instead of output
};

// Summary emission: per-lane sums over the occupied map slots [s0, s1)
// (stride 32) or over the nonzero direct counters.
struct GroupSums {
    unsigned long long g = 0, cs = 0, h = 0;
    __device__ __forceinline__ void add(uint32_t xv, uint32_t zv, uint32_t cnt) {
        g++;
        cs += cnt;
        h += group_hash(xv, zv, cnt);
    }
};
__device__ __forceinline__ void sum_map_slots(const RowCtx& c, const uint32_t* keys, const uint32_t* vals,
                                              uint32_t s0, uint32_t s1, uint32_t xv, GroupSums& gs) {
    for (uint32_t s = s0 + lane_id(); s < s1; s += 32) {
        const uint32_t key = keys[s];
        if (key != kEmpty32) gs.add(xv, __ldg(&c.id2z[key]), vals[s]);
    }
}
__device__ __forceinline__ void sum_counters(const RowCtx& c, const uint32_t* ctr, uint32_t s0, uint32_t s1,
                                             uint32_t lo, uint32_t xv, GroupSums& gs) {
    for (uint32_t s = s0 + lane_id(); s < s1; s += 32) {
        const uint32_t v = ctr[s];
        if (v) gs.add(xv, __ldg(&c.id2z[lo + s]), v);
    }
}

// Shared-memory map slot of z (inserting it if absent).
__device__ __forceinline__ uint32_t smem_map_slot(uint32_t* keys, uint32_t lg, uint32_t z, uint32_t* err) {
    const uint32_t mask = (1u << lg) - 1;
    uint32_t h = (z * 0x9E3779B1u) >> (32 - lg);
    volatile uint32_t* vk = keys;
    for (uint32_t p = 0; p <= mask; p++) {
        uint32_t cur = vk[h];
        if (cur == z) return h;
        if (cur == kEmpty32) {
            uint32_t prev = atomicCAS(&keys[h], kEmpty32, z);
            if (prev == kEmpty32 || prev == z) return h;
        }
        h = (h + 1) & mask;
    }
    raise_error(err, kErrTableFull);
    return 0xFFFFFFFFu;
}

// Counting "sets" for warp_expand: they count every candidate and report no
// first insertions (emission happens after the expansion).
struct CountMap {
    uint32_t* keys;
    uint32_t* vals;
    uint32_t lg;
    uint32_t* err;
    __device__ __forceinline__ bool insert(uint32_t z, bool act) {
        if (act) {
            uint32_t s = smem_map_slot(keys, lg, z, err);
            if (s != 0xFFFFFFFFu) atomicAdd(&vals[s], 1u);
        }
        return false;
    }
};
struct CountTile {
    uint32_t* ctr;
    uint32_t lo;
    __device__ __forceinline__ bool insert(uint32_t z, bool act) {
        if (act) atomicAdd(&ctr[z - lo], 1u);
        return false;
    }
};
struct NullSink {
    static constexpr bool kValues = false;
    template <uint32_t N>
    __device__ __forceinline__ void take(const uint32_t (&)[N], const uint32_t (&)[N]) {}
};

// Warp-collective emission of occupied map slots [s0, s1) with stride 32.
// shared_pos: CTA-wide row-local slot counter; nullptr for a warp-owned row
// (then *local_pos is the running slot).
__device__ __forceinline__ void emit_map_slots_warp(const RowCtx& c, AggOut ao, const uint32_t* keys,
                                                    const uint32_t* vals, uint32_t s0, uint32_t s1, uint32_t xv,
                                                    unsigned long long base, uint32_t lim, uint32_t* shared_pos,
                                                    uint32_t* local_pos) {
    const uint32_t lane = lane_id();
    for (uint32_t sb = s0; sb < s1; sb += 32) {
        uint32_t s = sb + lane;
        uint32_t key = (s < s1) ? keys[s] : kEmpty32;
        bool occ = key != kEmpty32;
        uint32_t b = __ballot_sync(0xffffffffu, occ);
        if (!b) continue;
        uint32_t pb;
        if (shared_pos) {
            pb = 0;
            if (lane == 0) pb = atomicAdd(shared_pos, (uint32_t)__popc(b));
            pb = __shfl_sync(0xffffffffu, pb, 0);
        } else {
            pb = *local_pos;
            *local_pos += __popc(b);
        }
        if (occ) {
            uint32_t pos = pb + __popc(b & lanemask_lt());
            if (pos < lim) {
                c.out[base + pos] = make_uint2(xv, __ldg(&c.id2z[key]));
                ao.cnt[base + pos] = vals[s];
            } else {
                raise_error(c.err, kErrOutputBound);
            }
        }
    }
}

// A map-class row counts with one counter per z of the whole domain instead
// of a z -> count hash map when the m counters fit the kernel's map memory
// (2^words_lg words) and scanning them costs little against the row's
// candidates (m <= 8 u).
__device__ __forceinline__ bool use_row_counters(uint32_t m, uint32_t u, uint32_t words_lg) {
    return (uint64_t)m <= (1ull << words_lg) && (uint64_t)m <= 8ull * u;
}

// Warp-collective emission of the nonzero direct counters ctr[s0, s1): the
// counter index is the z id.  shared_pos / local_pos as above.
__device__ __forceinline__ void emit_counters_warp(const RowCtx& c, AggOut ao, const uint32_t* ctr, uint32_t s0,
                                                   uint32_t s1, uint32_t xv, unsigned long long base, uint32_t lim,
                                                   uint32_t* shared_pos, uint32_t* local_pos) {
    const uint32_t lane = lane_id();
    for (uint32_t sb = s0; sb < s1; sb += 32) {
        const uint32_t s = sb + lane;
        const uint32_t v = (s < s1) ? ctr[s] : 0u;
        const uint32_t b = __ballot_sync(0xffffffffu, v != 0);
        if (!b) continue;
        uint32_t pb;
        if (shared_pos) {
            pb = 0;
            if (lane == 0) pb = atomicAdd(shared_pos, (uint32_t)__popc(b));
            pb = __shfl_sync(0xffffffffu, pb, 0);
        } else {
            pb = *local_pos;
            *local_pos += __popc(b);
        }
        if (v) {
            const uint32_t pos = pb + __popc(b & lanemask_lt());
            if (pos < lim) {
                c.out[base + pos] = make_uint2(xv, __ldg(&c.id2z[s]));
                ao.cnt[base + pos] = v;
            } else {
                raise_error(c.err, kErrOutputBound);
            }
        }
    }
}

// Class 1 write pass: one warp per row; per warp 2^lg keys + 2^lg counts.
static __global__ void __launch_bounds__(256) k_agg_warp(RowCtx c, AggOut ao, const uint32_t* __restrict__ rows,
                                                  const unsigned long long* __restrict__ nrows_p, uint32_t warp_lg) {
    extern __shared__ uint32_t smem[];
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = lane_id();
    uint32_t* keys = smem + ((size_t)wib << (warp_lg + 1));
    uint32_t* vals = keys + (1u << warp_lg);
    const uint32_t nrows = (uint32_t)*nrows_p;
    for (uint32_t ri = blockIdx.x * nw + wib; ri < nrows; ri += gridDim.x * nw) {
        const uint32_t x = rows[ri];
        const uint32_t u = c.ucap[x];
        const bool sum = ao.sum.tiles != nullptr;
        NullSink sink;
        uint32_t pos = 0;
        if (use_row_counters(c.m, u, warp_lg + 1)) {
            for (uint32_t s = lane; s < c.m; s += 32) keys[s] = 0;  // keys + vals: one counter array
            __syncwarp();
            CountTile set{keys, 0};
            warp_expand(c, c.JR_R[x], c.JR_R[x + 1], 0, 0, 0, c.T, set, sink);
            __syncwarp();
            if (sum) {
                GroupSums gs;
                sum_counters(c, keys, 0, c.m, 0, c.id2x[x], gs);
                ao.sum.commit(c.id2x[x], gs.g, gs.cs, gs.h);
            } else {
                emit_counters_warp(c, ao, keys, 0, c.m, c.id2x[x], c.off[x], c.cnt[x], nullptr, &pos);
            }
            __syncwarp();
            continue;
        }
        uint32_t lg = ceil_log2(2 * u);
        lg = lg < 5 ? 5 : (lg > warp_lg ? warp_lg : lg);
        for (uint32_t s = lane; s < (1u << lg); s += 32) {
            keys[s] = kEmpty32;
            vals[s] = 0;
        }
        __syncwarp();
        CountMap set{keys, vals, lg, c.err};
        warp_expand(c, c.JR_R[x], c.JR_R[x + 1], 0, 0, 0, c.T, set, sink);
        __syncwarp();
        if (sum) {
            GroupSums gs;
            sum_map_slots(c, keys, vals, 0, 1u << lg, c.id2x[x], gs);
            ao.sum.commit(c.id2x[x], gs.g, gs.cs, gs.h);
        } else {
            emit_map_slots_warp(c, ao, keys, vals, 0, 1u << lg, c.id2x[x], c.off[x], c.cnt[x], nullptr, &pos);
        }
        __syncwarp();
    }
}

// Class 2 write pass: one CTA per row.
static __global__ void __launch_bounds__(256) k_agg_block(RowCtx c, AggOut ao, const uint32_t* __restrict__ rows,
                                                   const unsigned long long* __restrict__ nrows_p, uint32_t block_lg) {
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t s_pos, s_row;
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5;
    const uint32_t nw_lg = 31 - __clz(nw);
    uint32_t* keys = smem;
    uint32_t* vals = smem + (1u << block_lg);
    const uint32_t nrows = (uint32_t)*nrows_p;
    for (uint32_t ri = cta_next_row(&c.next_row[2], &s_row); ri < nrows; ri = cta_next_row(&c.next_row[2], &s_row)) {
        const uint32_t x = rows[ri];
        const uint32_t u = c.ucap[x];
        const bool direct = use_row_counters(c.m, u, block_lg + 1);
        uint32_t lg = ceil_log2(2 * u);
        lg = lg < 5 ? 5 : (lg > block_lg ? block_lg : lg);
        if (direct) {
            for (uint32_t s = threadIdx.x; s < c.m; s += blockDim.x) keys[s] = 0;
        } else {
            for (uint32_t s = threadIdx.x; s < (1u << lg); s += blockDim.x) {
                keys[s] = kEmpty32;
                vals[s] = 0;
            }
        }
        if (threadIdx.x == 0) s_pos = 0;
        __syncthreads();
        NullSink sink;
        if (direct) {
            CountTile set{keys, 0};
            warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, 0, c.T, set, sink);
        } else {
            CountMap set{keys, vals, lg, c.err};
            warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, 0, c.T, set, sink);
        }
        __syncthreads();
        const uint32_t span = direct ? c.m : (1u << lg);
        const uint32_t per = (((span + nw - 1) / nw) + 31) & ~31u;
        const uint32_t s0 = min(span, wib * per), s1 = min(span, s0 + per);
        if (ao.sum.tiles) {
            GroupSums gs;
            if (direct) sum_counters(c, keys, s0, s1, 0, c.id2x[x], gs);
            else sum_map_slots(c, keys, vals, s0, s1, c.id2x[x], gs);
            ao.sum.commit(c.id2x[x], gs.g, gs.cs, gs.h);
        } else if (direct) {
            emit_counters_warp(c, ao, keys, s0, s1, c.id2x[x], c.off[x], c.cnt[x], &s_pos, nullptr);
        } else {
            emit_map_slots_warp(c, ao, keys, vals, s0, s1, c.id2x[x], c.off[x], c.cnt[x], &s_pos, nullptr);
        }
    }
}

// Classes 3/4 write pass: one CTA per row; a counter per z of one tile.
static __global__ void __launch_bounds__(1024) k_agg_tile(RowCtx c, AggOut ao, const uint32_t* __restrict__ rows,
                                                   const unsigned long long* __restrict__ n3,
                                                   const unsigned long long* __restrict__ n4) {
    extern __shared__ uint32_t ctr[];
    __shared__ uint32_t s_pos, s_row;
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = lane_id();
    const uint32_t nw_lg = 31 - __clz(nw);
    const uint32_t nrows = (uint32_t)(*n3 + *n4);
    for (uint32_t ri = cta_next_row(&c.next_row[3], &s_row); ri < nrows; ri = cta_next_row(&c.next_row[3], &s_row)) {
        const uint32_t x = rows[ri];
        const bool sum = ao.sum.tiles != nullptr;
        const unsigned long long base = sum ? 0 : c.off[x];
        const uint32_t lim = sum ? 0 : c.cnt[x], xv = c.id2x[x];
        GroupSums gs;
        if (threadIdx.x == 0) s_pos = 0;
        for (uint32_t t = 0; t < c.T; t++) {
            const uint32_t lo = t * c.tile_width;
            const uint32_t width = min(c.tile_width, c.m - lo);
            for (uint32_t w = threadIdx.x; w < width; w += blockDim.x) ctr[w] = 0;
            __syncthreads();
            CountTile set{ctr, lo};
            NullSink sink;
            warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, t, t + 1, set, sink);
            __syncthreads();
            if (sum) {
                for (uint32_t wb = wib * 32; wb < width; wb += nw * 32)
                    sum_counters(c, ctr, wb, min(width, wb + 32), lo, xv, gs);
                __syncthreads();
                continue;
            }
            // emit the nonzero counters of this tile
            for (uint32_t wb = wib * 32; wb < width; wb += nw * 32) {
                uint32_t w = wb + lane;
                uint32_t v = w < width ? ctr[w] : 0;
                uint32_t b = __ballot_sync(0xffffffffu, v != 0);
                if (!b) continue;
                uint32_t pb = 0;
                if (lane == 0) pb = atomicAdd(&s_pos, (uint32_t)__popc(b));
                pb = __shfl_sync(0xffffffffu, pb, 0);
                if (v) {
                    uint32_t pos = pb + __popc(b & lanemask_lt());
                    if (pos < lim) {
                        c.out[base + pos] = make_uint2(xv, __ldg(&c.id2z[lo + w]));
                        ao.cnt[base + pos] = v;
                    } else {
                        raise_error(c.err, kErrOutputBound);
                    }
                }
            }
            __syncthreads();
        }
        if (sum) ao.sum.commit(xv, gs.g, gs.cs, gs.h);
    }
}

}  // namespace dim3g

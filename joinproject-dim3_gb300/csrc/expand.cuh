// expand.cuh -- the sparse expansion with on-chip deduplication: the GPU
// form of Hybrid_solution's SPA loop (dim3.hpp:952-973).
//
// For an x row the candidates are every z of S row y for every y of R row x.
// Rows are binned by u = min(candidates, m), an upper bound on their distinct
// outputs:
//   class 1 (u <= cap_w): one warp per row, a private shared-memory hash set
//   class 2 (u <= cap_b): one CTA per row, a shared-memory hash set
//   class 3 (u >  cap_b): one CTA per row, a shared-memory bitmap over one
//                          z tile at a time (S is bucketed by (y, z tile)).
// Each kernel runs twice: a count pass writes cnt[x] = |distinct z|; after a
// prefix sum over cnt the write pass repeats the expansion and every first
// insertion of a z emits (x value, z value) at off[x] + a row-local slot, so
// each row's pairs are contiguous and the whole output is dense.
#pragma once
#include "common.cuh"

namespace dim3g {

constexpr uint32_t kEmpty32 = 0xFFFFFFFFu;

struct RowCtx {
    const uint32_t* JR_R;  // n+1 row pointers of R by x id
    const uint32_t* IC_R;  // y ids
    const uint32_t* JR_S;  // k*T+1 row pointers of S by (y id, z tile)
    const uint32_t* IC_S;  // z ids
    uint32_t T;            // z tiles
    uint32_t tile_width;   // z ids per tile (bitmap width)
    uint32_t m;            // z domain size
    const uint32_t* ucap;  // per row min(candidates, m)
    uint32_t* cnt;         // per row distinct count (count pass output)
    const unsigned long long* off;  // per row output offset (write pass input)
    const uint32_t* id2x;
    const uint32_t* id2z;
    uint2* out;
    uint32_t* err;
};

__device__ __forceinline__ uint32_t ceil_log2(uint32_t v) { return v <= 1 ? 0 : 32 - __clz(v - 1); }

// Insert z into an open-addressing set of 2^lg 32-bit slots in shared memory.
// Returns true for the first insertion of z.
__device__ __forceinline__ bool smem_set_insert(uint32_t* tab, uint32_t lg, uint32_t z, uint32_t* err) {
    const uint32_t mask = (1u << lg) - 1;
    uint32_t h = (z * 0x9E3779B1u) >> (32 - lg);
    volatile uint32_t* vt = tab;
    for (uint32_t p = 0; p <= mask; p++) {
        uint32_t cur = vt[h];
        if (cur == z) return false;
        if (cur == kEmpty32) {
            uint32_t prev = atomicCAS(&tab[h], kEmpty32, z);
            if (prev == kEmpty32) return true;
            if (prev == z) return false;
        }
        h = (h + 1) & mask;
    }
    raise_error(err, kErrTableFull);
    return false;
}

// Warp-cooperative expansion of R entries [e0, e1) over S tiles [t0, t1).
// The warp takes chunks of 32 entries starting at e0 + chunk0, stepping by
// chunk_step; within a chunk the candidate space is flattened by a warp
// prefix sum over segment lengths and every lane locates its segment by a
// 5-step binary search over the lanes' inclusive prefixes, so lanes stay
// busy whatever the segment lengths.  ins(z) -> bool runs per lane;
// emit(isnew, z) is warp-collective.
template <class Ins, class Emit>
__device__ __forceinline__ void warp_expand(const RowCtx& c, uint32_t e0, uint32_t e1, uint32_t chunk0,
                                            uint32_t chunk_step, uint32_t t0, uint32_t t1, Ins& ins, Emit& emit) {
    const uint32_t lane = lane_id();
    for (uint32_t eb = e0 + chunk0; eb < e1; eb += chunk_step) {
        uint32_t e = eb + lane;
        uint32_t s0 = 0, len = 0;
        if (e < e1) {
            uint32_t y = __ldg(&c.IC_R[e]);
            uint64_t r = (uint64_t)y * c.T;
            s0 = __ldg(&c.JR_S[r + t0]);
            len = __ldg(&c.JR_S[r + t1]) - s0;
        }
        uint32_t incl = warp_incl_scan(len);
        uint32_t excl = incl - len;
        uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        for (uint32_t base = 0; base < total; base += 32) {
            uint32_t ci = base + lane;
            int lo = 0;
#pragma unroll
            for (int step = 16; step >= 1; step >>= 1) {
                uint32_t v = __shfl_sync(0xffffffffu, incl, lo + step - 1);
                if (v <= ci) lo += step;
            }
            uint32_t ks0 = __shfl_sync(0xffffffffu, s0, lo);
            uint32_t kex = __shfl_sync(0xffffffffu, excl, lo);
            bool isnew = false;
            uint32_t z = 0;
            if (ci < total) {
                z = __ldg(&c.IC_S[ks0 + (ci - kex)]);
                isnew = ins(z);
            }
            emit(isnew, z);
        }
    }
}

// Class 1: one warp per row, 2^warp_lg slots per warp.
template <bool WRITE>
__global__ void __launch_bounds__(256) k_rows_warp(RowCtx c, const uint32_t* __restrict__ rows,
                                                   const uint32_t* __restrict__ nrows_p, uint32_t warp_lg) {
    extern __shared__ uint32_t smem[];
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = lane_id();
    uint32_t* tab = smem + ((size_t)wib << warp_lg);
    const uint32_t nrows = *nrows_p;
    for (uint32_t ri = blockIdx.x * nw + wib; ri < nrows; ri += gridDim.x * nw) {
        const uint32_t x = rows[ri];
        uint32_t lg = ceil_log2(2 * c.ucap[x]);
        lg = lg < 5 ? 5 : (lg > warp_lg ? warp_lg : lg);
        for (uint32_t s = lane; s < (1u << lg); s += 32) tab[s] = kEmpty32;
        __syncwarp();
        uint32_t count = 0;
        unsigned long long base = 0;
        uint32_t lim = 0, xv = 0;
        if (WRITE) {
            base = c.off[x];
            lim = c.cnt[x];
            xv = c.id2x[x];
        }
        auto ins = [&](uint32_t z) { return smem_set_insert(tab, lg, z, c.err); };
        auto emit = [&](bool isnew, uint32_t z) {
            uint32_t b = __ballot_sync(0xffffffffu, isnew);
            if (WRITE && isnew) {
                uint32_t pos = count + __popc(b & lanemask_lt());
                if (pos < lim) c.out[base + pos] = make_uint2(xv, __ldg(&c.id2z[z]));
                else raise_error(c.err, kErrOutputBound);
            }
            count += __popc(b);
        };
        warp_expand(c, c.JR_R[x], c.JR_R[x + 1], 0, 32, 0, c.T, ins, emit);
        if (!WRITE && lane == 0) c.cnt[x] = count;
        __syncwarp();
    }
}

// Class 2: one CTA per row, 2^block_lg slots.
template <bool WRITE>
__global__ void __launch_bounds__(256) k_rows_block(RowCtx c, const uint32_t* __restrict__ rows,
                                                    const uint32_t* __restrict__ nrows_p, uint32_t block_lg) {
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t s_count;
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = lane_id();
    const uint32_t nrows = *nrows_p;
    for (uint32_t ri = blockIdx.x; ri < nrows; ri += gridDim.x) {
        const uint32_t x = rows[ri];
        uint32_t lg = ceil_log2(2 * c.ucap[x]);
        lg = lg < 5 ? 5 : (lg > block_lg ? block_lg : lg);
        for (uint32_t s = threadIdx.x; s < (1u << lg); s += blockDim.x) smem[s] = kEmpty32;
        if (threadIdx.x == 0) s_count = 0;
        __syncthreads();
        unsigned long long base = 0;
        uint32_t lim = 0, xv = 0, wcount = 0;
        if (WRITE) {
            base = c.off[x];
            lim = c.cnt[x];
            xv = c.id2x[x];
        }
        auto ins = [&](uint32_t z) { return smem_set_insert(smem, lg, z, c.err); };
        auto emit = [&](bool isnew, uint32_t z) {
            uint32_t b = __ballot_sync(0xffffffffu, isnew);
            if (WRITE) {
                uint32_t pb = 0;
                if (lane == 0 && b) pb = atomicAdd(&s_count, (uint32_t)__popc(b));
                pb = __shfl_sync(0xffffffffu, pb, 0);
                if (isnew) {
                    uint32_t pos = pb + __popc(b & lanemask_lt());
                    if (pos < lim) c.out[base + pos] = make_uint2(xv, __ldg(&c.id2z[z]));
                    else raise_error(c.err, kErrOutputBound);
                }
            } else {
                wcount += __popc(b);
            }
        };
        warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib * 32, nw * 32, 0, c.T, ins, emit);
        if (!WRITE && lane == 0 && wcount) atomicAdd(&s_count, wcount);
        __syncthreads();
        if (!WRITE && threadIdx.x == 0) c.cnt[x] = s_count;
        __syncthreads();
    }
}

// Class 3: one CTA per row, a bitmap over one z tile at a time.
template <bool WRITE>
__global__ void __launch_bounds__(512) k_rows_bitmap(RowCtx c, const uint32_t* __restrict__ rows,
                                                     const uint32_t* __restrict__ nrows_p) {
    extern __shared__ uint32_t bm[];
    __shared__ uint32_t s_count;
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = lane_id();
    const uint32_t nrows = *nrows_p;
    for (uint32_t ri = blockIdx.x; ri < nrows; ri += gridDim.x) {
        const uint32_t x = rows[ri];
        if (threadIdx.x == 0) s_count = 0;
        unsigned long long base = 0;
        uint32_t lim = 0, xv = 0, wcount = 0;
        if (WRITE) {
            base = c.off[x];
            lim = c.cnt[x];
            xv = c.id2x[x];
        }
        for (uint32_t t = 0; t < c.T; t++) {
            const uint32_t lo = t * c.tile_width;
            const uint32_t width = min(c.tile_width, c.m - lo);
            const uint32_t words = (width + 31) >> 5;
            for (uint32_t w = threadIdx.x; w < words; w += blockDim.x) bm[w] = 0;
            __syncthreads();
            auto ins = [&](uint32_t z) {
                uint32_t zl = z - lo, bit = 1u << (zl & 31);
                uint32_t old = atomicOr(&bm[zl >> 5], bit);
                return (old & bit) == 0;
            };
            auto emit = [&](bool isnew, uint32_t z) {
                uint32_t b = __ballot_sync(0xffffffffu, isnew);
                if (WRITE) {
                    uint32_t pb = 0;
                    if (lane == 0 && b) pb = atomicAdd(&s_count, (uint32_t)__popc(b));
                    pb = __shfl_sync(0xffffffffu, pb, 0);
                    if (isnew) {
                        uint32_t pos = pb + __popc(b & lanemask_lt());
                        if (pos < lim) c.out[base + pos] = make_uint2(xv, __ldg(&c.id2z[z]));
                        else raise_error(c.err, kErrOutputBound);
                    }
                } else {
                    wcount += __popc(b);
                }
            };
            warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib * 32, nw * 32, t, t + 1, ins, emit);
            __syncthreads();
        }
        if (!WRITE && lane == 0 && wcount) atomicAdd(&s_count, wcount);
        __syncthreads();
        if (!WRITE && threadIdx.x == 0) c.cnt[x] = s_count;
        __syncthreads();
    }
}

// Per-row candidate count w = sum over y in R_x of |S_y|, u = min(w, m) and
// the row class (0: empty).  One warp per row.
// With check_range set (join-aggregate, 32-bit per-group counters) a row of
// 2^32 or more candidates raises kErrCountRange.
__global__ void k_row_work(RowCtx c, uint32_t n, uint32_t cap_w, uint32_t cap_b, bool check_range,
                           uint32_t* __restrict__ ucap, uint8_t* __restrict__ cls, unsigned long long* outj) {
    const uint32_t lane = lane_id();
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long acc = 0;
    for (uint64_t x = gw; x < n; x += nwarps) {
        uint32_t e0 = c.JR_R[x], e1 = c.JR_R[x + 1];
        unsigned long long w = 0;
        for (uint32_t e = e0 + lane; e < e1; e += 32) {
            uint64_t r = (uint64_t)c.IC_R[e] * c.T;
            w += c.JR_S[r + c.T] - c.JR_S[r];
        }
        w = warp_sum(w);
        if (lane == 0) {
            uint32_t u = (uint32_t)(w < c.m ? w : c.m);
            ucap[x] = u;
            cls[x] = u == 0 ? 0 : (u <= cap_w ? 1 : (u <= cap_b ? 2 : 3));
            if (check_range && w >= 0xFFFFFFFFull) raise_error(c.err, kErrCountRange);
            acc += w;
        }
    }
    if (lane == 0 && acc) atomicAdd(outj, acc);
}

struct ClassSrc {
    const uint8_t* cls;
    uint8_t want;
    __device__ uint64_t operator()(uint64_t i) const { return cls[i] == want ? 1u : 0u; }
};
struct ListDst {
    uint32_t* list;
    __device__ void operator()(uint64_t i, uint64_t e, uint64_t v) const {
        if (v) list[e] = (uint32_t)i;
    }
};
struct OffDst {
    unsigned long long* off;
    __device__ void operator()(uint64_t i, uint64_t e, uint64_t) const { off[i] = e; }
};

}  // namespace dim3g

// mapping.cuh -- value -> dense id mapping on the GPU (the role of the
// reference's mapping_step + LS_mapper, dim3.hpp:394-883 and
// Include/L+S_mapper.hpp:11-160), plus the CSR builds (divide_R
// dim3.hpp:1058-1086, the sparse half of divide_S dim3.hpp:1186-1253).
//
// Table layout: one 64-bit slot per entry, key in the high half, dense id in
// the low half; the all-ones word marks an empty slot, so every 32-bit key
// (0xFFFFFFFF included) is a valid key.  Open addressing with linear probing
// at load factor <= 1/2; ids are assigned after the build by a prefix sum
// over occupied slots, so they are dense in [0, count).
#pragma once
#include "common.cuh"
#include "scan.cuh"

namespace dim3g {

constexpr uint32_t kNotFound = 0xFFFFFFFFu;

struct DevTable {
    unsigned long long* slots;
    uint64_t mask;       // capacity - 1 (capacity is a power of two)
    uint64_t limit = 0;  // longest probe (0: the whole table)
};

__device__ __forceinline__ bool table_insert(DevTable t, uint32_t key, uint32_t* err) {
    uint64_t h = mix32(key) & t.mask;
    const unsigned long long want = (unsigned long long)key << 32;
    const uint64_t lim = t.limit ? t.limit : t.mask;
    for (uint64_t p = 0; p <= lim; p++) {
        unsigned long long cur = __ldcg(&t.slots[h]);
        if (cur == kEmpty64) {
            unsigned long long prev = atomicCAS(&t.slots[h], (unsigned long long)kEmpty64, want);
            if (prev == kEmpty64) return true;
            cur = prev;
        }
        if ((uint32_t)(cur >> 32) == key) return false;
        h = (h + 1) & t.mask;
    }
    raise_error(err, kErrProbeLimit);
    return false;
}

__device__ __forceinline__ uint32_t table_find(DevTable t, uint32_t key) {
    uint64_t h = mix32(key) & t.mask;
    const uint64_t lim = t.limit ? t.limit : t.mask;
    for (uint64_t p = 0; p <= lim; p++) {
        unsigned long long cur = __ldg(&t.slots[h]);
        if (cur == kEmpty64) return kNotFound;
        if ((uint32_t)(cur >> 32) == key) return (uint32_t)cur;
        h = (h + 1) & t.mask;
    }
    return kNotFound;
}

// Table sizing.  A table built for a relation's tuple count (load factor
// 1/2 if every key were distinct) is far larger than its distinct keys when
// keys repeat -- 2^26 slots, 512 MB, for the 2M vertices of a 20M-edge graph
// -- and every insert and probe then misses the L2.  A HyperLogLog sketch
// (2^kSketchLg registers, one pass, about 2.3 % standard error) of the three
// key columns sizes each table to about 1.5x its distinct keys instead.
// Probes of a sketch-sized table are bounded by kSizedProbeLimit; a build
// that exceeds it (a table fuller than the sketch said) is redone with the
// tuple-sized tables, so the result never depends on the estimate.
constexpr uint32_t kSketchLg = 11, kSketchRegs = 1u << kSketchLg;
constexpr uint64_t kSizedProbeLimit = 1u << 12;

// A key's register (the hash's top kSketchLg bits) and rank (leading zeros
// of the rest, plus one).
__device__ __forceinline__ uint2 sketch_slot(uint32_t key) {
    const unsigned long long h = mix64((unsigned long long)key + 0x9E3779B97F4A7C15ull);
    const unsigned long long w = h << kSketchLg;
    return make_uint2((uint32_t)(h >> (64 - kSketchLg)), (w ? (uint32_t)__clzll(w) : 64u - kSketchLg) + 1);
}
__device__ __forceinline__ void sketch_add(uint32_t* r, uint32_t key) {
    const uint2 s = sketch_slot(key);
    atomicMax(&r[s.x], s.y);
}

inline uint64_t next_pow2(uint64_t v) {
    uint64_t p = 1;
    while (p < v) p <<= 1;
    return p;
}

// sketch_add without the atomic when the register already holds the rank
// (most updates once the registers have filled).
__device__ __forceinline__ void sketch_add_if_larger(uint32_t* r, uint32_t key) {
    const uint2 s = sketch_slot(key);
    if (*(volatile uint32_t*)&r[s.x] < s.y) atomicMax(&r[s.x], s.y);
}

// HyperLogLog estimate (with the small-range correction) from a column's
// register sum (sum of 2^-r) and count of zero registers; the table slots for
// it, slack_pct slots per estimated key, a power of two no larger than full.
inline double sketch_estimate(double sum, uint32_t zeros) {
    const double M = kSketchRegs;
    double e = 0.7213 / (1.0 + 1.079 / M) * M * M / sum;
    if (e <= 2.5 * M && zeros) e = M * log(M / zeros);
    return e;
}
inline uint64_t sketch_capacity(double est, uint64_t full, uint32_t slack_pct) {
    const uint64_t cap = next_pow2((uint64_t)(slack_pct / 100.0 * est) + 1024);
    return cap < full ? cap : full;
}

// Registers of P's first and y columns and Q's first column, kSketchRegs
// each, merged into regs (zeroed by the caller).
static __global__ void __launch_bounds__(256) k_sketch(const uint2* __restrict__ P, uint64_t nP,
                                                       const uint2* __restrict__ Q, uint64_t nQ, uint32_t* regs) {
    __shared__ uint32_t r[3 * kSketchRegs];
    for (uint32_t k = threadIdx.x; k < 3 * kSketchRegs; k += blockDim.x) r[k] = 0;
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nP; i += stride) {
        const uint2 p = P[i];
        sketch_add_if_larger(r, p.x);
        sketch_add_if_larger(r + kSketchRegs, p.y);
    }
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nQ; i += stride)
        sketch_add_if_larger(r + 2 * kSketchRegs, Q[i].x);
    __syncthreads();
    for (uint32_t k = threadIdx.x; k < 3 * kSketchRegs; k += blockDim.x)
        if (r[k]) atomicMax(&regs[k], r[k]);
}

// Build pass over the larger relation P: insert its first column into tx and
// its y column into ty.
static __global__ void k_insert_p(const uint2* __restrict__ P, uint64_t n, DevTable tx, DevTable ty, uint32_t* err) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint2 p = P[i];
        table_insert(tx, p.x, err);
        table_insert(ty, p.y, err);
    }
}

// Semi-join of Q against ty (mapping_y's probe, dim3.hpp:816-827): keep the
// tuples whose y occurs in P as (c, y id), insert their first column into tz.
static __global__ void k_probe_q(const uint2* __restrict__ Q, uint64_t n, DevTable ty, DevTable tz, uint2* __restrict__ Qk,
                          unsigned long long* nkept, uint32_t* err) {
    for (uint64_t i0 = (uint64_t)blockIdx.x * blockDim.x; i0 < n; i0 += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t i = i0 + threadIdx.x;
        bool keep = false;
        uint2 q = make_uint2(0, 0);
        uint32_t yid = kNotFound;
        if (i < n) {
            q = Q[i];
            yid = table_find(ty, q.y);
            keep = (yid != kNotFound);
            if (keep) table_insert(tz, q.x, err);
        }
        uint32_t b = __ballot_sync(0xffffffffu, keep);
        if (b) {
            unsigned long long base = 0;
            int leader = __ffs(b) - 1;
            if ((int)lane_id() == leader) base = atomicAdd(nkept, (unsigned long long)__popc(b));
            base = __shfl_sync(0xffffffffu, base, leader);
            if (keep) Qk[base + __popc(b & lanemask_lt())] = make_uint2(q.x, yid);
        }
    }
}

// Table compaction: ids by prefix sum over occupied slots.
struct OccupiedSrc {
    const unsigned long long* slots;
    __device__ uint64_t operator()(uint64_t i) const { return slots[i] != kEmpty64 ? 1u : 0u; }
};
struct AssignIdDst {
    unsigned long long* slots;
    uint32_t* id2v;
    __device__ void operator()(uint64_t i, uint64_t e, uint64_t v) const {
        if (!v) return;
        unsigned long long s = slots[i];
        uint32_t key = (uint32_t)(s >> 32);
        slots[i] = ((unsigned long long)key << 32) | (uint32_t)e;
        if (id2v) id2v[e] = key;
    }
};

// P -> (x id, y id); per-x degree histogram.
static __global__ void k_map_p(const uint2* __restrict__ P, uint64_t n, DevTable tx, DevTable ty, uint2* __restrict__ Pm,
                        uint32_t* __restrict__ degx) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint2 p = P[i];
        uint32_t xi = table_find(tx, p.x);
        uint32_t yi = table_find(ty, p.y);
        Pm[i] = make_uint2(xi, yi);
        atomicAdd(&degx[xi], 1u);
    }
}

// Q' = (z value, y id) -> z id; histogram over the (y, z tile) CSR key
// y*T + z/TB.
static __global__ void k_map_q(const uint2* __restrict__ Qk, uint64_t n, DevTable tz, uint32_t T, uint32_t tile_shift,
                        uint32_t* __restrict__ zid, uint32_t* __restrict__ cnt_yt) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint2 q = Qk[i];
        uint32_t zi = table_find(tz, q.x);
        zid[i] = zi;
        atomicAdd(&cnt_yt[(uint64_t)q.y * T + (zi >> tile_shift)], 1u);
    }
}

// Row pointers from a histogram: JR[i] = cursor[i] = exclusive prefix.
struct U32Src {
    const uint32_t* a;
    __device__ uint64_t operator()(uint64_t i) const { return a[i]; }
};
struct RowPtrDst {
    uint32_t* jr;
    uint32_t* cursor;
    __device__ void operator()(uint64_t i, uint64_t e, uint64_t) const {
        jr[i] = (uint32_t)e;
        cursor[i] = (uint32_t)e;
    }
};

static __global__ void k_scatter_r(const uint2* __restrict__ Pm, uint64_t n, uint32_t* __restrict__ cursor,
                            uint32_t* __restrict__ ic) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint2 p = Pm[i];
        uint32_t pos = atomicAdd(&cursor[p.x], 1u);
        ic[pos] = p.y;
    }
}

// S CSR by (y id, z tile): z ids into ic and, beside them, z values into vs
// (the write pass emits values without a gather through id2z).
// vs, isv (either may be null): the z values beside the ids, and the z id
// and z value of each entry side by side for the expansion paths that emit
// values (one 8-byte load or copy per candidate).
static __global__ void k_scatter_s(const uint2* __restrict__ Qk, const uint32_t* __restrict__ zid, uint64_t n, uint32_t T,
                            uint32_t tile_shift, uint32_t* __restrict__ cursor, uint32_t* __restrict__ ic,
                            uint32_t* __restrict__ vs, uint2* __restrict__ isv) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint2 q = Qk[i];
        uint32_t zi = zid[i];
        uint32_t pos = atomicAdd(&cursor[(uint64_t)q.y * T + (zi >> tile_shift)], 1u);
        ic[pos] = zi;
        if (vs) vs[pos] = q.x;
        if (isv) isv[pos] = make_uint2(zi, q.x);
    }
}

}  // namespace dim3g

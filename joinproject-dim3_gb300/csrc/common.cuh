// common.cuh -- shared device helpers for the DIM3 GB300 join-project path.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace dim3g {

constexpr int kWarp = 32;
constexpr uint64_t kEmpty64 = ~0ull;

// Error flags written by kernels into a device word; the host reads it after
// each call and turns any set bit into a status code.
enum DeviceError : uint32_t {
    kErrProbeLimit = 1u,    // an open-addressing probe ran past the table size
    kErrTableFull = 2u,     // a shared-memory table overflowed its sizing bound
    kErrOutputBound = 4u,   // a write-pass position ran past the row's count
    kErrCountRange = 8u,    // a per-group count could exceed 32 bits
    kErrDenseTimeout = 16u, // a wait of the dense product ran out of time
    kErrStreamTimeout = 32u,  // a wait of the streamed bitmap rows ran out of time
};

__device__ __forceinline__ void raise_error(uint32_t* err, uint32_t bit) { atomicOr(err, bit); }

// murmur3 fmix32: the GPU tables use their own mixing hash (the reference's
// identity hash clusters adjacent keys under linear probing).
__device__ __forceinline__ uint32_t mix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}

// Order-independent hashes of output pairs and groups (summaries): the
// splitmix64 finaliser of x << 32 | z, and of that plus the group's count.
__device__ __forceinline__ unsigned long long mix64(unsigned long long v) {
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ull;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebull;
    return v ^ (v >> 31);
}
__device__ __forceinline__ unsigned long long pair_hash(uint32_t x, uint32_t z) {
    return mix64(((unsigned long long)x << 32) | z);
}
__device__ __forceinline__ unsigned long long group_hash(uint32_t x, uint32_t z, unsigned long long count) {
    return mix64(pair_hash(x, z) + count);
}

// Per-A-tile summary accumulators: tile(a) = mix32(a) & mask; three words a
// tile (groups, count sum, hash sum).  Rows whose tile is outside [lo, hi)
// are skipped.
struct SumAcc {
    unsigned long long* tiles;  // nullptr: no summary (outputs are written)
    uint32_t mask, lo, hi;
    __device__ __forceinline__ uint32_t tile(uint32_t a) const { return mix32(a) & mask; }
    __device__ __forceinline__ bool selected(uint32_t a) const {
        const uint32_t t = tile(a);
        return t >= lo && t < hi;
    }
    // warp-collective: adds the lanes' partial sums to a's tile
    __device__ __forceinline__ void commit(uint32_t a, unsigned long long groups, unsigned long long count_sum,
                                           unsigned long long hash) const {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            groups += __shfl_xor_sync(0xffffffffu, groups, o);
            count_sum += __shfl_xor_sync(0xffffffffu, count_sum, o);
            hash += __shfl_xor_sync(0xffffffffu, hash, o);
        }
        if ((threadIdx.x & 31) == 0 && groups) {
            unsigned long long* t = tiles + 3ull * tile(a);
            atomicAdd(&t[0], groups);
            atomicAdd(&t[1], count_sum);
            atomicAdd(&t[2], hash);
        }
    }
};

// L2 residency: the CSR rows are re-read by many x rows and should stay in
// L2, while the output pairs stream through once.  Loads of CSR data carry
// an evict_last policy; output stores use the evict-first (.cs) path.
__device__ __forceinline__ uint64_t l2_keep_policy() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint32_t ld_keep(const uint32_t* a, uint64_t pol) {
    uint32_t v;
    asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ uint2 ld_keep2(const uint2* a, uint64_t pol) {
    uint2 v;
    asm volatile("ld.global.nc.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;" : "=r"(v.x), "=r"(v.y) : "l"(a), "l"(pol));
    return v;
}
__device__ __forceinline__ void st_stream(uint2* a, uint2 v) { __stcs(a, v); }
// Asks L2 to fetch the bytes [lo, hi) (a hint: no data returns to the SM).
// The range is shrunk to 16-byte boundaries inside it -- the bulk prefetch
// wants a 16-byte aligned start and a multiple of 16 bytes -- and to at most
// kPrefetchMax bytes, so nothing outside [lo, hi) is named.
constexpr uint32_t kPrefetchMax = 32u << 10;
__device__ __forceinline__ void l2_prefetch(const void* lo, const void* hi, uint64_t pol) {
    const uint64_t a = (reinterpret_cast<uint64_t>(lo) + 15) & ~15ull;
    uint64_t e = reinterpret_cast<uint64_t>(hi) & ~15ull;
    if (e > a + kPrefetchMax) e = a + kPrefetchMax;
    if (e > a)
        asm volatile("cp.async.bulk.prefetch.L2.global.L2::cache_hint [%0], %1, %2;" ::"l"(a), "r"((uint32_t)(e - a)),
                     "l"(pol)
                     : "memory");
}

__device__ __forceinline__ uint32_t lane_id() { return threadIdx.x & 31; }
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Warp-aggregated increment: every calling lane adds 1 to base[key]; lanes
// sharing a key get consecutive old values from one atomic (skewed keys
// would otherwise serialise on one address).  Returns the lane's old value.
__device__ __forceinline__ uint32_t atomic_inc_agg(uint32_t* base, uint64_t key) {
    const unsigned act = __activemask();
    const unsigned grp = __match_any_sync(act, key);
    const int leader = __ffs(grp) - 1;
    uint32_t old = 0;
    if ((int)(threadIdx.x & 31) == leader) old = atomicAdd(&base[key], (uint32_t)__popc(grp));
    old = __shfl_sync(grp, old, leader);
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    return old + __popc(grp & lt);
}

// Adds v of every calling lane into *dst, lanes grouped by key (the lanes of
// a group pass the same dst): one atomic per group.  v < 2^48 (larger
// values are added by the lane alone).  The group sum is formed from three
// 16-bit slices, each of whose sums fits 32 bits.
__device__ __forceinline__ void atomic_add_grouped(unsigned long long* dst, uint64_t key, unsigned long long v) {
    if (v >> 48) {
        atomicAdd(dst, v);
        v = 0;
    }
    const unsigned act = __activemask();
    const unsigned grp = __match_any_sync(act, key);
    const unsigned a = __reduce_add_sync(grp, (unsigned)(v & 0xFFFFu));
    const unsigned b = __reduce_add_sync(grp, (unsigned)((v >> 16) & 0xFFFFu));
    const unsigned c = __reduce_add_sync(grp, (unsigned)(v >> 32));
    if ((int)(threadIdx.x & 31) == __ffs(grp) - 1) {
        const unsigned long long s =
            (unsigned long long)a + ((unsigned long long)b << 16) + ((unsigned long long)c << 32);
        if (s) atomicAdd(dst, s);
    }
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Inclusive warp scan.
template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T t = __shfl_up_sync(0xffffffffu, v, o);
        if ((int)lane_id() >= o) v += t;
    }
    return v;
}

// Exclusive block scan of one value per thread; returns the prefix and the
// block total through *total.  smem must hold BLOCK/32 + 1 T.
template <int BLOCK, typename T>
__device__ __forceinline__ T block_excl_scan(T v, T* smem, T* total) {
    constexpr int NW = BLOCK / 32;
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    T inc = warp_incl_scan(v);
    if (l == 31) smem[w] = inc;
    __syncthreads();
    if (w == 0) {
        T s = (l < NW) ? smem[l] : T(0);
        T si = warp_incl_scan(s);
        if (l < NW) smem[l] = si - s;
        if (l == NW - 1) smem[NW] = si;
    }
    __syncthreads();
    T r = smem[w] + inc - v;
    *total = smem[NW];
    __syncthreads();
    return r;
}

}  // namespace dim3g

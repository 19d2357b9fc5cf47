// scan.cuh -- device-wide exclusive prefix sums (reduce / scan-of-sums /
// apply), driven by functors so one pass both computes and consumes the
// prefix (CSR row pointers, table compaction, output offsets).
#pragma once
#include "common.cuh"

namespace dim3g {

constexpr int kScanBlock = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanBlock * kScanItems;

// Src:  __device__ uint64_t operator()(uint64_t i) const      -- value of item i
// Dst:  __device__ void operator()(uint64_t i, uint64_t excl, uint64_t v) const
template <class Src>
__global__ void __launch_bounds__(kScanBlock) k_scan_reduce(Src src, uint64_t n, uint64_t* block_sums) {
    __shared__ uint64_t sm[kScanBlock / 32 + 1];
    uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    uint64_t acc = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        uint64_t i = base + (uint64_t)k * kScanBlock + threadIdx.x;
        if (i < n) acc += src(i);
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint64_t t = 0;
        for (int w = 0; w < kScanBlock / 32; w++) t += sm[w];
        block_sums[blockIdx.x] = t;
    }
}

// Single-block exclusive scan of nb block sums in place; writes the grand
// total to *total.
static __global__ void __launch_bounds__(1024) k_scan_sums(uint64_t* sums, uint64_t nb, unsigned long long* total) {
    __shared__ uint64_t sm[1024 / 32 + 1];
    uint64_t carry = 0;
    for (uint64_t c = 0; c < nb; c += 1024) {
        uint64_t i = c + threadIdx.x;
        uint64_t v = i < nb ? sums[i] : 0;
        uint64_t t;
        uint64_t e = block_excl_scan<1024>(v, sm, &t);
        if (i < nb) sums[i] = carry + e;
        carry += t;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}

template <class Src, class Dst>
__global__ void __launch_bounds__(kScanBlock) k_scan_apply(Src src, uint64_t n, const uint64_t* block_sums, Dst dst) {
    __shared__ uint64_t sm[kScanBlock / 32 + 1];
    uint64_t base = (uint64_t)blockIdx.x * kScanTile;
    // Each thread owns kScanItems consecutive items so the scan order is the
    // item order.
    uint64_t v[kScanItems];
    uint64_t local = 0;
    uint64_t first = base + (uint64_t)threadIdx.x * kScanItems;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        uint64_t i = first + k;
        v[k] = i < n ? src(i) : 0;
        local += v[k];
    }
    uint64_t t;
    uint64_t e = block_excl_scan<kScanBlock>(local, sm, &t) + block_sums[blockIdx.x];
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        uint64_t i = first + k;
        if (i < n) dst(i, e, v[k]);
        e += v[k];
    }
}

// Host driver.  block_sums must hold scan_storage(n) entries; total
// (device) receives the sum of all items.  Up to kScanSumsDirect block sums
// are scanned by one CTA; more are scanned by the same three kernels one
// level up (their own block sums stored after them).
inline uint64_t scan_blocks(uint64_t n) { return (n + kScanTile - 1) / kScanTile; }
constexpr uint64_t kScanSumsDirect = 32768;
inline uint64_t scan_storage(uint64_t n) {
    uint64_t nb = scan_blocks(n), s = nb + 1;
    while (nb > kScanSumsDirect) {
        nb = scan_blocks(nb);
        s += nb + 1;
    }
    return s;
}
// Number of kernel launches device_scan makes for n items.
inline uint64_t scan_launches(uint64_t n) {
    uint64_t nb = scan_blocks(n), k = 0;
    if (nb == 0) return 0;
    k = 3;
    while (nb > kScanSumsDirect) {
        nb = scan_blocks(nb);
        k += 2;
    }
    return k;
}

struct SumsSrc {
    const uint64_t* a;
    __device__ uint64_t operator()(uint64_t i) const { return a[i]; }
};
// In place: k_scan_apply reads all items of a thread before writing them.
struct SumsDst {
    uint64_t* a;
    __device__ void operator()(uint64_t i, uint64_t e, uint64_t) const { a[i] = e; }
};

// A scan whose length is only known on the device: items at or past *lim
// count as 0 and are neither read nor written (the launch still covers the
// host's upper bound n, and blocks past the limit do no memory traffic).
template <class Src>
struct BoundSrc {
    Src s;
    const unsigned long long* lim;
    __device__ uint64_t operator()(uint64_t i) const { return i < *lim ? s(i) : 0u; }
};
template <class Dst>
struct BoundDst {
    Dst d;
    const unsigned long long* lim;
    __device__ void operator()(uint64_t i, uint64_t e, uint64_t v) const {
        if (i < *lim) d(i, e, v);
    }
};

template <class Src, class Dst>
inline void device_scan(Src src, Dst dst, uint64_t n, uint64_t* block_sums, unsigned long long* total, cudaStream_t st);

inline void scan_block_sums(uint64_t* sums, uint64_t nb, unsigned long long* total, cudaStream_t st) {
    if (nb <= kScanSumsDirect) k_scan_sums<<<1, 1024, 0, st>>>(sums, nb, total);
    else device_scan(SumsSrc{sums}, SumsDst{sums}, nb, sums + nb + 1, total, st);
}

template <class Src, class Dst>
inline void device_scan(Src src, Dst dst, uint64_t n, uint64_t* block_sums, unsigned long long* total, cudaStream_t st) {
    uint64_t nb = scan_blocks(n);
    if (nb == 0) {
        if (total) cudaMemsetAsync(total, 0, sizeof(uint64_t), st);
        return;
    }
    k_scan_reduce<<<(unsigned)nb, kScanBlock, 0, st>>>(src, n, block_sums);
    scan_block_sums(block_sums, nb, total, st);
    k_scan_apply<<<(unsigned)nb, kScanBlock, 0, st>>>(src, n, block_sums, dst);
}

}  // namespace dim3g

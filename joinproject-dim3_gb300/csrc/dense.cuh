// dense.cuh -- the dense block of the join-project on the tensor cores: the
// GPU form of Hybrid_solution's dense part (dim3.hpp:894-950), where the
// reference tests X_row AND Z_col over bitmaps of y for every (x, dense z).
//
// Here the heavy rows X_d (the bitmap classes) are joined through the K join
// values y with the largest candidate mass deg_Xd(y) * deg_S(y) as one
// matrix product on tcgen05:
//   A (|X_d| x K)  A[i][h] = multiplicity of (x_i, y_h) in R   (fp8 e4m3)
//   B (m x K)      B[z][h] = multiplicity of (z, y_h) in S
//   C = A * B^T    f32 accumulators in TMEM: the number of join tuples of
//                  (x_i, z) through the K values, exact: multiplicities are
//                  at most 16 (exact in e4m3) and K at most 4096, so
//                  C <= 16 * 16 * 4096 = 2^20 < 2^24
// (the join-project writes 1.0 for any multiplicity; only C > 0 matters).
// The other (light) join values of the heavy rows go through a sparse pass.
//   join-project: the epilogue keeps one bit per (x_i, z), C > 0, in a
//     row-major bitmap D (|X_d| x m); the light candidates are OR-ed in and
//     the rows' pairs are emitted from it.
//   per-A-tile summaries: the light candidates are bucketed by product tile
//     and the epilogue adds them to C group by group, summing groups,
//     counts and group hashes per A-tile; nothing is materialised.
// Either way the result is exact: a bit or a group exists iff some y joins
// x and z, and a group's count is its number of join tuples.
//
// The product is a persistent kernel, one CTA per SM: warp 0 loads A and B
// tiles with TMA (128-byte swizzle) through a 4-stage shared-memory ring,
// warp 1 issues the MMAs (one thread; 128 x 256 x 32 per instruction) into
// one of two TMEM accumulators, and the epilogue warps (8 for the bitmap,
// 16 for summaries) read the other accumulator (tcgen05.ld).  Every wait on
// an mbarrier is bounded by time; a wait that runs out sets
// kErrDenseTimeout, stops the CTA's loops, and the CTA still frees its TMEM
// before it exits.
#pragma once
#include <cuda.h>

#include "common.cuh"

namespace dim3g {

constexpr uint32_t kDenseBM = 128;          // rows of A (x) per tile = TMEM lanes
constexpr uint32_t kDenseBN = 256;          // rows of B (z) per tile = TMEM columns
constexpr uint32_t kDenseBK = 128;          // K bytes (fp8 elements) per stage = one 128-byte swizzle row
constexpr uint32_t kDenseStages = 4;
constexpr uint32_t kDenseAStage = kDenseBM * kDenseBK;  // 16 KB
constexpr uint32_t kDenseBStage = kDenseBN * kDenseBK;  // 32 KB
constexpr uint32_t kDenseSmem = kDenseStages * (kDenseAStage + kDenseBStage) + 1024 + 256;
constexpr uint32_t kDenseThreads = 320;     // bitmap mode: TMA warp, MMA warp, 8 epilogue warps
constexpr uint32_t kDenseSumThreads = 576;  // summary modes: 16 epilogue warps (the group hashes are ALU work)
constexpr uint32_t kDenseTmemCols = 2 * kDenseBN;  // two accumulators
constexpr uint32_t kDenseBins = 512;               // candidate-mass bins: 8 per octave
constexpr uint8_t kFp8One = 0x38;                  // e4m3 1.0
constexpr unsigned long long kDenseWaitNs = 2000000000ull;  // 2 s per wait

// Candidate-mass bin of c > 0: 8 * floor(log2 c) + the next three bits.
__device__ __forceinline__ uint32_t dense_bin(unsigned long long c) {
    const uint32_t lg = 63 - __clzll(c);
    const uint32_t frac = (uint32_t)((c << (63 - lg)) >> 60) & 7u;
    return lg * 8 + frac;
}

// ------------------------------------------------------- heavy-y selection
// deg_d[y] += 1 for every R entry of every step-th heavy row (warp per
// row).  The heavy set only steers the cost, never the result, so a sample
// of the rows estimates it (and keeps the atomics off the hottest y).
static __global__ void k_dense_deg(const uint32_t* __restrict__ JR_R, const uint32_t* __restrict__ IC_R,
                                   const uint32_t* __restrict__ rows, uint32_t nd, uint32_t step,
                                   uint32_t* __restrict__ deg_d) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * step; i < nd; i += nw * step) {
        const uint32_t x = rows[i];
        for (uint32_t e = JR_R[x] + lane; e < JR_R[x + 1]; e += 32) atomicAdd(&deg_d[IC_R[e]], 1u);
    }
}

__device__ __forceinline__ unsigned long long dense_mass(const uint32_t* deg_d, const uint32_t* JR_S, uint32_t T,
                                                         uint32_t y) {
    return (unsigned long long)deg_d[y] * (JR_S[(unsigned long long)(y + 1) * T] - JR_S[(unsigned long long)y * T]);
}

// Per-bin count and candidate mass of the join values.
static __global__ void k_dense_bins(const uint32_t* __restrict__ deg_d, const uint32_t* __restrict__ JR_S, uint32_t T,
                                    uint32_t k, unsigned int* __restrict__ bin_n,
                                    unsigned long long* __restrict__ bin_mass) {
    for (uint32_t y = blockIdx.x * blockDim.x + threadIdx.x; y < k; y += gridDim.x * blockDim.x) {
        const unsigned long long c = dense_mass(deg_d, JR_S, T, y);
        if (c == 0) continue;
        const uint32_t b = dense_bin(c);
        atomicAdd(&bin_n[b], 1u);
        atomicAdd(&bin_mass[b], c);
    }
}

// Column of every heavy join value (bin >= cut), -1 for the others; hy
// lists the heavy values by column.
static __global__ void k_dense_hid(const uint32_t* __restrict__ deg_d, const uint32_t* __restrict__ JR_S, uint32_t T,
                                   uint32_t k, uint32_t cut, int32_t* __restrict__ hid, uint32_t* __restrict__ hy,
                                   unsigned int* __restrict__ kcnt) {
    for (uint32_t y = blockIdx.x * blockDim.x + threadIdx.x; y < k; y += gridDim.x * blockDim.x) {
        const unsigned long long c = dense_mass(deg_d, JR_S, T, y);
        int32_t h = -1;
        if (c != 0 && dense_bin(c) >= cut) {
            h = (int32_t)atomicAdd(kcnt, 1u);
            hy[h] = y;
        }
        hid[y] = h;
    }
}

// ------------------------------------------------------------ operands
// A[i][hid[y]] = 1 for the heavy entries of heavy row i (warp per row).
static __global__ void k_dense_fill_a(const uint32_t* __restrict__ JR_R, const uint32_t* __restrict__ IC_R,
                                      const uint32_t* __restrict__ rows, uint32_t nd, const int32_t* __restrict__ hid,
                                      uint8_t* __restrict__ A, uint32_t Kp) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nd; i += nw) {
        const uint32_t x = rows[i];
        for (uint32_t e = JR_R[x] + lane; e < JR_R[x + 1]; e += 32) {
            const int32_t h = hid[IC_R[e]];
            if (h >= 0) A[(size_t)i * Kp + h] = kFp8One;
        }
    }
}

// B[z][h] = 1 for every S entry (z, hy[h]); blockIdx.y = column h, the
// x blocks split its S row.
static __global__ void k_dense_fill_b(const uint32_t* __restrict__ JR_S, const uint32_t* __restrict__ IC_S, uint32_t T,
                                      const uint32_t* __restrict__ hy, uint8_t* __restrict__ B, uint32_t Kp) {
    const uint32_t h = blockIdx.y, y = hy[h];
    const uint32_t e1 = JR_S[(unsigned long long)(y + 1) * T];
    for (uint32_t e = JR_S[(unsigned long long)y * T] + blockIdx.x * blockDim.x + threadIdx.x; e < e1;
         e += gridDim.x * blockDim.x)
        B[(size_t)IC_S[e] * Kp + h] = kFp8One;
}

// Summary modes: the product counts join tuples, so the operands hold
// multiplicities (duplicate tuples count): first as 32-bit counts, then
// as e4m3 codes, exact for integers up to 16 (a larger multiplicity sets
// *flag and the caller keeps the sparse path).
static __global__ void k_dense_cnt_a(const uint32_t* __restrict__ JR_R, const uint32_t* __restrict__ IC_R,
                                     const uint32_t* __restrict__ rows, uint32_t nd, const int32_t* __restrict__ hid,
                                     uint32_t* __restrict__ A32, uint32_t Kp) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nd; i += nw) {
        const uint32_t x = rows[i];
        for (uint32_t e = JR_R[x] + lane; e < JR_R[x + 1]; e += 32) {
            const int32_t h = hid[IC_R[e]];
            if (h >= 0) atomicAdd(&A32[(size_t)i * Kp + h], 1u);
        }
    }
}
static __global__ void k_dense_cnt_b(const uint32_t* __restrict__ JR_S, const uint32_t* __restrict__ IC_S, uint32_t T,
                                     const uint32_t* __restrict__ hy, uint32_t* __restrict__ B32, uint32_t Kp) {
    const uint32_t h = blockIdx.y, y = hy[h];
    const uint32_t e1 = JR_S[(unsigned long long)(y + 1) * T];
    for (uint32_t e = JR_S[(unsigned long long)y * T] + blockIdx.x * blockDim.x + threadIdx.x; e < e1;
         e += gridDim.x * blockDim.x)
        atomicAdd(&B32[(size_t)IC_S[e] * Kp + h], 1u);
}
__device__ __forceinline__ uint8_t e4m3_of(uint32_t v) {  // exact for v <= 16
    if (v == 0) return 0;
    const uint32_t e = 31 - __clz(v);
    return (uint8_t)(((e + 7) << 3) | (((v << 3) >> e) & 7u));
}
static __global__ void k_dense_to_fp8(const uint32_t* __restrict__ src, uint8_t* __restrict__ dst, size_t n,
                                      uint32_t* flag) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const uint32_t v = src[i];
        if (v > 16) *flag = 1;
        dst[i] = e4m3_of(v);
    }
}

// ------------------------------------------------ PTX: mbarrier, TMA, tcgen05
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait for the phase of `parity`; false when it ran out or another
// role of the CTA gave up (abort flag).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, volatile uint32_t* abort) {
    if (mbar_try(bar, parity)) return true;
    const unsigned long long t0 = global_ns();
    while (!mbar_try(bar, parity)) {
        if (*abort) return false;
        if (global_ns() - t0 > kDenseWaitNs) return false;
    }
    return true;
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, uint32_t bar, uint32_t c0,
                                            uint32_t c1) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];"
        ::"r"(dst), "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor of a K-major tile in the 128-byte swizzle
// layout (rows of 128 bytes, 8-row groups 1024 bytes apart), as TMA writes it.
__device__ __forceinline__ uint64_t dense_desc(uint32_t saddr) {
    return (uint64_t)((saddr & 0x3FFFFu) >> 4)  // start address
           | ((uint64_t)1 << 16)                // leading byte offset (unused for this layout)
           | ((uint64_t)(1024 >> 4) << 32)      // stride byte offset: 8 rows x 128 B
           | ((uint64_t)1 << 46)                // descriptor version
           | ((uint64_t)2 << 61);               // 128-byte swizzle
}

// Instruction descriptor: kind::f8f6f4, A and B e4m3, D f32, both K-major,
// N = 256, M = 128.
constexpr uint32_t kDenseIdesc = (1u << 4) | ((kDenseBN >> 3) << 17) | ((kDenseBM >> 4) << 24);

__device__ __forceinline__ void dense_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f8f6f4 [%0], %1, %2, %3, p;\n\t}"
        ::"r"(d_tmem), "l"(a), "l"(b), "r"(kDenseIdesc), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void dense_commit(uint32_t bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}

// 32 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]), "=r"(v[8]),
          "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]), "=r"(v[16]),
          "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]), "=r"(v[24]),
          "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// ------------------------------------------------------------ the product
// Epilogue modes: the bitmap (join-project), or per-A-tile summaries of the
// groups (join-project summary: pair hashes; COUNT summary: group hashes of
// the exact counts) with each tile's light candidates added in.
enum DenseMode : int { kDenseBits = 0, kDenseSumProject = 1, kDenseSumCount = 2 };

struct DenseSum {
    const uint32_t* rows;  // block rows (x ids)
    uint32_t nd;
    const uint32_t* id2x;
    const uint32_t* id2z;
    const uint32_t* toff;  // light candidates of tile t: lb[toff[t] .. toff[t + 1])
    const uint16_t* lb;    // (row in tile << 8) | (z in tile)
    SumAcc sum;
};

// pair_hash(a, c) = splitmix64 finaliser of a << 32 | c, with the terms
// that depend on the row's a alone hoisted out: after the first shift-xor
// the high word is a ^ (a >> 30) and the low word c ^ (a << 2) ^ (c >> 30),
// and the high word's share of the first product is a constant shifted
// into the high half.  Equal to pair_hash for every a, c.
struct PairRow {
    uint32_t a2;             // a << 2
    unsigned long long k1;   // ((a ^ (a >> 30)) * low word of the multiplier) << 32
};
__device__ __forceinline__ PairRow pair_row(uint32_t a) {
    return PairRow{a << 2, (unsigned long long)((a ^ (a >> 30)) * 0x1ce4e5b9u) << 32};
}
__device__ __forceinline__ unsigned long long pair_hash_row(const PairRow& r, uint32_t c) {
    unsigned long long v = (unsigned long long)(c ^ r.a2 ^ (c >> 30)) * 0xbf58476d1ce4e5b9ull + r.k1;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebull;
    return v ^ (v >> 31);
}
// An exact f32 integer below 2^23 as an integer: one add, no conversion.
__device__ __forceinline__ uint32_t count_of(uint32_t fbits) {
    return __float_as_uint(__uint_as_float(fbits) + 8388608.0f) - 0x4B000000u;
}

// Adds a group's summary terms; light corrections replace a group's count.
template <int kMode>
__device__ __forceinline__ void dense_group(uint32_t a, uint32_t c, uint32_t cnt, unsigned long long& g,
                                            unsigned long long& cs, unsigned long long& h) {
    g += 1;
    if (kMode == kDenseSumCount) {
        cs += cnt;
        h += group_hash(a, c, cnt);
    } else {
        cs += 1;
        h += pair_hash(a, c);
    }
}

// Summary of one 32-column chunk of a tile row: the product's counts v,
// then the tile's light candidates of this row and chunk (each distinct
// (row, z) once, with the number of its entries as its light count).
template <int kMode>
__device__ __forceinline__ void dense_sum_chunk(const uint32_t (&v)[32], const DenseSum& ds, uint32_t a,
                                                const PairRow& pr, uint32_t z0,
                                                uint32_t key0, uint32_t l0, uint32_t l1, unsigned long long& g,
                                                unsigned long long& cs, unsigned long long& h) {
    // branch-free over the 32 columns so their hash chains interleave; the
    // chunk's z values 4 at a time in vector loads (z0 is a multiple of 32)
#pragma unroll
    for (uint32_t q = 0; q < 8; q++) {
        const uint4 t = __ldg(reinterpret_cast<const uint4*>(ds.id2z + z0) + q);
        const uint32_t zq[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
        for (uint32_t r = 0; r < 4; r++) {
            const uint32_t cnt = count_of(v[4 * q + r]);
            const bool p = cnt != 0;
            const unsigned long long ph = pair_hash_row(pr, zq[r]);
            const unsigned long long hv = kMode == kDenseSumCount ? mix64(ph + cnt) : ph;
            h += p ? hv : 0ull;
            g += p;
            cs += kMode == kDenseSumCount ? cnt : (uint32_t)p;
        }
    }
    for (uint32_t k = l0; k < l1; k++) {
        const uint32_t e = ds.lb[k];
        if ((e & ~31u) != key0) continue;  // another row or chunk
        uint32_t L = 0;
        bool first = true;
        for (uint32_t k2 = l0; k2 < l1; k2++)
            if (ds.lb[k2] == e) {
                L++;
                if (k2 < k) first = false;
            }
        if (!first) continue;
        const uint32_t u = e & 31;
        uint32_t bv = 0;
#pragma unroll
        for (uint32_t w = 0; w < 32; w++) bv = w == u ? v[w] : bv;
        const uint32_t base = (uint32_t)__uint_as_float(bv);
        const uint32_t c = ds.id2z[z0 + u];
        if (kMode == kDenseSumCount) {
            if (base) {
                h -= group_hash(a, c, base);
                g -= 1;
                cs -= base;
            }
            dense_group<kMode>(a, c, base + L, g, cs, h);
        } else if (!base) {
            dense_group<kMode>(a, c, 1, g, cs, h);
        }
    }
}

// Adds a lane's sums to its row's A-tile (warp-reduced when the warp's
// rows share one tile).
__device__ __forceinline__ void dense_sum_flush(const SumAcc& sum, uint32_t tile, unsigned long long g,
                                                unsigned long long cs, unsigned long long h) {
    const uint32_t t0 = __shfl_sync(0xffffffffu, tile, 0);
    if (__all_sync(0xffffffffu, tile == t0)) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            g += __shfl_xor_sync(0xffffffffu, g, o);
            cs += __shfl_xor_sync(0xffffffffu, cs, o);
            h += __shfl_xor_sync(0xffffffffu, h, o);
        }
        if ((threadIdx.x & 31) == 0 && g) {
            unsigned long long* t = sum.tiles + 3ull * t0;
            atomicAdd(&t[0], g);
            atomicAdd(&t[1], cs);
            atomicAdd(&t[2], h);
        }
    } else if (g) {
        unsigned long long* t = sum.tiles + 3ull * tile;
        atomicAdd(&t[0], g);
        atomicAdd(&t[1], cs);
        atomicAdd(&t[2], h);
    }
}

// kDenseBits: D[i][z / 32] bit z % 32 = (A_i . B_z > 0) for i < mt * 128,
// z < nt * 256; D has Wd 32-bit words per row (Wd >= nt * 8).  Summary
// modes: the groups of block rows i < ds.nd go into ds.sum; tiles are taken
// row-block-major so an epilogue thread keeps its row across ~nt / grid
// consecutive tiles.  nk = K bytes / 128.
template <int kMode>
static __global__ void __launch_bounds__(kMode == kDenseBits ? kDenseThreads : kDenseSumThreads, 1)
    k_dense_mma(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                uint32_t* __restrict__ D, uint32_t Wd, uint32_t mt, uint32_t nt, uint32_t nk, uint32_t* err,
                const DenseSum ds) {
    extern __shared__ uint8_t dsm_raw[];
    const uint32_t raw = smem_addr(dsm_raw);
    const uint32_t base = (raw + 1023u) & ~1023u;  // 128-byte swizzle tiles sit on 1 KB boundaries
    const uint32_t sA = base;
    const uint32_t sB = base + kDenseStages * kDenseAStage;
    const uint32_t sBar = sB + kDenseStages * kDenseBStage;
    uint8_t* gen = dsm_raw + (sBar - raw);
    // barriers: full[S], empty[S], tfull[2], tempty[2]; then the TMEM address and the abort flag
    const uint32_t full = sBar, empty = sBar + 8 * kDenseStages, tfull = sBar + 16 * kDenseStages,
                   tempty = tfull + 16;
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(gen + 16 * kDenseStages + 32);
    volatile uint32_t* abort = reinterpret_cast<volatile uint32_t*>(gen + 16 * kDenseStages + 36);

    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (uint32_t s = 0; s < kDenseStages; s++) {
            mbar_init(full + 8 * s, 1);
            mbar_init(empty + 8 * s, 1);
        }
        for (uint32_t b = 0; b < 2; b++) {
            mbar_init(tfull + 8 * b, 1);
            mbar_init(tempty + 8 * b, blockDim.x - 64);
        }
        *abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(tmem_slot)),
                     "r"(kDenseTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t ntile = mt * nt;
    bool bad = false;

    if (warp == 0 && lane == 0) {
        // producer: A and B tiles of every K block into the ring
        uint32_t s = 0, ph = 0;
        for (uint32_t t = blockIdx.x; t < ntile && !bad; t += gridDim.x) {
            const uint32_t mi = kMode == kDenseBits ? t % mt : t / nt, ni = kMode == kDenseBits ? t / mt : t % nt;
            for (uint32_t kb = 0; kb < nk; kb++) {
                if (!mbar_wait(empty + 8 * s, ph ^ 1, abort)) {
                    bad = true;
                    break;
                }
                mbar_expect_tx(full + 8 * s, kDenseAStage + kDenseBStage);
                tma_load_2d(sA + s * kDenseAStage, &tmA, full + 8 * s, kb * kDenseBK, mi * kDenseBM);
                tma_load_2d(sB + s * kDenseBStage, &tmB, full + 8 * s, kb * kDenseBK, ni * kDenseBN);
                if (++s == kDenseStages) {
                    s = 0;
                    ph ^= 1;
                }
            }
        }
    } else if (warp == 1 && lane == 0) {
        // MMA issuer: one thread
        uint32_t s = 0, ph = 0, tb = 0, tph = 0;
        for (uint32_t t = blockIdx.x; t < ntile && !bad; t += gridDim.x) {
            if (!mbar_wait(tempty + 8 * tb, tph ^ 1, abort)) {
                bad = true;
                break;
            }
            tc_fence_after();
            const uint32_t d = tmem + tb * kDenseBN;
            for (uint32_t kb = 0; kb < nk; kb++) {
                if (!mbar_wait(full + 8 * s, ph, abort)) {
                    bad = true;
                    break;
                }
                tc_fence_after();
                const uint64_t da = dense_desc(sA + s * kDenseAStage), db = dense_desc(sB + s * kDenseBStage);
#pragma unroll
                for (uint32_t kk = 0; kk < kDenseBK / 32; kk++)  // 32 fp8 of K per MMA: +32 B = +2 encoded
                    dense_mma(d, da + 2 * kk, db + 2 * kk, (kb | kk) != 0);
                dense_commit(empty + 8 * s);
                if (++s == kDenseStages) {
                    s = 0;
                    ph ^= 1;
                }
            }
            if (bad) break;
            dense_commit(tfull + 8 * tb);
            if (++tb == 2) {
                tb = 0;
                tph ^= 1;
            }
        }
    } else if (warp >= 2) {
        // epilogue: warp w reads TMEM lanes 32q..32q+31 (q = w % 4; a warp
        // may only reach its own quadrant) and part hc of the columns: halves
        // (8 epilogue warps) or quarters (16)
        const uint32_t q = warp & 3, hc = (warp - 2) >> 2;
        const uint32_t parts = (blockDim.x - 64) / 128, pcols = kDenseBN / parts;
        const uint32_t row = q * 32 + lane;
        uint32_t tb = 0, tph = 0;
        // summary state: this lane's row (block row cur_mi * 128 + row)
        uint32_t cur_mi = ~0u, a = 0, stile = 0;
        PairRow pr{0, 0};
        bool live = false;
        unsigned long long g = 0, cs = 0, h = 0;
        for (uint32_t t = blockIdx.x; t < ntile && !bad; t += gridDim.x) {
            const uint32_t mi = kMode == kDenseBits ? t % mt : t / nt, ni = kMode == kDenseBits ? t / mt : t % nt;
            __syncwarp();
            if (kMode != kDenseBits && mi != cur_mi) {
                // a new row block: the sums are per A-tile, so a lane keeps
                // accumulating while its rows stay in one tile; flush when
                // some lane with sums moves to another
                const uint32_t i = mi * kDenseBM + row;
                const bool nlive = i < ds.nd;
                const uint32_t na = nlive ? ds.id2x[ds.rows[i]] : 0u;
                const uint32_t ntl = nlive ? ds.sum.tile(na) : 0u;
                if (!__all_sync(0xffffffffu, !g || !nlive || ntl == stile)) {
                    dense_sum_flush(ds.sum, stile, g, cs, h);
                    g = cs = h = 0;
                }
                if (nlive) stile = ntl;
                cur_mi = mi;
                a = na;
                pr = pair_row(na);
                live = nlive;
            }
            // warp-uniform outcome: the TMEM loads below are warp-collective
            if (!__all_sync(0xffffffffu, mbar_wait(tfull + 8 * tb, tph, abort))) {
                bad = true;
                break;
            }
            tc_fence_after();
            if (kMode != kDenseBits) {
                const uint32_t l0 = ds.toff[t], l1 = ds.toff[t + 1];
#pragma unroll 1
                for (uint32_t j = 0; j < pcols / 32; j++) {
                    uint32_t v[32];
                    __syncwarp();  // tcgen05.ld is warp-collective; the sums before it diverge
                    tmem_ld32(tmem + ((q * 32) << 16) + tb * kDenseBN + hc * pcols + j * 32, v);
                    if (j == pcols / 32 - 1) {
                        tc_fence_before();
                        mbar_arrive(tempty + 8 * tb);  // the accumulator is in registers
                    }
                    if (live)
                        dense_sum_chunk<kMode>(v, ds, a, pr, ni * kDenseBN + hc * pcols + j * 32,
                                               (row << 8) | (hc * pcols + j * 32), l0, l1, g, cs, h);
                }
                if (++tb == 2) {
                    tb = 0;
                    tph ^= 1;
                }
                continue;
            }
            uint32_t w[kDenseBN / 64];
#pragma unroll
            for (uint32_t j = 0; j < kDenseBN / 64; j++) {
                uint32_t v[32];
                tmem_ld32(tmem + ((q * 32) << 16) + tb * kDenseBN + hc * (kDenseBN / 2) + j * 32, v);
                uint32_t bits = 0;
#pragma unroll
                for (uint32_t c = 0; c < 32; c++) bits |= (__uint_as_float(v[c]) > 0.0f ? 1u : 0u) << c;
                w[j] = bits;
            }
            tc_fence_before();
            mbar_arrive(tempty + 8 * tb);
            *reinterpret_cast<uint4*>(D + ((size_t)mi * kDenseBM + row) * Wd + (size_t)ni * (kDenseBN / 32) + hc * 4) =
                make_uint4(w[0], w[1], w[2], w[3]);
            if (++tb == 2) {
                tb = 0;
                tph ^= 1;
            }
        }
        __syncwarp();
        if (kMode != kDenseBits && !bad) dense_sum_flush(ds.sum, stile, g, cs, h);
    }
    if (bad) {
        *abort = 1;
        atomicOr(err, kErrDenseTimeout);
        // let this thread's copies or MMAs in flight land before the CTA ends
        const unsigned long long t0 = global_ns();
        while (global_ns() - t0 < 1000000ull) {
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kDenseTmemCols)
                     : "memory");
}

// ------------------------------------------------------------ light pass
// The light join values of every block row: their S rows' z are OR-ed into
// the row's bitmap (warp per row; an atomic only for a bit not yet set).
// The row's entries are taken 32 at a time, one per lane (their S rows'
// bounds loaded in parallel).  When the batch's light S rows average 32 z or
// more, the warp streams them one after another; otherwise a warp prefix sum
// over their lengths flattens the candidates, which the lanes take 32 at a
// time, each finding its entry by a 5-step search over the prefix.
// The largest bucket of light candidates (summaries apply a tile's bucket
// in the epilogue, each epilogue thread scanning it, so it must be small).
constexpr uint32_t kDenseBucketMax = 64;
static __global__ void k_dense_maxcnt(const uint32_t* __restrict__ tcnt, uint64_t n, unsigned int* out) {
    uint32_t m = 0;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        m = tcnt[i] > m ? tcnt[i] : m;
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0 && m) atomicMax(out, m);
}

// The visitor takes every light candidate (block row i, z id).
struct LightOr {  // join-project: into the bitmap
    uint32_t* D;
    uint32_t Wd;
    __device__ __forceinline__ void operator()(uint32_t i, uint32_t z) const {
        uint32_t* w = D + (size_t)i * Wd + (z >> 5);
        const uint32_t bit = 1u << (z & 31);
        if (!(*w & bit)) atomicOr(w, bit);
    }
};
struct LightCount {  // summaries: candidates per product tile
    uint32_t* tcnt;
    uint32_t nt;
    __device__ __forceinline__ void operator()(uint32_t i, uint32_t z) const {
        atomicAdd(&tcnt[(size_t)(i / kDenseBM) * nt + z / kDenseBN], 1u);
    }
};
struct LightScatter {  // summaries: candidates into their tile's bucket
    uint32_t* tcur;
    uint16_t* lb;
    uint32_t nt;
    __device__ __forceinline__ void operator()(uint32_t i, uint32_t z) const {
        const uint32_t p = atomicAdd(&tcur[(size_t)(i / kDenseBM) * nt + z / kDenseBN], 1u);
        lb[p] = (uint16_t)(((i % kDenseBM) << 8) | (z % kDenseBN));
    }
};

template <class V>
static __global__ void k_dense_light(const uint32_t* __restrict__ JR_R, const uint32_t* __restrict__ IC_R,
                                     const uint32_t* __restrict__ JR_S, const uint32_t* __restrict__ IC_S, uint32_t T,
                                     const uint32_t* __restrict__ rows, uint32_t nd, const int32_t* __restrict__ hid,
                                     V visit) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nd; i += nw) {
        const uint32_t x = rows[i];
        const uint32_t e1 = JR_R[x + 1];
        for (uint32_t eb = JR_R[x]; eb < e1; eb += 32) {
            const uint32_t e = eb + lane;
            uint32_t s0 = 0, len = 0;
            if (e < e1) {
                const uint32_t y = IC_R[e];
                if (hid[y] < 0) {
                    s0 = JR_S[(unsigned long long)y * T];
                    len = JR_S[(unsigned long long)(y + 1) * T] - s0;
                }
            }
            uint32_t incl = len;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
                if ((int)lane >= o) incl += v;
            }
            const uint32_t excl = incl - len;
            const uint32_t tot = __shfl_sync(0xffffffffu, incl, 31);
            uint32_t lights = __ballot_sync(0xffffffffu, len != 0);
            if (tot >= 32u * __popc(lights)) {
                while (lights) {
                    const uint32_t l = __ffs(lights) - 1;
                    lights &= lights - 1;
                    const uint32_t os = __shfl_sync(0xffffffffu, s0, l), n = __shfl_sync(0xffffffffu, len, l);
                    for (uint32_t j = lane; j < n; j += 32) visit(i, IC_S[os + j]);
                }
                continue;
            }
            for (uint32_t j0 = 0; j0 < tot; j0 += 32) {
                const uint32_t j = j0 + lane;
                uint32_t pos = 0;  // first lane whose inclusive prefix exceeds j
#pragma unroll
                for (uint32_t st = 16; st > 0; st >>= 1)
                    if (__shfl_sync(0xffffffffu, incl, pos + st - 1) <= j) pos += st;
                const uint32_t os = __shfl_sync(0xffffffffu, s0, pos);
                const uint32_t oe = __shfl_sync(0xffffffffu, excl, pos);
                if (j < tot) visit(i, IC_S[os + (j - oe)]);
            }
        }
    }
}

// ------------------------------------------------------------ emission
// The bitmap is read in chunks of 32 words (1024 z): chunk c is chunk
// c % cpr of block row c / cpr.  Pairs are placed by an exclusive prefix
// over the chunks' popcounts, so a row's pairs are contiguous (x-grouped)
// and the chunks running at one time write adjacent ranges.
constexpr uint32_t kDenseEmitSmem = 8 * 2 * 1024 * 4;  // two 1024-entry z buffers per warp, 8 warps

// cc[c] = set bits of chunk c (8 lanes per chunk, 16 bytes a lane); cc[nc] = 0.
static __global__ void k_dense_chunks(uint32_t nd, const uint32_t* __restrict__ D, uint32_t Wd, uint32_t cpr,
                                      uint32_t* __restrict__ cc) {
    const uint64_t nq = (uint64_t)nd * cpr * 8;                  // 4-word quads
    const uint64_t lim = (nq + 31) & ~31ull;                     // whole warps stay in the loop
    for (uint64_t g = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; g < lim;
         g += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t v = 0;
        if (g < nq) {
            const uint32_t row = (uint32_t)(g / ((uint64_t)cpr * 8)), w = (uint32_t)(g % ((uint64_t)cpr * 8)) * 4;
            if (w < Wd) {  // words past Wd (chunk padding) are empty
                const uint4 t = *reinterpret_cast<const uint4*>(D + (size_t)row * Wd + w);
                v = __popc(t.x) + __popc(t.y) + __popc(t.z) + __popc(t.w);
            }
        }
        v += __shfl_xor_sync(0xffffffffu, v, 1);
        v += __shfl_xor_sync(0xffffffffu, v, 2);
        v += __shfl_xor_sync(0xffffffffu, v, 4);
        if (g < nq && (g & 7) == 0) cc[g >> 3] = v;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) cc[(uint64_t)nd * cpr] = 0;
}

// Distinct count of every block row: cnt[x] from the chunk offsets.
static __global__ void k_dense_rowcnt(const uint32_t* __restrict__ rows, uint32_t nd, uint32_t cpr,
                                      const unsigned long long* __restrict__ coff, uint32_t* __restrict__ cnt) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nd; i += gridDim.x * blockDim.x)
        cnt[rows[i]] = (uint32_t)(coff[(uint64_t)(i + 1) * cpr] - coff[(uint64_t)i * cpr]);
}

// Single pass: the block's pairs take one range of the cursor (total =
// coff[nd * cpr]); *base = its start, or ~0 when it ends past cap.
static __global__ void k_dense_reserve(const unsigned long long* __restrict__ total, unsigned long long* cursor,
                                       unsigned long long cap, unsigned long long* base) {
    const unsigned long long t = *total;
    const unsigned long long b = atomicAdd(cursor, t);
    *base = b + t <= cap ? b : ~0ull;
}

__device__ __forceinline__ void dense_zcopy(uint32_t dst, const uint32_t* src, uint32_t lane) {
#pragma unroll
    for (uint32_t q = 0; q < 8; q++)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst + (q * 32 + lane) * 16),
                     "l"(src + (q * 32 + lane) * 4)
                     : "memory");
}

struct DenseChunk {
    uint32_t bits, xv;
    unsigned long long base;
};

// Pairs (x value, z value) of the block.  ordered: row x's pairs start at
// off[x]; otherwise at *base0 + the chunk offset (nothing when *base0 is ~0,
// a reservation past the capacity).  A warp takes chunks c, c + warps, ...;
// the chunk's 1024 z values (id2z holds whole 1024-entry chunks) are copied
// into the warp's shared buffer one chunk ahead (cp.async), with its bitmap
// word and placement loaded into registers one chunk ahead too.  For bit
// position t every lane tests bit (lane + t) % 32 of its word (conflict-free
// shared reads) and the set bits are written as one contiguous run.
static __global__ void __launch_bounds__(256) k_dense_emit(
    const uint32_t* __restrict__ rows, uint32_t nd, const uint32_t* __restrict__ D, uint32_t Wd, uint32_t Wm,
    uint32_t cpr, const unsigned long long* __restrict__ coff, const uint32_t* __restrict__ id2x,
    const uint32_t* __restrict__ id2z, uint2* __restrict__ out, const unsigned long long* __restrict__ off,
    const unsigned long long* __restrict__ base0) {
    extern __shared__ __align__(16) uint32_t zsm[];
    const uint32_t lane = threadIdx.x & 31, lt = (1u << lane) - 1u;
    uint32_t* const zw = zsm + (threadIdx.x >> 5) * 2048;
    const uint32_t zs = smem_addr(zw);
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    const uint64_t nc = (uint64_t)nd * cpr;
    unsigned long long b0 = 0;
    if (!off) {
        b0 = *base0;
        if (b0 == ~0ull) return;
    }
    auto fetch = [&](uint64_t c, uint32_t buf) {
        const uint32_t row = (uint32_t)(c / cpr), j = (uint32_t)(c % cpr), w = j * 32 + lane;
        DenseChunk k;
        k.bits = w < Wm ? D[(size_t)row * Wd + w] : 0u;
        const uint32_t x = rows[row];
        k.xv = id2x[x];
        k.base = off ? off[x] + coff[c] - coff[(uint64_t)row * cpr] : b0 + coff[c];
        dense_zcopy(zs + buf * 4096, id2z + (size_t)j * 1024, lane);
        return k;
    };
    uint64_t c = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    DenseChunk cur{0, 0, 0};
    if (c < nc) cur = fetch(c, 0);
    asm volatile("cp.async.commit_group;" ::: "memory");
    uint32_t buf = 0;
    for (; c < nc; c += nw) {
        const uint64_t n = c + nw;
        DenseChunk nxt{0, 0, 0};
        if (n < nc) nxt = fetch(n, buf ^ 1);
        asm volatile("cp.async.commit_group;" ::: "memory");
        asm volatile("cp.async.wait_group 1;" ::: "memory");
        __syncwarp();
        const uint32_t* z = zw + buf * 1024 + lane * 32;
        unsigned long long base = cur.base;
#pragma unroll
        for (uint32_t t = 0; t < 32; t++) {
            const uint32_t b = (lane + t) & 31;
            const bool p = (cur.bits >> b) & 1u;
            const uint32_t mk = __ballot_sync(0xffffffffu, p);
            if (p) st_stream(&out[base + __popc(mk & lt)], make_uint2(cur.xv, z[b]));
            base += __popc(mk);
        }
        __syncwarp();
        cur = nxt;
        buf ^= 1;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
}

}  // namespace dim3g

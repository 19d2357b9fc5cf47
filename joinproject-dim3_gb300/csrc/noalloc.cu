// noalloc.cu -- join-project for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc at the point where they need a join:
// code running under a custom or fixed-budget allocator that forbids the
// runtime's allocator, real-time or embedded hosts that preallocate
// everything at start-up, and pipelines that must not trigger the implicit
// device synchronisation an allocation can cause.  dim3g_join_project_noalloc
// serves them: it takes device inputs and a caller-provided output buffer,
// and keeps all of its scratch in one file-scope device array of fixed size,
// so it never calls cudaMalloc, cudaFree or any allocating routine.
//
// Costs and limits (stated in include/dim3gpu.h):
//   - every GPU that loads this library holds kScratchBytes (about 19 MB)
//     for the life of the process;
//   - the larger relation may hold at most DIM3G_NOALLOC_MAX_TUPLES tuples
//     and the result at most DIM3G_NOALLOC_MAX_PAIRS distinct pairs;
//   - all calls share the one array, so calls whose work overlaps on the GPU
//     (different streams, different host threads) race and corrupt each
//     other; serialise them.
// The scratch array's name is a host-side stand-in, not a device address;
// the host resolves the real address with cudaGetSymbolAddress, once per
// device, with that device current, on the first call made on that device.
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>

#include "../../include/dim3gpu.h"

namespace {

constexpr uint32_t kMaxTuples = DIM3G_NOALLOC_MAX_TUPLES;  // larger relation
constexpr uint32_t kMaxPairs = DIM3G_NOALLOC_MAX_PAIRS;    // distinct output pairs
constexpr uint32_t kBuckets = 1u << 19;                     // chain heads on the join key
constexpr uint32_t kPairSlots = 2 * kMaxPairs;              // pair set, load factor <= ~1/2
constexpr uint32_t kNil = 0xFFFFFFFFu;
constexpr unsigned long long kEmptyPair = ~0ull;

// Layout of the scratch array (byte offsets, 256-aligned).
constexpr size_t kOffHead = 0;
constexpr size_t kOffNext = kOffHead + (size_t)kBuckets * 4;
constexpr size_t kOffPairs = kOffNext + (size_t)kMaxTuples * 4;
constexpr size_t kOffCounters = kOffPairs + (size_t)kPairSlots * 8;
constexpr size_t kScratchBytes = kOffCounters + 256;

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// counters: [0] distinct pairs found, [1] flags (bit 1: a probe walked the
// whole pair table), [2] the all-ones pair seen
struct Scratch {
    uint32_t* head;
    uint32_t* next;
    unsigned long long* pairs;
    unsigned long long* counters;
};

__device__ __forceinline__ uint32_t mix32(uint32_t h) {
    h ^= h >> 16;
    h *= 0x85ebca6bu;
    h ^= h >> 13;
    h *= 0xc2b2ae35u;
    h ^= h >> 16;
    return h;
}
__device__ __forceinline__ unsigned long long mix64(unsigned long long v) {
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ull;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebull;
    return v ^ (v >> 31);
}

// Chained hash table on the larger relation's join key: next[i] links tuple
// i to the previous head of its bucket.
__global__ void k_na_build(const uint2* __restrict__ P, uint32_t nP, Scratch s) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nP; i += gridDim.x * blockDim.x)
        s.next[i] = atomicExch(&s.head[mix32(P[i].y) & (kBuckets - 1)], i);
}

__device__ __forceinline__ void emit(Scratch s, uint2* out, unsigned long long cap, uint32_t px, uint32_t qc) {
    unsigned long long pos = atomicAdd(&s.counters[0], 1ull);
    if (pos < cap) out[pos] = make_uint2(px, qc);
}

// Distinct-pair set: 64-bit keys (P.first << 32 | Q.first) with linear
// probing; the all-ones key is tracked by a flag.  New pairs are counted
// and, while they fit, written straight to the caller's buffer.
__device__ void insert_pair(Scratch s, uint2* out, unsigned long long cap, uint32_t px, uint32_t qc) {
    const unsigned long long key = ((unsigned long long)px << 32) | qc;
    if (key == kEmptyPair) {
        if (atomicExch(&s.counters[2], 1ull) == 0ull) emit(s, out, cap, px, qc);
        return;
    }
    uint32_t h = (uint32_t)mix64(key) & (kPairSlots - 1);
    for (uint32_t p = 0; p < kPairSlots; p++) {
        unsigned long long cur = ((volatile unsigned long long*)s.pairs)[h];
        if (cur == key) return;
        if (cur == kEmptyPair) {
            // The limit is decided after the fact: the counter only counts
            // pairs that were claimed, so once it is above the limit the
            // result is known to be too large and no more pairs are claimed
            // (the host reports it from the final count).  Threads that pass
            // this test together overshoot by at most the threads in flight,
            // which the table's 2x slot count absorbs.
            if (((volatile unsigned long long*)s.counters)[0] > kMaxPairs) return;
            unsigned long long prev = atomicCAS(&s.pairs[h], kEmptyPair, key);
            if (prev == kEmptyPair) {
                emit(s, out, cap, px, qc);
                return;
            }
            if (prev == key) return;
        }
        h = (h + 1) & (kPairSlots - 1);
    }
    atomicOr(&s.counters[1], 2ull);
}

// Probe with the smaller relation: every P tuple on the chain of q's key
// with the same key forms the candidate (P.first, q.first).
__global__ void k_na_probe(const uint2* __restrict__ P, const uint2* __restrict__ Q, uint32_t nQ, Scratch s,
                           uint2* out, unsigned long long cap) {
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < nQ; j += gridDim.x * blockDim.x) {
        const uint2 q = Q[j];
        for (uint32_t i = s.head[mix32(q.y) & (kBuckets - 1)]; i != kNil; i = s.next[i])
            if (P[i].y == q.y) insert_pair(s, out, cap, P[i].x, q.x);
    }
}

// Per-device scratch address and grid size, resolved once with that device
// current.
std::mutex g_setup_mutex;
std::atomic<unsigned char*> g_base[64];
int g_grid[64];

int scratch_for_device(int dev, unsigned char** base, int* grid) {
    if (dev < 0 || dev >= 64) return DIM3G_ERR_UNSUPPORTED;
    unsigned char* p = g_base[dev].load(std::memory_order_acquire);
    if (!p) {
        std::lock_guard<std::mutex> lock(g_setup_mutex);
        p = g_base[dev].load(std::memory_order_relaxed);
        if (!p) {
            int sms = 0;
            if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
                cudaGetLastError();
                return DIM3G_ERR_CUDA;
            }
            void* addr = nullptr;
            cudaError_t e = cudaGetSymbolAddress(&addr, g_scratch);
            if (e != cudaSuccess || !addr) {
                cudaGetLastError();
                return DIM3G_ERR_CUDA;
            }
            g_grid[dev] = 4 * sms;  // 4 CTAs of 256 threads per SM
            p = (unsigned char*)addr;
            g_base[dev].store(p, std::memory_order_release);
        }
    }
    *base = p;
    *grid = g_grid[dev];
    return DIM3G_OK;
}

bool aligned8(const void* p) { return ((uintptr_t)p & 7u) == 0; }

}  // namespace

extern "C" int dim3g_join_project_noalloc(const uint32_t* d_R, uint64_t nR, const uint32_t* d_S, uint64_t nS,
                                          uint32_t* d_out, uint64_t capacity, uint64_t* n_out, void* cuda_stream) {
    if (!n_out || (nR && !d_R) || (nS && !d_S) || (capacity && !d_out)) return DIM3G_ERR_INVALID;
    *n_out = 0;
    // the kernels read and write pairs as 8-byte words
    if (!aligned8(d_R) || !aligned8(d_S) || !aligned8(d_out)) return DIM3G_ERR_INVALID;
    // the larger relation drives the build, exactly the reference's swap
    const bool swap = nR < nS;
    const uint2* P = (const uint2*)(swap ? d_S : d_R);
    const uint2* Q = (const uint2*)(swap ? d_R : d_S);
    const uint64_t nP = swap ? nS : nR, nQ = swap ? nR : nS;
    if (nP == 0 || nQ == 0) return DIM3G_OK;            // an empty input joins to nothing
    if (nP > kMaxTuples) return DIM3G_ERR_UNSUPPORTED;  // beyond the fixed scratch
    // An error the caller left pending (from earlier, unrelated work) is
    // reported and left in place, not taken as this call's launch status.
    if (cudaPeekAtLastError() != cudaSuccess) return DIM3G_ERR_CUDA;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        return DIM3G_ERR_CUDA;
    }
    unsigned char* base = nullptr;
    int grid = 0;
    int r = scratch_for_device(dev, &base, &grid);
    if (r) return r;
    Scratch s{(uint32_t*)(base + kOffHead), (uint32_t*)(base + kOffNext), (unsigned long long*)(base + kOffPairs),
              (unsigned long long*)(base + kOffCounters)};
    cudaStream_t st = (cudaStream_t)cuda_stream;
    // the previous call's contents stay in the array: reset what must start
    // empty (chain heads, pair set, counters)
    if (cudaMemsetAsync(s.head, 0xff, (size_t)kBuckets * 4, st) != cudaSuccess ||
        cudaMemsetAsync(s.pairs, 0xff, (size_t)kPairSlots * 8, st) != cudaSuccess ||
        cudaMemsetAsync(s.counters, 0, 256, st) != cudaSuccess) {
        cudaGetLastError();
        return DIM3G_ERR_CUDA;
    }
    k_na_build<<<grid, 256, 0, st>>>(P, (uint32_t)nP, s);
    k_na_probe<<<grid, 256, 0, st>>>(P, Q, (uint32_t)nQ, s, (uint2*)d_out, capacity);
    unsigned long long h[2] = {0, 0};
    if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(h, s.counters, sizeof h, cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
        cudaGetLastError();
        return DIM3G_ERR_CUDA;
    }
    if (h[0] > kMaxPairs) return DIM3G_ERR_UNSUPPORTED;  // more distinct pairs than DIM3G_NOALLOC_MAX_PAIRS
    if (h[1] & 2ull) return DIM3G_ERR_DEVICE;
    *n_out = h[0];
    return h[0] > capacity ? DIM3G_ERR_CAPACITY : DIM3G_OK;
}

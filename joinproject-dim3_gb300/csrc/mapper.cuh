// mapper.cuh -- the L+S mapper interface on the GPU
// (LS_mapper, Include/L+S_mapper.hpp:11-160).
//
// A batch insert must give each key the id a sequence of the reference's
// insert() calls would give: an existing key keeps its id; a new key gets the
// next dense id in the order of its FIRST occurrence inside the batch.  Three
// passes do that without any ordering between threads:
//   claim   every occurrence i of a key stores min(i) in its slot
//           (slot low half = 0x80000000 | i; settled ids are < 0x80000000, so
//           a 64-bit atomicMin keeps an existing id and the smallest index)
//   rank    occurrences that hold their key's minimum are first occurrences;
//           a prefix sum over them in batch order gives the new ids
//   gather  every occurrence reads its key's id.
#pragma once
#include "common.cuh"
#include "mapping.cuh"
#include "scan.cuh"

namespace dim3g {

constexpr uint32_t kPendingBit = 0x80000000u;

static __global__ void k_mapper_claim(DevTable t, const uint32_t* __restrict__ keys, uint64_t n, uint32_t* err) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t key = keys[i];
        const unsigned long long want = ((unsigned long long)key << 32) | (kPendingBit | (uint32_t)i);
        uint64_t h = mix32(key) & t.mask;
        bool done = false;
        for (uint64_t p = 0; p <= t.mask && !done; p++) {
            unsigned long long cur = __ldcg(&t.slots[h]);
            if (cur == kEmpty64) {
                unsigned long long prev = atomicCAS(&t.slots[h], (unsigned long long)kEmpty64, want);
                if (prev == kEmpty64) { done = true; break; }
                cur = prev;
            }
            if ((uint32_t)(cur >> 32) == key) {
                atomicMin(&t.slots[h], want);
                done = true;
                break;
            }
            h = (h + 1) & t.mask;
        }
        if (!done) raise_error(err, kErrProbeLimit);
    }
}

__device__ __forceinline__ unsigned long long* mapper_slot(DevTable t, uint32_t key) {
    uint64_t h = mix32(key) & t.mask;
    for (uint64_t p = 0; p <= t.mask; p++) {
        unsigned long long cur = t.slots[h];
        if (cur == kEmpty64) return nullptr;
        if ((uint32_t)(cur >> 32) == key) return &t.slots[h];
        h = (h + 1) & t.mask;
    }
    return nullptr;
}

// first[i] = 1 when occurrence i is its key's first occurrence in the batch.
struct FirstOccSrc {
    DevTable t;
    const uint32_t* keys;
    __device__ uint64_t operator()(uint64_t i) const {
        unsigned long long* s = mapper_slot(t, keys[i]);
        return (s && (uint32_t)*s == (kPendingBit | (uint32_t)i)) ? 1u : 0u;
    }
};
struct AssignNewIdDst {
    DevTable t;
    const uint32_t* keys;
    long long base;
    __device__ void operator()(uint64_t i, uint64_t e, uint64_t v) const {
        if (!v) return;
        unsigned long long* s = mapper_slot(t, keys[i]);
        *s = ((unsigned long long)keys[i] << 32) | (uint32_t)(base + (long long)e);
    }
};

static __global__ void k_mapper_gather(DevTable t, const uint32_t* __restrict__ keys, uint64_t n, int32_t* __restrict__ ids) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        unsigned long long* s = mapper_slot(t, keys[i]);
        ids[i] = s ? (int32_t)(uint32_t)*s : -1;
    }
}

static __global__ void k_mapper_find(DevTable t, const uint32_t* __restrict__ keys, uint64_t n, int32_t* __restrict__ ids) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t id = table_find(t, keys[i]);
        ids[i] = id == kNotFound ? -1 : (int32_t)id;
    }
}

// Rehash every settled slot of `from` into `to` (capacity growth).
static __global__ void k_mapper_rehash(DevTable from, DevTable to, uint32_t* err) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i <= from.mask; i += (uint64_t)gridDim.x * blockDim.x) {
        unsigned long long v = from.slots[i];
        if (v == kEmpty64) continue;
        uint32_t key = (uint32_t)(v >> 32);
        uint64_t h = mix32(key) & to.mask;
        bool done = false;
        for (uint64_t p = 0; p <= to.mask; p++) {
            if (atomicCAS(&to.slots[h], (unsigned long long)kEmpty64, v) == kEmpty64) { done = true; break; }
            h = (h + 1) & to.mask;
        }
        if (!done) raise_error(err, kErrProbeLimit);
    }
}

}  // namespace dim3g

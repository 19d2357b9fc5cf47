// structures.hpp -- drop-in type names of the GPU join-project headers.
//
// The reference declares its hashers and CSR/dense structures in
// Include/structures.hpp:1-134.  The GPU path hashes with its own mixing
// function, so the hasher types are accepted for template-signature
// compatibility only; the structures keep their names and fields for code
// that declares them.
#pragma once

#include <cstdint>

#include "myBitVector.hpp"

using LL = long long;
using uLL = unsigned long long;

struct myHasher {
    inline uint32_t operator()(const int key) const { return (uint32_t)key; }
};

// The dense part of S in the reference's hybrid layout (structures.hpp:14-20):
// one bit vector per dense z over the y ids, with the z value and count.
struct S_DENSE {
    myBitVector<>* data;
    int* id2v;
    int* id2cnt;
    int size;
    int dense_bitvector_len;
};

template <typename _Tv = int>
struct CSR {
    int *JR, *IC;
    _Tv* VAL;
};

template <typename _Tx, typename _Tz>
struct ID2VALUE {
    _Tx* x;
    _Tz* z;
};

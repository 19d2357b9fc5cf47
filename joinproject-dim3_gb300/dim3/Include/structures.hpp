// structures.hpp -- drop-in type names of the GPU join-project headers.
//
// The reference declares its hashers and CSR/dense structures in
// Include/structures.hpp:1-134.  The GPU path hashes with its own mixing
// function, so the hasher types are accepted for template-signature
// compatibility only; the structures keep their names and fields for code
// that declares them.
#pragma once

#include <cstdint>

using LL = long long;
using uLL = unsigned long long;

struct myHasher {
    inline uint32_t operator()(const int key) const { return (uint32_t)key; }
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

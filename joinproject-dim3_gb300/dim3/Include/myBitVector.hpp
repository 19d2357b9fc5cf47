// myBitVector.hpp -- drop-in bit vector type of the GPU join-project headers.
//
// Same name, members and operations as the reference's myBitVector
// (Include/myBitVector.hpp:6-39): a malloc'd array of words `_Array`, bit
// `pos` at word pos / bits-per-word, bit pos % bits-per-word.  Code that
// declares the reference's S_DENSE (which holds these) keeps compiling; the
// GPU path keeps its own bitmaps on the device.
#pragma once

#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>

template <typename _T = int>
struct myBitVector {
    static_assert(sizeof(_T) == 1 || sizeof(_T) == 2 || sizeof(_T) == 4, "words of 1, 2 or 4 bytes");
    static constexpr int _Bitsperword = CHAR_BIT * (int)sizeof(_T);
    // log2 of the bits per word, and the mask of a bit's position in its word
    static constexpr int _Posshr = sizeof(_T) == 4 ? 5 : (sizeof(_T) == 2 ? 4 : 3);
    static constexpr int _Posmask = _Bitsperword - 1;

    _T* _Array = nullptr;

    myBitVector() {}
    // n words, all bits clear
    explicit myBitVector(int n) {
        _Array = (_T*)calloc(n > 0 ? (size_t)n : 1, sizeof(_T));
        if (!_Array) {
            printf("Failed to malloc an BitVector of %fG\n", (double)n * sizeof(_T) / 1073741824.0);
            exit(-1);
        }
    }
    inline void setTrue(int pos) { _Array[pos >> _Posshr] |= (_T)((_T)1 << (pos & _Posmask)); }
    inline bool checkIfTrue(int pos) { return (_Array[pos >> _Posshr] >> (pos & _Posmask)) & 1; }
    void clear(int n) { memset(_Array, 0, (size_t)n * sizeof(_T)); }
};

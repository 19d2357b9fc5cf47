// myvector.hpp -- drop-in container type of the GPU join-project headers.
//
// Same memory layout and members as the reference's myvector
// (Include/myvector.hpp:8-85): `T* data; Count cur_num; Count max_num;`
// with malloc/realloc-owned storage, so code written against the reference
// (and the C ABI, which fills `data` with malloc'd memory) keeps working.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <cstdint>

template <class T, typename _CountType = uint32_t>
struct myvector {
    T* data;
    _CountType cur_num;
    _CountType max_num;

    myvector(_CountType ini_size = 8) { init(ini_size); }

    void init(_CountType ini_size = 8) {
        max_num = ini_size;
        data = (T*)malloc(sizeof(T) * (max_num ? max_num : 1));
        cur_num = 0;
    }
    inline bool isEmpty() { return cur_num == 0; }
    void push_back(T x) {
        if (cur_num == max_num) {
            _CountType grown = max_num ? max_num * 2 : 8;
            if (grown <= max_num) {
                printf("myvector capacity overflow at %llu elements\n", (unsigned long long)max_num);
                exit(1);
            }
            T* p = (T*)realloc(data, sizeof(T) * grown);
            if (!p) {
                printf("Failed when resize myvector to %llu\n", (unsigned long long)grown);
                free(data);
                exit(1);
            }
            data = p;
            max_num = grown;
        }
        data[cur_num++] = x;
    }
    void reserve(_CountType size) {
        if (size < max_num) return;
        T* p = (T*)realloc(data, sizeof(T) * (size ? size : 1));
        if (!p) {
            printf("Failed when reserve myvector to %llu\n", (unsigned long long)size);
            free(data);
            exit(1);
        }
        data = p;
        max_num = size;
    }
    void fixSize(_CountType size) {
        if (size == 0) return;
        reserve(size);
        cur_num = size;
    }
    // Removes and returns the last element; an empty vector returns a
    // value-initialised T (the reference returns NULL, which only compiles
    // for pointer and arithmetic element types).
    T pop_back() {
        if (cur_num == 0) return T();
        return data[--cur_num];
    }
    inline _CountType size() const { return cur_num; }
    inline void clear() { cur_num = 0; }
};

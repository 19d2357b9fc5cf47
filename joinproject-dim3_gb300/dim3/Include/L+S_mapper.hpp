// L+S_mapper.hpp -- drop-in LS_mapper on the GPU mapper of the C ABI
// (reference Include/L+S_mapper.hpp:11-160).
//
// Same constructor and members: insert(v) returns v's id or the next dense id,
// insert(v, recorder) also records recorder[id] = v, find(v) returns the id or
// -1, size(), clear() (drops keys, keeps the counter), reset_cnt(),
// __set_cnt(v), cache_map_bucket_count().  Each single-key call is one GPU
// round trip (a launch and a synchronisation, microseconds): code that maps
// many keys should call insert_batch / find_batch, which give the same ids
// for a whole array in one call (ids in first-occurrence order, as a loop of
// insert() would).  All mappers share the process's one GPU context.  Keys
// are 32-bit; the hasher type is accepted for signature compatibility.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <functional>
#include <vector>

#include "dim3g_context.hpp"

template <typename T = int, typename H = std::hash<T>, typename _Tcounter = int>
struct LS_mapper {
    static_assert(sizeof(T) == 4, "the GPU mapper maps 32-bit keys");

   private:
    dim3g_ctx* ctx_ = nullptr;
    dim3g_mapper* m_ = nullptr;
    static void check(int rc, dim3g_ctx* c, const char* what) {
        if (rc != DIM3G_OK) {
            printf("Fail in LS_mapper::%s: %s (status %d).\n", what, c ? dim3g_last_error(c) : "", rc);
            exit(-1);
        }
    }

   public:
    LS_mapper(_Tcounter n, int /*shr_bits*/ = 0, int /*cache_n*/ = 16384) {
        ctx_ = dim3g_dropin::context();
        check(dim3g_mapper_create(ctx_, (uint64_t)(n > 0 ? n : 1), &m_), ctx_, "create");
    }
    ~LS_mapper() { dim3g_mapper_destroy(m_); }
    LS_mapper(const LS_mapper&) = delete;
    LS_mapper& operator=(const LS_mapper&) = delete;

    void clear() { check(dim3g_mapper_clear(m_), ctx_, "clear"); }
    void reset_cnt() { check(dim3g_mapper_set_cnt(m_, 0), ctx_, "reset_cnt"); }
    void __set_cnt(_Tcounter val) { check(dim3g_mapper_set_cnt(m_, (int64_t)val), ctx_, "__set_cnt"); }
    _Tcounter size() { return (_Tcounter)dim3g_mapper_size(m_); }
    int cache_map_bucket_count() { return 0; }  // no spill map on the GPU

    void insert_batch(const T* keys, size_t n, _Tcounter* ids) {
        std::vector<int32_t> tmp(n);
        check(dim3g_mapper_insert(m_, (const uint32_t*)keys, n, tmp.data()), ctx_, "insert");
        for (size_t i = 0; i < n; i++) ids[i] = (_Tcounter)tmp[i];
    }
    void find_batch(const T* keys, size_t n, _Tcounter* ids) {
        std::vector<int32_t> tmp(n);
        check(dim3g_mapper_find(m_, (const uint32_t*)keys, n, tmp.data()), ctx_, "find");
        for (size_t i = 0; i < n; i++) ids[i] = (_Tcounter)tmp[i];
    }
    _Tcounter insert(T origin_val) {
        _Tcounter id;
        insert_batch(&origin_val, 1, &id);
        return id;
    }
    _Tcounter insert(T origin_val, T* recorder) {
        _Tcounter id = insert(origin_val);
        recorder[id] = origin_val;
        return id;
    }
    _Tcounter find(T origin_val) {
        _Tcounter id;
        find_batch(&origin_val, 1, &id);
        return id;
    }
};

// dim3.hpp -- drop-in replacement for the reference's dim3.hpp entry points,
// forwarding to the GB300 C ABI (include/dim3gpu.h).
//
//   DIM3<Tx,Ty,Tz,Hx,Hy,Hz,Hxz,Tcounter>::doJoinProject(R, S, result)
//       (reference dim3.hpp:982-1055)
//   DIM3JoinAggregate<Tx,Ty,Tz,Tv,Agg,...>::doJoinAggregate(R, S, result)
//       (reference dim3.hpp:1313-1373) with Agg = AggregateFunctionCount<Tv>
//   gen_rand_data(R, S, ...)  (reference dim3.hpp:1556-1591), same tuples
//
// Keys are 32-bit (Tx, Ty, Tz of size 4).  The result's `data` is malloc'd
// (as the reference's myvector storage is) and its order is unspecified.
// Errors print a line and exit(-1), the reference's error behaviour.  Link
// with libdim3gpu.so.
#pragma once

#include <bits/stdc++.h>

#include "../../include/dim3gpu.h"
#include "Include/dim3g_context.hpp"
#include "Include/myvector.hpp"
#include "Include/structures.hpp"

using namespace std;

template <typename _Tx, typename _Ty, typename _Tv>
struct TUPLE {
    _Tx x;
    _Ty y;
    _Tv v;
    TUPLE(_Tx x_, _Ty y_, _Tv v_) : x(x_), y(y_), v(v_) {}
};

namespace dim3g_dropin {

inline void check(int rc, const char* what) {
    if (rc != DIM3G_OK) {
        printf("Fail in %s: %s (status %d).\n", what, dim3g_last_error(context()), rc);
        exit(-1);
    }
}

template <class T, class C>
inline void adopt(myvector<T, C>& result, void* data, uint64_t n) {
    if (n > (uint64_t)std::numeric_limits<C>::max()) {
        printf("Result of %llu tuples exceeds the counter type of myvector.\n", (unsigned long long)n);
        free(data);
        exit(-1);
    }
    free(result.data);
    result.data = (T*)data;
    result.cur_num = result.max_num = (C)n;
}

}  // namespace dim3g_dropin

template <typename _Tx, typename _Ty, typename _Tz, typename _Hx = hash<_Tx>, typename _Hy = hash<_Ty>,
          typename _Hz = hash<_Tz>, typename _Hxz = hash<pair<_Tx, _Tz>>, typename _Tcounter = uint32_t>
struct DIM3 {
    static_assert(sizeof(_Tx) == 4 && sizeof(_Ty) == 4 && sizeof(_Tz) == 4, "the GPU path joins 32-bit keys");
    static void doJoinProject(const myvector<pair<_Tx, _Ty>, _Tcounter> R, const myvector<pair<_Tz, _Ty>, _Tcounter> S,
                              myvector<pair<_Tx, _Tz>, _Tcounter>& result) {
        uint32_t* out = nullptr;
        uint64_t n = 0;
        dim3g_dropin::check(dim3g_join_project(dim3g_dropin::context(), (const uint32_t*)R.data, R.size(),
                                               (const uint32_t*)S.data, S.size(), &out, &n),
                            "doJoinProject");
        dim3g_dropin::adopt(result, out, n);
    }
};

// COUNT(*) aggregate plug-in with the reference's aggregate interface
// (construct with the z domain, insert / update / get, dim3.hpp:1275-1305);
// on the GPU path it selects the exact integer COUNT kernels.
template <typename _Tv>
struct AggregateFunctionCount {
    _Tv* c;
    AggregateFunctionCount(int len) { c = (_Tv*)malloc((size_t)(len > 0 ? len : 1) * sizeof(_Tv)); }
    ~AggregateFunctionCount() { free(c); }
    inline void insert(const int key, const _Tv, const _Tv) { c[key] = 1; }
    inline void update(const int key, const _Tv, const _Tv) { c[key]++; }
    inline _Tv get(const int key) const { return c[key]; }
};

// The reference's shipped AVG(R.v + S.v) plug-in (dim3.hpp:1453-1480), with
// its interface: a float sum and a count per z, get = sum / count.  The GPU
// path has no AVG kernel: DIM3JoinAggregate with this plug-in compiles (so
// join_aggregate.cpp builds unchanged) and reports DIM3G_ERR_UNSUPPORTED at
// run time, the reference's print-and-exit error behaviour.
template <typename _Tv>
struct AggregateFunctionAvg {
    std::pair<_Tv, int>* acc;
    AggregateFunctionAvg(int len) {
        acc = (std::pair<_Tv, int>*)malloc((size_t)(len > 0 ? len : 1) * sizeof(std::pair<_Tv, int>));
        if (!acc) {
            printf("Fail to malloc the AVG accumulators.\n");
            exit(-1);
        }
    }
    ~AggregateFunctionAvg() { free(acc); }
    inline void insert(const int key, const _Tv a, const _Tv b) { acc[key] = {a + b, 1}; }
    inline void update(const int key, const _Tv a, const _Tv b) {
        acc[key].first += a + b;
        acc[key].second++;
    }
    inline _Tv get(const int key) const { return acc[key].first / acc[key].second; }
};

template <class A>
struct dim3g_is_count : std::false_type {};
template <class V>
struct dim3g_is_count<AggregateFunctionCount<V>> : std::true_type {};

template <typename _Tx, typename _Ty, typename _Tz, typename _Tv, typename _Aggregate_type, typename _Hx = hash<_Tx>,
          typename _Hy = hash<_Ty>, typename _Hz = hash<_Tz>, typename _Hxz = hash<pair<_Tx, _Tz>>,
          typename _Tcounter = uint32_t>
struct DIM3JoinAggregate {
    static_assert(!dim3g_is_count<_Aggregate_type>::value || std::is_integral<_Tv>::value,
                  "COUNT needs an integer value type");
    static void doJoinAggregate(myvector<TUPLE<_Tx, _Ty, _Tv>, _Tcounter>& R, myvector<TUPLE<_Tz, _Ty, _Tv>, _Tcounter>& S,
                                myvector<TUPLE<_Tx, _Tz, _Tv>, _Tcounter>& result) {
        if (!dim3g_is_count<_Aggregate_type>::value) {
            printf("Fail in doJoinAggregate: only the COUNT aggregate runs on the GPU path (status %d).\n",
                   DIM3G_ERR_UNSUPPORTED);
            exit(-1);
        }
        std::vector<uint32_t> r(2 * (size_t)R.size()), s(2 * (size_t)S.size());
        for (size_t i = 0; i < R.size(); i++) {
            r[2 * i] = (uint32_t)R.data[i].x;
            r[2 * i + 1] = (uint32_t)R.data[i].y;
        }
        for (size_t i = 0; i < S.size(); i++) {
            s[2 * i] = (uint32_t)S.data[i].x;
            s[2 * i + 1] = (uint32_t)S.data[i].y;
        }
        uint32_t* xz = nullptr;
        uint64_t* cnt = nullptr;
        uint64_t n = 0;
        dim3g_dropin::check(dim3g_join_count(dim3g_dropin::context(), r.data(), R.size(), s.data(), S.size(), &xz, &cnt, &n),
                            "doJoinAggregate");
        typedef TUPLE<_Tx, _Tz, _Tv> T;
        T* data = (T*)malloc(sizeof(T) * (n ? n : 1));
        if (!data) {
            printf("Fail to malloc the join-aggregate result.\n");
            exit(-1);
        }
        for (uint64_t i = 0; i < n; i++) data[i] = T((_Tx)xz[2 * i], (_Tz)xz[2 * i + 1], (_Tv)(uint64_t)cnt[i]);
        free(xz);
        free(cnt);
        dim3g_dropin::adopt(result, data, n);
    }
};

// The reference's generator: default_random_engine (minstd_rand0) seeded
// with `seed`, each tuple drawn as (first % MOD, y % MODY), R before S.
inline void gen_rand_data(myvector<pair<int, int>>& R, myvector<pair<int, int>>& S, int nR = 1e7, int nS = 1e7,
                          int MODX = 1e6, int MODY = 1e6, int MODZ = 1e6, int seed = 492) {
    R.clear();
    S.clear();
    minstd_rand0 e(seed);
    for (int i = 0; i < nR; i++) {
        int x = e() % MODX;
        int y = e() % MODY;
        R.push_back({x, y});
    }
    for (int i = 0; i < nS; i++) {
        int z = e() % MODZ;
        int y = e() % MODY;
        S.push_back({z, y});
    }
}

// The reference's generator for valued tuples (dim3.hpp:1570-1591): the same
// keys as above, each tuple's value its index as a float.
inline void gen_rand_data(myvector<TUPLE<int, int, float>>& R, myvector<TUPLE<int, int, float>>& S, int nR = 1e7,
                          int nS = 1e7, int MODX = 1e6, int MODY = 1e6, int MODZ = 1e6, int seed = 492) {
    R.clear();
    S.clear();
    minstd_rand0 e(seed);
    for (int i = 0; i < nR; i++) {
        int x = e() % MODX;
        int y = e() % MODY;
        R.push_back(TUPLE<int, int, float>(x, y, (float)i));
    }
    for (int i = 0; i < nS; i++) {
        int z = e() % MODZ;
        int y = e() % MODY;
        S.push_back(TUPLE<int, int, float>(z, y, (float)i));
    }
}

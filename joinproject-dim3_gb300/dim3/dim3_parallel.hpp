// dim3_parallel.hpp -- drop-in replacement for the reference's
// dim3_parallel.hpp: DIM3_parallel<...>::doJoinProject_parallel
// (reference dim3_parallel.hpp:137-210) runs the same GPU path as DIM3.
// THREAD_NUM is kept for code that reads it; the GPU path ignores it.
#pragma once

#ifndef THREAD_NUM
#define THREAD_NUM 8
#endif

#include "dim3.hpp"

template <typename _Tx, typename _Ty, typename _Tz, typename _Hx = hash<_Tx>, typename _Hy = hash<_Ty>,
          typename _Hz = hash<_Tz>, typename _Hxz = hash<pair<_Tx, _Tz>>, typename _Tcounter = uint32_t>
struct DIM3_parallel : public DIM3<_Tx, _Ty, _Tz, _Hx, _Hy, _Hz, _Hxz, _Tcounter> {
    static void doJoinProject_parallel(const myvector<pair<_Tx, _Ty>, _Tcounter> R,
                                       const myvector<pair<_Tz, _Ty>, _Tcounter> S,
                                       myvector<pair<_Tx, _Tz>, _Tcounter>& result) {
        DIM3<_Tx, _Ty, _Tz, _Hx, _Hy, _Hz, _Hxz, _Tcounter>::doJoinProject(R, S, result);
    }
};

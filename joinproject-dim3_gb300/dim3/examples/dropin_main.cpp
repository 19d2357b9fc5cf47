// dropin_main.cpp -- the reference's drivers (main.cpp, main_parallel.cpp,
// join_aggregate.cpp) written against the drop-in headers: generate the
// reference's default relations, run the join, print |Result| and an
// order-independent hash of the result.
//
//   dropin_main project|parallel|count|mapper [nR nS MODX MODY MODZ]
#include <cstring>

#include "../Include/L+S_mapper.hpp"
#include "../dim3_parallel.hpp"

static uint64_t mix64(uint64_t v) {
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31);
}

int main(int argc, char* argv[]) {
    const char* mode = argc > 1 ? argv[1] : "project";
    int nR = argc > 2 ? atoi(argv[2]) : (int)1e7, nS = argc > 3 ? atoi(argv[3]) : (int)1e7;
    int mx = argc > 4 ? atoi(argv[4]) : (int)1e6, my = argc > 5 ? atoi(argv[5]) : (int)1e6;
    int mz = argc > 6 ? atoi(argv[6]) : (int)1e6;
    myvector<pair<int, int>> R, S, result;
    gen_rand_data(R, S, nR, nS, mx, my, mz);
    auto t0 = chrono::high_resolution_clock::now();
    uint64_t h = 0, n = 0;
    if (!strcmp(mode, "project") || !strcmp(mode, "parallel")) {
        if (!strcmp(mode, "project"))
            DIM3<int, int, int, myHasher, myHasher, myHasher, myHasher, uint32_t>::doJoinProject(R, S, result);
        else
            DIM3_parallel<int, int, int, myHasher, myHasher, myHasher, myHasher, uint32_t>::doJoinProject_parallel(R, S, result);
        n = result.size();
        for (uint32_t i = 0; i < result.size(); i++)
            h += mix64(((uint64_t)(uint32_t)result.data[i].first << 32) | (uint32_t)result.data[i].second);
    } else if (!strcmp(mode, "count")) {
        myvector<TUPLE<int, int, long long>> r, s, out;
        for (uint32_t i = 0; i < R.size(); i++) r.push_back(TUPLE<int, int, long long>(R.data[i].first, R.data[i].second, 0));
        for (uint32_t i = 0; i < S.size(); i++) s.push_back(TUPLE<int, int, long long>(S.data[i].first, S.data[i].second, 0));
        DIM3JoinAggregate<int, int, int, long long, AggregateFunctionCount<long long>, myHasher, myHasher, myHasher,
                          myHasher, uint32_t>::doJoinAggregate(r, s, out);
        n = out.size();
        for (uint32_t i = 0; i < out.size(); i++)
            h += mix64(mix64(((uint64_t)(uint32_t)out.data[i].x << 32) | (uint32_t)out.data[i].y) + (uint64_t)out.data[i].v);
    } else if (!strcmp(mode, "mapper")) {
        LS_mapper<int, myHasher> m(R.size());
        std::vector<int> ids(R.size());
        std::vector<int> ys(R.size());
        for (uint32_t i = 0; i < R.size(); i++) ys[i] = R.data[i].second;
        m.insert_batch(ys.data(), ys.size(), ids.data());
        n = (uint64_t)m.size();
        for (size_t i = 0; i < ids.size(); i++) h += mix64(((uint64_t)(uint32_t)ys[i] << 32) | (uint32_t)ids[i]);
    } else {
        printf("unknown mode %s\n", mode);
        return 2;
    }
    auto t1 = chrono::high_resolution_clock::now();
    printf("It takes %f seconds.\n", chrono::duration<double>(t1 - t0).count());
    printf("|Result|=%llu\n", (unsigned long long)n);
    printf("hash=%llu\n", (unsigned long long)h);
    return 0;
}

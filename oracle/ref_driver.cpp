// ref_driver.cpp -- C entry points around the UNMODIFIED reference headers
// (schencoding/JoinProject-DIM3: dim3.hpp, dim3_parallel.hpp), compiled from
// the reference's own sources by oracle/Makefile.ref into oracle/_ref/.
// TEST INFRASTRUCTURE ONLY: used to pin the C oracle and to produce golden
// fixtures in tests/golden/.  Nothing in the product links it.
#include "dim3_parallel.hpp"

static myvector<pair<int, int>> wrap(const int* p, unsigned n) {
    myvector<pair<int, int>> v;
    free(v.data);
    v.data = (pair<int, int>*)p;
    v.cur_num = v.max_num = n;
    return v;
}

// COUNT(*) plug-in written against the reference's aggregate interface
// (dim3.hpp:1275 construct, :1295 insert, :1299 update, :1305 get).
template <typename Tv>
struct RefAggregateCount {
    Tv* c;
    RefAggregateCount(int len) { c = (Tv*)malloc((size_t)len * sizeof(Tv)); }
    ~RefAggregateCount() { free(c); }
    void insert(const int key, const Tv, const Tv) { c[key] = 1; }
    void update(const int key, const Tv, const Tv) { c[key]++; }
    Tv get(const int key) const { return c[key]; }
};


extern "C" {

// Reference's gen_rand_data (dim3.hpp:1556-1568) into caller buffers of
// interleaved (x, y) pairs.
void ref_gen_rand_data(int nR, int nS, int MODX, int MODY, int MODZ, int seed, int* R, int* S) {
    myvector<pair<int, int>> r, s;
    gen_rand_data(r, s, nR, nS, MODX, MODY, MODZ, seed);
    memcpy(R, r.data, (size_t)nR * 8);
    memcpy(S, s.data, (size_t)nS * 8);
    free(r.data);
    free(s.data);
}

// DIM3::doJoinProject (dim3.hpp:987) / DIM3_parallel::doJoinProject_parallel
// (dim3_parallel.hpp:142).  *out is the reference's own malloc'd result.
unsigned ref_join_project(const int* R, unsigned nR, const int* S, unsigned nS, int parallel, int** out) {
    myvector<pair<int, int>> r = wrap(R, nR), s = wrap(S, nS), result;
    if (parallel)
        DIM3_parallel<int, int, int, myHasher, myHasher, myHasher, myHasher, uint32_t>::doJoinProject_parallel(r, s, result);
    else
        DIM3<int, int, int, myHasher, myHasher, myHasher, myHasher, uint32_t>::doJoinProject(r, s, result);
    *out = (int*)result.data;
    return result.size();
}

// Classical radix hash join + projection (dim3.hpp:273-391), driven the way
// baseline_Classical.cpp:19-21 drives it.
unsigned ref_classical(const int* R, unsigned nR, const int* S, unsigned nS, int** out) {
    myvector<pair<int, int>> r = wrap(R, nR), s = wrap(S, nS), result;
    result.clear();
    LL est = EstimateJoinCardinality<int, int, int, myHasher>::estimate(r, s);
    Radix_hash_join_and_project<int, int, int, myHasher, myHasher> cj;
    cj.dojoinproject(r, s, est, result);
    *out = (int*)result.data;
    return result.size();
}

long long ref_estimate(const int* R, unsigned nR, const int* S, unsigned nS) {
    myvector<pair<int, int>> r = wrap(R, nR), s = wrap(S, nS);
    return EstimateJoinCardinality<int, int, int, myHasher>::estimate(r, s);
}

// DIM3JoinAggregate::doJoinAggregate (dim3.hpp:1318) with COUNT.
// Output: xz pairs and int64 counts, both malloc'd here.
unsigned ref_join_count(const int* R, unsigned nR, const int* S, unsigned nS, int** out_xz, long long** out_cnt) {
    typedef TUPLE<int, int, long long> T;
    myvector<T> r(nR ? nR : 1), s(nS ? nS : 1), result;
    for (unsigned i = 0; i < nR; i++) r.push_back(T(R[2 * i], R[2 * i + 1], 0));
    for (unsigned i = 0; i < nS; i++) s.push_back(T(S[2 * i], S[2 * i + 1], 0));
    DIM3JoinAggregate<int, int, int, long long, RefAggregateCount<long long>,
                      myHasher, myHasher, myHasher, myHasher, uint32_t>::doJoinAggregate(r, s, result);
    unsigned n = result.size();
    int* xz = (int*)malloc((size_t)(n ? n : 1) * 8);
    long long* cnt = (long long*)malloc((size_t)(n ? n : 1) * 8);
    for (unsigned i = 0; i < n; i++) {
        xz[2 * i] = result.data[i].x;
        xz[2 * i + 1] = result.data[i].y;
        cnt[i] = result.data[i].v;
    }
    free(r.data);
    free(s.data);
    free(result.data);
    *out_xz = xz;
    *out_cnt = cnt;
    return n;
}

// DIM3JoinAggregate with the shipped AVG(R.v+S.v) float aggregate
// (dim3.hpp:1453-1480), as join_aggregate.cpp:20-22 calls it.
unsigned ref_join_avg(const int* R, const float* Rv, unsigned nR, const int* S, const float* Sv, unsigned nS,
                      int** out_xz, float** out_avg) {
    typedef TUPLE<int, int, float> T;
    myvector<T> r(nR ? nR : 1), s(nS ? nS : 1), result;
    for (unsigned i = 0; i < nR; i++) r.push_back(T(R[2 * i], R[2 * i + 1], Rv[i]));
    for (unsigned i = 0; i < nS; i++) s.push_back(T(S[2 * i], S[2 * i + 1], Sv[i]));
    DIM3JoinAggregate<int, int, int, float, AggregateFunctionAvg<float>,
                      myHasher, myHasher, myHasher, myHasher, uint32_t>::doJoinAggregate(r, s, result);
    unsigned n = result.size();
    int* xz = (int*)malloc((size_t)(n ? n : 1) * 8);
    float* avg = (float*)malloc((size_t)(n ? n : 1) * 4);
    for (unsigned i = 0; i < n; i++) {
        xz[2 * i] = result.data[i].x;
        xz[2 * i + 1] = result.data[i].y;
        avg[i] = result.data[i].v;
    }
    free(r.data);
    free(s.data);
    free(result.data);
    *out_xz = xz;
    *out_avg = avg;
    return n;
}

void ref_free(void* p) { free(p); }
}

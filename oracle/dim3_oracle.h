/*
 * dim3_oracle.h -- CPU oracle for the DIM3 join-project / join-aggregate path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (schencoding/JoinProject-DIM3: dim3.hpp, dim3_parallel.hpp,
 * Include/L+S_mapper.hpp) used as the checker for the GPU path and as the
 * timed CPU baseline.  Only tests, the smoke check and the CPU-baseline leg
 * of the benchmark may load it.  The product path never calls it.
 *
 * Parity pin: the restatement is checked against the reference itself
 * (compiled from its own sources by oracle/Makefile.ref into oracle/_ref/)
 * and against the reference's known answer on its default generator
 * (|Result| = 98,931,829), through fixtures under tests/golden/.
 *
 * Relations are arrays of interleaved uint32 pairs: R = (x, y), S = (z, y),
 * exactly the memory layout of myvector<pair<int,int>> in the reference.
 */
#ifndef DIM3_ORACLE_H
#define DIM3_ORACLE_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Per-call statistics (phase sizes the tests look at). */
typedef struct {
    int32_t used_classical; /* 1 if f1 chose the radix hash join (dim3.hpp:1000) */
    int32_t swapped;        /* 1 if |R| < |S| so the roles were swapped (dim3.hpp:993) */
    int32_t nx, ny, nz;     /* dense id domain sizes after mapping */
    int32_t n_dense_z;      /* z columns chosen as dense by f2 (dim3.hpp:1120) */
    int64_t out_j_hat;      /* sampled join-size estimate (dim3.hpp:193) */
    uint64_t out_j;         /* exact join size sum_b degR(b)*degS(b) after the semi-join */
    double t_estimate, t_mapping, t_divide, t_expand; /* seconds */
} dim3o_stats;

/* Order-independent hash of a set of (x, z) pairs: sum of mix64(x<<32|z). */
uint64_t dim3o_pair_hash(uint32_t x, uint32_t z);
/* Hash of one (x, z, count) group: mix64(mix64(x<<32|z) + count). */
uint64_t dim3o_group_hash(uint32_t x, uint32_t z, uint64_t count);

/*
 * Join-project: the distinct set {(P.x, Q.x) | P.y == Q.y} where P is the
 * larger input (R when |R| >= |S|, else S -- the reference's swap).
 *   threads <= 1 : DIM3::doJoinProject (dim3.hpp:987-1055), serial.
 *   threads  > 1 : DIM3_parallel::doJoinProject_parallel (dim3_parallel.hpp:142),
 *                  OpenMP over x with `threads` threads.  Where the reference's
 *                  parallel entry asserts on the classical branch
 *                  (dim3_parallel.hpp:155-161) the oracle runs the hybrid path.
 *   hash_only    : do not store pairs; return count and set hash only.
 * *out (malloc'd, interleaved pairs) is owned by the caller; free with dim3o_free.
 * Returns 0 on success, -1 on allocation failure.
 */
int dim3o_join_project(const uint32_t* R, uint64_t nR, const uint32_t* S, uint64_t nS,
                       int threads, int hash_only,
                       uint32_t** out, uint64_t* n_out, uint64_t* set_hash,
                       dim3o_stats* stats);

/*
 * Join-aggregate COUNT(*) GROUP BY (P.x, Q.x): DIM3JoinAggregate::doJoinAggregate
 * (dim3.hpp:1318-1373) with a COUNT plug-in written against the reference's
 * aggregate interface (insert / update / get, dim3.hpp:1295-1305).
 * Emits (x, z) pairs into *out_xz and int64 counts into *out_cnt.
 */
int dim3o_join_count(const uint32_t* R, uint64_t nR, const uint32_t* S, uint64_t nS,
                     int threads, int hash_only,
                     uint32_t** out_xz, uint64_t** out_cnt, uint64_t* n_out,
                     uint64_t* set_hash, dim3o_stats* stats);

/*
 * Join-aggregate AVG(R.v + S.v) in float, exactly the reference's shipped
 * aggregate (AggregateFunctionAvg, dim3.hpp:1453-1480) and summation order.
 * Rv / Sv hold one float per tuple.
 */
int dim3o_join_avg(const uint32_t* R, const float* Rv, uint64_t nR,
                   const uint32_t* S, const float* Sv, uint64_t nS,
                   uint32_t** out_xz, float** out_avg, uint64_t* n_out,
                   dim3o_stats* stats);

/* Classical radix hash join + hash-set projection (dim3.hpp:273-391). */
int dim3o_classical(const uint32_t* R, uint64_t nR, const uint32_t* S, uint64_t nS,
                    uint32_t** out, uint64_t* n_out, uint64_t* set_hash);

/* Sampled join-size estimate (dim3.hpp:193-224); R must be the larger input. */
int64_t dim3o_estimate(const uint32_t* R, uint64_t nR, const uint32_t* S, uint64_t nS);

void dim3o_free(void* p);

#ifdef __cplusplus
}
#endif
#endif

/* dim3gen.h -- seeded synthetic relations (deterministic on x86-64 and
 * aarch64) for the join-project workloads.  Pairs are interleaved uint32. */
#ifndef DIM3GEN_H
#define DIM3GEN_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
/* The reference's gen_rand_data (minstd_rand0, `% MOD`), R then S. */
void dim3gen_minstd(uint32_t nR, uint32_t nS, uint32_t modx, uint32_t mody, uint32_t modz, uint32_t seed,
                    uint32_t* R, uint32_t* S);
/* n pairs: first column uniform in [0, dom_a), y Zipf(s) over dom_b ranks. */
int dim3gen_zipf_side(uint64_t n, uint32_t dom_a, uint32_t dom_b, double s, uint64_t seed, uint32_t* out);
/* Chung-Lu graph, both edge directions; out must hold 4*M uint32. */
uint64_t dim3gen_chung_lu(uint32_t n, double beta, uint64_t M, uint64_t seed, uint32_t* out,
                          uint32_t* max_weight_out);
/* Parameters of query q of the mixed batch. */
void dim3gen_batch_params(uint64_t seed, uint32_t q, double n_lo, double n_hi, double s_lo, double s_hi,
                          double d_lo, double d_hi, uint64_t* n_out, double* s_out, uint32_t* dom_out);
uint32_t dim3gen_rank_value(uint32_t rank);
/* One relation of a served set (see dim3gen.c). */
int dim3gen_serve_relation(uint64_t n, uint32_t dom_a, uint32_t dom_b_log2, double s, uint32_t mul, uint32_t add,
                           uint64_t seed, uint32_t* out);
double dim3gen_det_pow(double b, double e);
#ifdef __cplusplus
}
#endif
#endif

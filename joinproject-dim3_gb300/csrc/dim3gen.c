/*
 * dim3gen.c -- seeded synthetic relations for the join-project workloads.
 *
 * Every generator is deterministic across x86-64 and aarch64: it uses only
 * integer arithmetic and IEEE +,-,*,/ (compiled with -ffp-contract=off), its
 * own logarithm and exponential, and per-chunk PRNG streams, so the output is
 * identical for any thread count and on both machines.
 *
 * Relations are arrays of interleaved uint32 pairs (first, y): R = (a, b),
 * S = (c, b), the layout of myvector<pair<int,int>> in the reference.
 */
#include "dim3gen.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---------------------------------------------------------------- PRNG */
/* SplitMix64 (Steele, Lea, Flood 2014). */
static inline uint64_t sm64(uint64_t* s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static inline uint64_t stream_seed(uint64_t seed, uint64_t stream) {
    uint64_t s = seed ^ (stream * 0xD1B54A32D192ED03ULL);
    return sm64(&s);
}
/* Uniform double in [0, 1) with 53 random bits. */
static inline double u01(uint64_t* s) { return (double)(sm64(s) >> 11) * (1.0 / 9007199254740992.0); }
/* Uniform integer in [0, n), n < 2^32 (multiply-shift). */
static inline uint32_t below(uint64_t* s, uint32_t n) {
    return (uint32_t)(((sm64(s) >> 32) * (uint64_t)n) >> 32);
}

/* ------------------------------------------- deterministic log / exp */
static const double LN2 = 0.69314718055994530942;

static double det_log(double x) { /* x > 0 */
    int e = 0;
    while (x >= 2.0) { x *= 0.5; e++; }
    while (x < 1.0) { x *= 2.0; e--; }
    if (x > 1.41421356237309504880) { x *= 0.5; e++; }
    double t = (x - 1.0) / (x + 1.0), t2 = t * t, term = t, sum = 0.0;
    for (int k = 1; k < 60; k += 2) {
        sum += term / k;
        term *= t2;
    }
    return 2.0 * sum + e * LN2;
}

static double det_exp(double x) {
    double kd = x / LN2;
    long k = (long)(kd < 0 ? kd - 0.5 : kd + 0.5);
    double r = x - (double)k * LN2, term = 1.0, sum = 1.0;
    for (int i = 1; i < 30; i++) {
        term *= r / i;
        sum += term;
    }
    while (k > 0) { sum *= 2.0; k--; }
    while (k < 0) { sum *= 0.5; k++; }
    return sum;
}

static double det_pow(double b, double e) { return det_exp(e * det_log(b)); }

/* ------------------------------------------------ value permutations */
/* Odd-multiplier bijection of uint32: scatters ranks over the key space. */
uint32_t dim3gen_rank_value(uint32_t rank) { return rank * 2654435761u + 0x3C6EF372u; }

/* ----------------------------------------------------------- Zipf CDF */
/* Inverse-CDF sampler over ranks 0..n-1 with P(r) ~ (r+1)^-s. */
typedef struct {
    double* cdf;
    uint32_t n;
} zipf_t;

static int zipf_init(zipf_t* z, uint32_t n, double s) {
    z->n = n;
    z->cdf = (double*)malloc((size_t)n * sizeof(double));
    if (!z->cdf) return -1;
    double acc = 0.0;
    for (uint32_t r = 0; r < n; r++) {
        double w = (s == 1.0) ? 1.0 / (double)(r + 1) : det_exp(-s * det_log((double)(r + 1)));
        acc += w;
        z->cdf[r] = acc;
    }
    for (uint32_t r = 0; r < n; r++) z->cdf[r] /= acc;
    z->cdf[n - 1] = 1.0;
    return 0;
}

static inline uint32_t zipf_draw(const zipf_t* z, uint64_t* s) {
    double u = u01(s);
    uint32_t lo = 0, hi = z->n - 1;
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (z->cdf[mid] > u) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

#define CHUNK 65536u

/* ------------------------------------------------- reference generator */
/* gen_rand_data (dim3.hpp:1556-1568): the C++ default_random_engine of
 * libstdc++ is minstd_rand0 (x <- 16807 x mod 2^31-1); per tuple the first
 * draw gives the first column and the second draw y, R before S. */
void dim3gen_minstd(uint32_t nR, uint32_t nS, uint32_t modx, uint32_t mody, uint32_t modz, uint32_t seed,
                    uint32_t* R, uint32_t* S) {
    uint64_t x = seed % 2147483647u;
    if (x == 0) x = 1;
#define NEXT() (x = (x * 16807u) % 2147483647u, (uint32_t)x)
    for (uint32_t i = 0; i < nR; i++) {
        R[2 * i] = NEXT() % modx;
        R[2 * i + 1] = NEXT() % mody;
    }
    for (uint32_t i = 0; i < nS; i++) {
        S[2 * i] = NEXT() % modz;
        S[2 * i + 1] = NEXT() % mody;
    }
#undef NEXT
}

/* ------------------------------------------------ Zipf-B join relation */
/* One side: first column uniform in [0, dom_a), y = rank_value(Zipf(s) over
 * dom_b ranks).  Duplicates are kept. */
int dim3gen_zipf_side(uint64_t n, uint32_t dom_a, uint32_t dom_b, double s, uint64_t seed, uint32_t* out) {
    zipf_t z;
    if (zipf_init(&z, dom_b, s)) return -1;
    uint64_t nchunks = (n + CHUNK - 1) / CHUNK;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < (int64_t)nchunks; c++) {
        uint64_t st = stream_seed(seed, (uint64_t)c);
        uint64_t i0 = (uint64_t)c * CHUNK, i1 = i0 + CHUNK < n ? i0 + CHUNK : n;
        for (uint64_t i = i0; i < i1; i++) {
            out[2 * i] = below(&st, dom_a);
            out[2 * i + 1] = dim3gen_rank_value(zipf_draw(&z, &st));
        }
    }
    free(z.cdf);
    return 0;
}

/* One relation of a served set: first column uniform in [0, dom_a); y rank
 * Zipf(s) over 2^dom_b_log2 ranks, mapped to a B value through this
 * relation's own bijection rank -> (mul * rank + add) mod 2^dom_b_log2 (mul
 * odd) and rank_value, so relations share the B domain but not the order of
 * their heavy values.  Duplicates are kept. */
int dim3gen_serve_relation(uint64_t n, uint32_t dom_a, uint32_t dom_b_log2, double s, uint32_t mul, uint32_t add,
                           uint64_t seed, uint32_t* out) {
    zipf_t z;
    const uint32_t dom_b = 1u << dom_b_log2, mask = dom_b - 1;
    if (zipf_init(&z, dom_b, s)) return -1;
    mul |= 1u;
    uint64_t nchunks = (n + CHUNK - 1) / CHUNK;
#pragma omp parallel for schedule(static)
    for (int64_t c = 0; c < (int64_t)nchunks; c++) {
        uint64_t st = stream_seed(seed, (uint64_t)c);
        uint64_t i0 = (uint64_t)c * CHUNK, i1 = i0 + CHUNK < n ? i0 + CHUNK : n;
        for (uint64_t i = i0; i < i1; i++) {
            out[2 * i] = below(&st, dom_a);
            out[2 * i + 1] = dim3gen_rank_value((mul * zipf_draw(&z, &st) + add) & mask);
        }
    }
    free(z.cdf);
    return 0;
}

/* ---------------------------------------------------- Chung-Lu graph */
/* Undirected Chung-Lu power-law graph: vertex i has weight
 * (i+1)^(-1/(beta-1)) scaled to mean degree 2M/n and capped at sqrt(sum w);
 * M edge samples pick both endpoints proportionally to weight (Vose alias
 * tables), self-loops are dropped, each kept edge is emitted in both
 * directions (u,v),(v,u).  Multi-edges are kept.  Vertex i is named
 * rank_value(i).  Returns the number of directed edges written (<= 2M). */
uint64_t dim3gen_chung_lu(uint32_t n, double beta, uint64_t M, uint64_t seed, uint32_t* out,
                          uint32_t* max_weight_out) {
    double* w = (double*)malloc((size_t)n * sizeof(double));
    double* prob = (double*)malloc((size_t)n * sizeof(double));
    uint32_t* alias = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
    uint32_t* small = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
    uint32_t* large = (uint32_t*)malloc((size_t)n * sizeof(uint32_t));
    uint8_t* keep = NULL;
    uint64_t total = 0;
    if (!w || !prob || !alias || !small || !large) goto done;
    {
        double ex = -1.0 / (beta - 1.0), sum = 0.0;
        for (uint32_t i = 0; i < n; i++) {
            w[i] = det_exp(ex * det_log((double)(i + 1)));
            sum += w[i];
        }
        double scale = (2.0 * (double)M / (double)n) / (sum / (double)n);
        sum = 0.0;
        for (uint32_t i = 0; i < n; i++) {
            w[i] *= scale;
            sum += w[i];
        }
        /* cap at sqrt(sum w): Newton iterations on y*y = sum */
        double cap = sum > 1 ? sum / 2 : 1;
        for (int it = 0; it < 200; it++) cap = 0.5 * (cap + sum / cap);
        double wsum = 0.0;
        for (uint32_t i = 0; i < n; i++) {
            if (w[i] > cap) w[i] = cap;
            wsum += w[i];
        }
        if (max_weight_out) *max_weight_out = (uint32_t)w[0];
        /* Vose alias construction (deterministic order) */
        uint32_t ns = 0, nl = 0;
        for (uint32_t i = 0; i < n; i++) {
            prob[i] = w[i] * (double)n / wsum;
            if (prob[i] < 1.0) small[ns++] = i;
            else large[nl++] = i;
        }
        while (ns && nl) {
            uint32_t l = small[--ns], g = large[--nl];
            alias[l] = g;
            prob[g] = (prob[g] + prob[l]) - 1.0;
            if (prob[g] < 1.0) small[ns++] = g;
            else large[nl++] = g;
        }
        while (nl) { uint32_t g = large[--nl]; prob[g] = 1.0; alias[g] = g; }
        while (ns) { uint32_t l = small[--ns]; prob[l] = 1.0; alias[l] = l; }
    }
    keep = (uint8_t*)malloc((size_t)M);
    if (!keep) goto done;
    {
        uint64_t nchunks = (M + CHUNK - 1) / CHUNK;
#pragma omp parallel for schedule(static)
        for (int64_t c = 0; c < (int64_t)nchunks; c++) {
            uint64_t st = stream_seed(seed, (uint64_t)c);
            uint64_t i0 = (uint64_t)c * CHUNK, i1 = i0 + CHUNK < M ? i0 + CHUNK : M;
            for (uint64_t i = i0; i < i1; i++) {
                uint32_t k1 = below(&st, n);
                uint32_t u = u01(&st) < prob[k1] ? k1 : alias[k1];
                uint32_t k2 = below(&st, n);
                uint32_t v = u01(&st) < prob[k2] ? k2 : alias[k2];
                keep[i] = (u != v);
                out[4 * i] = dim3gen_rank_value(u);
                out[4 * i + 1] = dim3gen_rank_value(v);
                out[4 * i + 2] = dim3gen_rank_value(v);
                out[4 * i + 3] = dim3gen_rank_value(u);
            }
        }
        /* compact away self-loops, preserving order */
        for (uint64_t i = 0; i < M; i++) {
            if (!keep[i]) continue;
            if (2 * i != total) memmove(out + 2 * total, out + 4 * i, 16);
            total += 2;
        }
    }
done:
    free(w);
    free(prob);
    free(alias);
    free(small);
    free(large);
    free(keep);
    return total;
}

/* --------------------------------------------------- batched workload */
/* Parameters of query q of a seeded mixed batch: per-side tuple count
 * log-uniform in [n_lo, n_hi], Zipf exponent uniform in [s_lo, s_hi],
 * dom(A)=dom(C) log-uniform in [d_lo, d_hi], dom(B)=dom(A). */
void dim3gen_batch_params(uint64_t seed, uint32_t q, double n_lo, double n_hi, double s_lo, double s_hi,
                          double d_lo, double d_hi, uint64_t* n_out, double* s_out, uint32_t* dom_out) {
    uint64_t st = stream_seed(seed ^ 0xB47C4ULL, q);
    double ln_lo = det_log(n_lo), ln_hi = det_log(n_hi);
    *n_out = (uint64_t)det_exp(ln_lo + u01(&st) * (ln_hi - ln_lo));
    *s_out = s_lo + u01(&st) * (s_hi - s_lo);
    double d0 = det_log(d_lo), d1 = det_log(d_hi);
    *dom_out = (uint32_t)det_exp(d0 + u01(&st) * (d1 - d0));
}

double dim3gen_det_pow(double b, double e) { return det_pow(b, e); }

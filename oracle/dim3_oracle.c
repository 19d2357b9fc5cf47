/*
 * dim3_oracle.c -- CPU oracle (test infrastructure only) for the DIM3
 * join-project and join-aggregate path.
 *
 * A plain-C restatement of the reference algorithm, step by step, so that
 * (1) its output sets can be compared bit-exactly with the GPU path and
 * (2) its run time stands in for the reference's own CPU implementation on
 * machines where the reference sources are not present.  Every function
 * names the reference file:line it follows.  Layout choices (struct-of-arrays
 * columns instead of arrays of pairs, an own spill table instead of the
 * vendored ska::flat_hash_map) do not change any id assignment or output.
 *
 * Deliberate deviations from the reference, all of which only avoid
 * undefined behaviour and none of which changes an output set:
 *   - the estimator's fallback reads min(1000, n) tuples, not always 1000
 *     (dim3.hpp:215-221 reads past short inputs);
 *   - the f3 threshold cache is sized max(ny, longest x row + 1)
 *     (dim3.hpp:899 sizes it ny and indexes it by row length);
 *   - f2's interval cache is bypassed when Sm_cnt/interval >= 105
 *     (dim3.hpp:98-101 indexes a 105-entry array);
 *   - counters are 64-bit, so outputs past 2^31 pairs do not wrap
 *     (Include/myvector.hpp:35, dim3.hpp:892);
 *   - an empty semi-join result returns an empty answer in join-aggregate
 *     too (dim3.hpp:1342-1350 has no such check).
 */
#define _POSIX_C_SOURCE 199309L
#include "dim3_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------ */
/* Machine model constants of the reference (server_parameters.hpp:9-39). */
#define L2_BYTES 262144u
#define L3_BYTES 12582912u
#define L2_INTS (L2_BYTES / 4u)
#define L3_INTS (L3_BYTES / 4u)
#define LINE_BYTES 64u
#define PARTITION_PARA 10000u

static const double C_FLAT_HASH = 38.006142;
static const double C_LS_BUILD = 21.381317;
static const double C_LS_PROBE = 17.218456;
static const double C_RX_DENSE = 1.956135;
static const double C_RX_SPARSE = 4.879672;
static const double C_SZ_BITMAP = 3.484022;
static const double C_SEQ_READ = 0.121759;
/* random read / read-write cost at 1k, 2xL2, 0.5xL3, 1.5xL3, 3xL3, 10xL3 */
static const double C_RR[6] = {0.499693, 1.005135, 1.552501, 3.750952, 5.417254, 7.198486};
static const double C_RW[6] = {0.443129, 1.324415, 1.914639, 5.359059, 7.911922, 11.245022};

static double now_s(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* Piecewise-linear miss-cost curve (server_parameters.hpp:42-95). */
static double mem_cost(int array_size, const double* c) {
    unsigned int n = (unsigned int)array_size;
    unsigned int xs[6];
    xs[0] = 1000u;
    xs[1] = 2u * L2_INTS;
    xs[2] = (unsigned int)(0.5 * L3_INTS);
    xs[3] = (unsigned int)(1.5 * L3_INTS);
    xs[4] = (unsigned int)(3 * L3_INTS);
    xs[5] = (unsigned int)(10 * L3_INTS);
    if (n <= xs[0]) return c[0];
    for (int i = 1; i < 6; i++) {
        if (n <= xs[i])
            return (double)(n - xs[i - 1]) / (double)(xs[i] - xs[i - 1]) * (c[i] - c[i - 1]) + c[i - 1];
    }
    return c[5];
}
static double rand_read_cost(int n) { return mem_cost(n, C_RR); }
static double rand_rw_cost(int n) { return mem_cost(n, C_RW); }

/* std::min semantics: (b < a) ? b : a -- NaN handling matters in f2. */
static double stdmin(double a, double b) { return (b < a) ? b : a; }

/* ------------------------------------------------------------------ */
/* Output sinks. */
uint64_t dim3o_pair_hash(uint32_t x, uint32_t z) {
    uint64_t v = ((uint64_t)x << 32) | (uint64_t)z;
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31);
}
static uint64_t mix64(uint64_t v) {
    v = (v ^ (v >> 30)) * 0xbf58476d1ce4e5b9ULL;
    v = (v ^ (v >> 27)) * 0x94d049bb133111ebULL;
    return v ^ (v >> 31);
}
uint64_t dim3o_group_hash(uint32_t x, uint32_t z, uint64_t count) {
    return mix64(dim3o_pair_hash(x, z) + count);
}

typedef struct {
    uint32_t* xz;
    uint64_t* cnt; /* join-aggregate only */
    float* avg;    /* AVG aggregate only */
    uint64_t n, cap;
    int hash_only;
    uint64_t hash;
    int oom;
} sink_t;

static int sink_grow(sink_t* s) {
    uint64_t nc = s->cap ? s->cap * 2 : 1024;
    uint32_t* p = (uint32_t*)realloc(s->xz, nc * 2 * sizeof(uint32_t));
    if (!p) { s->oom = 1; return -1; }
    s->xz = p;
    if (s->cnt) {
        uint64_t* q = (uint64_t*)realloc(s->cnt, nc * sizeof(uint64_t));
        if (!q) { s->oom = 1; return -1; }
        s->cnt = q;
    }
    if (s->avg) {
        float* q = (float*)realloc(s->avg, nc * sizeof(float));
        if (!q) { s->oom = 1; return -1; }
        s->avg = q;
    }
    s->cap = nc;
    return 0;
}

static inline void emit_pair(sink_t* s, uint32_t x, uint32_t z) {
    if (s->hash_only) {
        s->hash += dim3o_pair_hash(x, z);
        s->n++;
        return;
    }
    if (s->n == s->cap && sink_grow(s)) return;
    s->xz[2 * s->n] = x;
    s->xz[2 * s->n + 1] = z;
    s->n++;
}

static inline void emit_group(sink_t* s, uint32_t x, uint32_t z, uint64_t c) {
    if (s->hash_only) {
        s->hash += dim3o_group_hash(x, z, c);
        s->n++;
        return;
    }
    if (s->n == s->cap && sink_grow(s)) return;
    s->xz[2 * s->n] = x;
    s->xz[2 * s->n + 1] = z;
    s->cnt[s->n] = c;
    s->n++;
}

/* ------------------------------------------------------------------ */
/* uint32 -> int32 map used for the L+S mapper's small spill map and the
 * estimator's sample map (the reference uses the vendored
 * ska::flat_hash_map for both; only lookups, never ordering, matter). */
typedef struct {
    uint32_t* keys;
    int64_t* vals;
    uint8_t* used;
    uint64_t cap, n;
} u32map;

static uint64_t hmix32(uint32_t k) {
    uint64_t v = k * 0x9E3779B97F4A7C15ULL;
    return v ^ (v >> 29);
}

static int u32map_init(u32map* m, uint64_t want) {
    uint64_t cap = 16;
    while (cap < 2 * want) cap <<= 1;
    m->keys = (uint32_t*)malloc(cap * sizeof(uint32_t));
    m->vals = (int64_t*)malloc(cap * sizeof(int64_t));
    m->used = (uint8_t*)calloc(cap, 1);
    m->cap = cap;
    m->n = 0;
    return (m->keys && m->vals && m->used) ? 0 : -1;
}
static void u32map_free(u32map* m) {
    free(m->keys);
    free(m->vals);
    free(m->used);
    memset(m, 0, sizeof(*m));
}
static void u32map_clear(u32map* m) {
    if (m->n) memset(m->used, 0, m->cap);
    m->n = 0;
}
/* Returns a pointer to the value slot of key k; *fresh = 1 if inserted. */
static int64_t* u32map_slot(u32map* m, uint32_t k, int* fresh) {
    if (2 * (m->n + 1) > m->cap) {
        u32map old = *m;
        if (u32map_init(m, old.cap)) { *m = old; return NULL; }
        for (uint64_t i = 0; i < old.cap; i++) {
            if (!old.used[i]) continue;
            int f;
            int64_t* p = u32map_slot(m, old.keys[i], &f);
            *p = old.vals[i];
        }
        u32map_free(&old);
    }
    uint64_t mask = m->cap - 1, i = hmix32(k) & mask;
    while (m->used[i]) {
        if (m->keys[i] == k) { *fresh = 0; return &m->vals[i]; }
        i = (i + 1) & mask;
    }
    m->used[i] = 1;
    m->keys[i] = k;
    m->vals[i] = 0;
    m->n++;
    *fresh = 1;
    return &m->vals[i];
}
static const int64_t* u32map_find(const u32map* m, uint32_t k) {
    uint64_t mask = m->cap - 1, i = hmix32(k) & mask;
    while (m->used[i]) {
        if (m->keys[i] == k) return &m->vals[i];
        i = (i + 1) & mask;
    }
    return NULL;
}

/* ------------------------------------------------------------------ */
/* L+S mapper (Include/L+S_mapper.hpp:11-160): a power-of-two "large" array
 * of (key, id) with a linear probe of 4 and a small spill map behind it;
 * insert returns the existing id or the next dense id (cnt++), find returns
 * the id or -1.  The hasher is the reference's identity myHasher
 * (Include/structures.hpp:93-95). */
typedef struct {
    uint32_t* key;
    int32_t* id;
    uint32_t size, mask;
    int32_t cnt;
    int shr;
    u32map spill;
} lsmap;

static int lsmap_init(lsmap* m, uint32_t n, int shr, int cache_n) {
    if (n < 1) n = 1; /* log2(0) is undefined in the reference */
    uint32_t sz = 1u << ((uint32_t)log2((double)n) + 2); /* L+S_mapper.hpp:23 */
    m->mask = sz - 1;
    m->size = sz + 3; /* linear probe 4 (L+S_mapper.hpp:25) */
    m->key = (uint32_t*)malloc((size_t)m->size * sizeof(uint32_t));
    m->id = (int32_t*)malloc((size_t)m->size * sizeof(int32_t));
    if (!m->key || !m->id) return -1;
    memset(m->key, 0xff, (size_t)m->size * sizeof(uint32_t));
    memset(m->id, 0xff, (size_t)m->size * sizeof(int32_t));
    m->cnt = 0;
    m->shr = shr;
    return u32map_init(&m->spill, (uint64_t)cache_n);
}
static void lsmap_free(lsmap* m) {
    free(m->key);
    free(m->id);
    u32map_free(&m->spill);
}
static void lsmap_clear(lsmap* m) { /* L+S_mapper.hpp:37-40 (cnt survives) */
    memset(m->key, 0xff, (size_t)m->size * sizeof(uint32_t));
    memset(m->id, 0xff, (size_t)m->size * sizeof(int32_t));
    u32map_clear(&m->spill);
}
static inline int32_t lsmap_insert(lsmap* m, uint32_t v) { /* L+S_mapper.hpp:64-114 */
    uint32_t b = (v >> m->shr) & m->mask;
    for (int p = 0; p < 4; p++, b++) {
        if (m->key[b] == v && m->id[b] != -1) return m->id[b];
        if (m->id[b] == -1) {
            m->key[b] = v;
            m->id[b] = m->cnt;
            return m->cnt++;
        }
    }
    int fresh;
    int64_t* s = u32map_slot(&m->spill, v, &fresh);
    if (fresh) { *s = m->cnt; return m->cnt++; }
    return (int32_t)*s;
}
static inline int32_t lsmap_find(const lsmap* m, uint32_t v) { /* L+S_mapper.hpp:116-159 */
    uint32_t b = (v >> m->shr) & m->mask;
    for (int p = 0; p < 4; p++, b++) {
        if (m->key[b] == v) return m->id[b];
        if (m->id[b] == -1) return -1;
    }
    const int64_t* s = u32map_find(&m->spill, v);
    return s ? (int32_t)*s : -1;
}

/* ------------------------------------------------------------------ */
/* Relations as columns: a = x (or z), b = y, v = optional payload. */
typedef struct {
    uint32_t* a;
    uint32_t* b;
    uint32_t* v; /* NULL when the relation carries no payload */
    uint32_t n;
} rel_t;

static int rel_alloc(rel_t* r, uint32_t n, int with_v) {
    size_t m = (size_t)(n ? n : 1);
    r->a = (uint32_t*)malloc(m * 4);
    r->b = (uint32_t*)malloc(m * 4);
    r->v = with_v ? (uint32_t*)malloc(m * 4) : NULL;
    r->n = n;
    return (r->a && r->b && (!with_v || r->v)) ? 0 : -1;
}
static void rel_free(rel_t* r) {
    free(r->a);
    free(r->b);
    free(r->v);
    memset(r, 0, sizeof(*r));
}

/* Radix partition by the low bits of a column under the identity hash:
 * histogram, prefix sum, stable scatter (dim3.hpp:668-698 partition_y,
 * dim3.hpp:600-631 partition_xz).  by_b selects the y column. */
static int partition_rel(const rel_t* in, rel_t* out, uint32_t* psum, int nparts, int by_b) {
    uint32_t mask = (uint32_t)nparts - 1;
    const uint32_t* key = by_b ? in->b : in->a;
    uint32_t* cur = (uint32_t*)calloc((size_t)nparts + 1, sizeof(uint32_t));
    if (!cur) return -1;
    for (uint32_t i = 0; i < in->n; i++) cur[key[i] & mask]++;
    psum[0] = 0;
    for (int i = 1; i <= nparts; i++) psum[i] = psum[i - 1] + cur[i - 1];
    memcpy(cur, psum, ((size_t)nparts + 1) * sizeof(uint32_t));
    if (rel_alloc(out, in->n, in->v != NULL)) { free(cur); return -1; }
    for (uint32_t i = 0; i < in->n; i++) {
        uint32_t d = cur[key[i] & mask]++;
        out->a[d] = in->a[i];
        out->b[d] = in->b[i];
        if (in->v) out->v[d] = in->v[i];
    }
    free(cur);
    return 0;
}

/* Partition count of mapping_step::mapping (dim3.hpp:406-409). */
static int mapping_partition_bits(uint32_t nR, uint32_t nS, unsigned tuple_bytes) {
    unsigned int target = 4u * L2_BYTES / tuple_bytes;
    if (target < PARTITION_PARA) target = PARTITION_PARA;
    unsigned int mx = nR > nS ? nR : nS;
    if (mx < (target << 1)) mx = target << 1;
    return (int)ceil(log2((double)(mx / target)));
}

typedef struct {
    uint32_t* id2x; /* ID2V.x */
    uint32_t* id2z; /* ID2V.z */
    int nx, ny, nz;
    rel_t Rm, Sm; /* (x id, y id[, v]) and (z id, y id[, v]) */
} mapped_t;

static void mapped_free(mapped_t* m) {
    free(m->id2x);
    free(m->id2z);
    rel_free(&m->Rm);
    rel_free(&m->Sm);
}

/* mapping_xz (dim3.hpp:734-792): dense ids for the a column, partition by
 * partition; one L+S mapper sized by the first partition, cleared per
 * partition with its counter kept, so ids stay dense across partitions. */
static int mapping_xz(const rel_t* V, const uint32_t* psum, int pbits, uint32_t** id2v, int* the_max, rel_t* out) {
    int nparts = 1 << pbits;
    lsmap hm;
    if (lsmap_init(&hm, psum[1] - psum[0], pbits, 16384 / 4)) return -1;
    uint32_t* rec = (uint32_t*)malloc((size_t)(V->n ? V->n : 1) * 4);
    if (!rec || rel_alloc(out, V->n, V->v != NULL)) { lsmap_free(&hm); free(rec); return -1; }
    for (int p = 0; p < nparts; p++) {
        lsmap_clear(&hm);
        for (uint32_t j = psum[p]; j < psum[p + 1]; j++) {
            int32_t id = lsmap_insert(&hm, V->a[j]);
            rec[id] = V->a[j]; /* insert(v, recorder) (L+S_mapper.hpp:58-62) */
            out->a[j] = (uint32_t)id;
            out->b[j] = V->b[j];
            if (V->v) out->v[j] = V->v[j];
        }
    }
    *the_max = hm.cnt - 1;
    *id2v = rec;
    lsmap_free(&hm);
    return 0;
}

/* mapping_step::mapping (dim3.hpp:399-455 pairs, :458-514 tuples). */
static int do_mapping(const rel_t* R, const rel_t* S, unsigned tuple_bytes, mapped_t* M) {
    memset(M, 0, sizeof(*M));
    int pbits = mapping_partition_bits(R->n, S->n, tuple_bytes);
    int nparts = 1 << pbits;
    uint32_t* psumR = (uint32_t*)malloc(((size_t)nparts + 1) * 4);
    uint32_t* psumS = (uint32_t*)malloc(((size_t)nparts + 1) * 4);
    rel_t pR = {0}, pS = {0}, Rt = {0}, St = {0}, Rp = {0}, Sp = {0};
    int rc = -1;
    if (!psumR || !psumS) goto done;
    if (partition_rel(R, &pR, psumR, nparts, 1) || partition_rel(S, &pS, psumS, nparts, 1)) goto done;

    /* mapping_y (dim3.hpp:795-836): build on R.y, probe with S.y, drop S
     * tuples without a partner (the semi-join). */
    {
        lsmap hm;
        if (lsmap_init(&hm, psumR[1] - psumR[0], pbits, 16384 / 4)) goto done;
        if (rel_alloc(&Rt, pR.n, pR.v != NULL) || rel_alloc(&St, pS.n, pS.v != NULL)) { lsmap_free(&hm); goto done; }
        uint32_t v2 = 0;
        for (int p = 0; p < nparts; p++) {
            lsmap_clear(&hm);
            for (uint32_t j = psumR[p]; j < psumR[p + 1]; j++) {
                Rt.a[j] = pR.a[j];
                Rt.b[j] = (uint32_t)lsmap_insert(&hm, pR.b[j]);
                if (pR.v) Rt.v[j] = pR.v[j];
            }
            for (uint32_t j = psumS[p]; j < psumS[p + 1]; j++) {
                int32_t t = lsmap_find(&hm, pS.b[j]);
                if (t != -1) {
                    St.a[v2] = pS.a[j];
                    St.b[v2] = (uint32_t)t;
                    if (pS.v) St.v[v2] = pS.v[j];
                    v2++;
                }
            }
        }
        M->ny = hm.cnt; /* ymax + 1 */
        St.n = v2;
        lsmap_free(&hm);
    }
    if (Rt.n == 0 || St.n == 0) { rc = 0; goto done; }

    /* x ids: partition_xz + mapping_xz on R (dim3.hpp:439-440). */
    {
        int xmax, zmax;
        if (partition_rel(&Rt, &Rp, psumR, nparts, 0)) goto done;
        if (mapping_xz(&Rp, psumR, pbits, &M->id2x, &xmax, &M->Rm)) goto done;
        M->nx = xmax + 1;
        /* z ids on the surviving S tuples (dim3.hpp:444-445). */
        if (partition_rel(&St, &Sp, psumS, nparts, 0)) goto done;
        if (mapping_xz(&Sp, psumS, pbits, &M->id2z, &zmax, &M->Sm)) goto done;
        M->nz = zmax + 1;
    }
    rc = 0;
done:
    free(psumR);
    free(psumS);
    rel_free(&pR);
    rel_free(&pS);
    rel_free(&Rt);
    rel_free(&St);
    rel_free(&Rp);
    rel_free(&Sp);
    return rc;
}

/* ------------------------------------------------------------------ */
/* CSR (dim3.hpp:22-26 CSR, :1058-1086 divide_R). */
typedef struct {
    int32_t* JR;
    int32_t* IC;
    uint32_t* VAL;
} csr_t;

static void csr_free(csr_t* c) {
    free(c->JR);
    free(c->IC);
    free(c->VAL);
    memset(c, 0, sizeof(*c));
}

/* Stable counting sort of (row, col[, val]) into CSR by row. */
static int build_csr(const uint32_t* row, const uint32_t* col, const uint32_t* val, uint32_t n, int nrows, csr_t* c) {
    c->JR = (int32_t*)malloc(((size_t)nrows + 1) * 4);
    c->IC = (int32_t*)malloc((size_t)(n ? n : 1) * 4);
    c->VAL = val ? (uint32_t*)malloc((size_t)(n ? n : 1) * 4) : NULL;
    int32_t* cur = (int32_t*)calloc((size_t)nrows + 1, 4);
    if (!c->JR || !c->IC || !cur || (val && !c->VAL)) { free(cur); return -1; }
    for (uint32_t i = 0; i < n; i++) cur[row[i]]++;
    c->JR[0] = 0;
    for (int i = 1; i <= nrows; i++) c->JR[i] = c->JR[i - 1] + cur[i - 1];
    memcpy(cur, c->JR, ((size_t)nrows + 1) * 4);
    for (uint32_t i = 0; i < n; i++) {
        int32_t d = cur[row[i]]++;
        c->IC[d] = (int32_t)col[i];
        if (val) c->VAL[d] = val[i];
    }
    free(cur);
    return 0;
}

/* ------------------------------------------------------------------ */
/* f2: per-z dense/sparse cost model (dim3.hpp:52-142). */
typedef struct {
    int32_t cnt_hist[200];
    int cnt_max;
    double base_sparse, base_dense, rw_nz;
    double cache[105];
    int interval;
} f2_t;

static int val2idx(int val) { /* dim3.hpp:108-112: decade*10 + leading digit */
    if (val <= 0) return 0;
    int d = 0, p = 1;
    while (val / p >= 10) { p *= 10; d++; }
    return d * 10 + val / p;
}

static void f2_init(f2_t* f, const int32_t* JR, int nx, int ny, int nz) {
    double rr_ny = rand_read_cost(ny);
    f->rw_nz = rand_rw_cost(nz);
    double dnR = (double)JR[nx] / 1e3;
    f->base_sparse = 2 * (double)nx / 1e3 * C_SEQ_READ / nz;
    f->base_sparse += dnR * C_SEQ_READ / nz;
    f->base_sparse += 2 * dnR * rr_ny / nz;
    f->base_dense = dnR * C_SZ_BITMAP / nz;
    memset(f->cnt_hist, 0, sizeof(f->cnt_hist));
    f->cnt_max = 0;
    for (int i = 0; i < nx; i++) {
        int t = val2idx(JR[i + 1] - JR[i]);
        if (t > f->cnt_max) f->cnt_max = t;
        f->cnt_hist[t]++;
    }
    for (int i = 0; i < 105; i++) f->cache[i] = -1;
    f->interval = ny / 100 > 1 ? ny / 100 : 1;
}

static double f2_sparse_hat(const f2_t* f, double outj) {
    return f->base_sparse + outj / 1e3 * (C_SEQ_READ + f->rw_nz);
}

static double f2_dense_hat(const f2_t* f, int Sm_cnt, int ny) {
    double p1 = stdmin(Sm_cnt / (double)ny, 1.);
    double pp = (double)Sm_cnt / ((double)ny * (double)ny);
    int nblk = (ny - 1) / 256 + 1;
    double ret = 0.;
    for (int i = 0, t = 0, tp = 1; i <= f->cnt_max; i++, t += tp) {
        double p256 = 1 - pow(1 - stdmin(pp * t, 1.), 256);
        double hat256 = p256 < 1e-5 ? 9e99 : (1 - pow(1 - p256, nblk)) / p256 * C_RX_DENSE;
        double hat1 = (1 - pow(1 - p1, t)) / p1 * C_RX_SPARSE;
        ret += stdmin(hat256, hat1) * f->cnt_hist[i];
        if (i != 0 && i % 10 == 0) {
            t -= tp / 2;
            tp *= 10;
            t -= tp / 2;
        }
    }
    return f->base_dense + (Sm_cnt * C_SZ_BITMAP + ret) * 1e-3;
}

static int f2_is_dense_better(f2_t* f, int Sm_cnt, int ny, int outj) {
    int t = Sm_cnt / f->interval;
    double dh;
    if (t < 105) {
        if (f->cache[t] == -1) f->cache[t] = f2_dense_hat(f, t * f->interval + f->interval / 2, ny);
        dh = f->cache[t];
    } else {
        dh = f2_dense_hat(f, t * f->interval + f->interval / 2, ny);
    }
    return dh < f2_sparse_hat(f, outj);
}

/* f3: per-row-length AVX-vs-probe threshold (dim3.hpp:144-186). */
static double f3_dense_hat(int nr, int ns, int k) {
    double p = (double)nr / (double)k * (double)ns / (double)k;
    p = 1 - pow(1 - p, 256);
    int kb = (k - 1) / 256 + 1;
    return (1 - pow(1 - p, kb)) / p * 1e-3 * C_RX_DENSE;
}
static double f3_sparse_hat(int nr, int ns, int k) {
    double p = (double)ns / (double)k;
    return (1 - pow(1 - p, nr)) / p * 1e-3 * C_RX_SPARSE;
}
static int f3_threshold(int nr, int k) {
    int lo = 1, hi = k;
    while (hi - lo > 5) {
        int mid = (lo + hi) >> 1;
        if (f3_dense_hat(nr, mid, k) < f3_sparse_hat(nr, mid, k)) hi = mid;
        else lo = mid;
    }
    for (int i = lo; i <= hi; i++)
        if (f3_dense_hat(nr, i, k) <= f3_sparse_hat(nr, i, k)) return i;
    return hi;
}

/* f1: classical vs hybrid (dim3.hpp:42-49). */
static int f1_classical_better(int nR, int nS, int64_t outj) {
    double f1 = (2 * nR + nS) * C_LS_BUILD + nS * C_LS_PROBE
              + outj * rand_rw_cost(nR < nS ? nR : nS) - outj * C_FLAT_HASH;
    return f1 > 0;
}

/* ------------------------------------------------------------------ */
/* divide_S (dim3.hpp:1088-1259): per-z S degree, OUTJ_CNT, f2 split into
 * dense z (one bitmap over y per z, ceil(ny/32) words padded to 8) and a
 * sparse CSR by y over the remaining tuples. */
typedef struct {
    int size;
    int words;      /* dense_bitvector_len */
    int32_t* id2v;  /* dense id -> z id */
    int32_t* id2cnt;
    uint32_t* bits; /* size * words */
} sdense_t;

static int divide_S(const rel_t* Sm, int nx, int ny, int nz, const csr_t* R, sdense_t* D, csr_t* Ssp) {
    memset(D, 0, sizeof(*D));
    memset(Ssp, 0, sizeof(*Ssp));
    int32_t* zcnt = (int32_t*)calloc((size_t)nz, 4);
    int32_t* z2d = (int32_t*)malloc((size_t)nz * 4);
    int32_t* rycnt = (int32_t*)calloc((size_t)ny, 4);
    uint32_t* outj = (uint32_t*)calloc((size_t)nz, 4);
    if (!zcnt || !z2d || !rycnt || !outj) return -1;
    memset(z2d, 0xff, (size_t)nz * 4);
    for (uint32_t i = 0; i < Sm->n; i++) zcnt[Sm->a[i]]++;
    for (int i = 0; i < R->JR[nx]; i++) rycnt[R->IC[i]]++;
    /* OUTJ_CNT is an int in the reference and may wrap; keep that. */
    for (uint32_t i = 0; i < Sm->n; i++) outj[Sm->a[i]] += (uint32_t)rycnt[Sm->b[i]];

    f2_t f2;
    f2_init(&f2, R->JR, nx, ny, nz);
    int dense = 0;
    for (int z = 0; z < nz; z++)
        if (f2_is_dense_better(&f2, zcnt[z], ny, (int32_t)outj[z])) z2d[z] = dense++;

    D->size = dense;
    D->words = ny / 32 + (ny % 32 ? 1 : 0);
    if (D->words % 8) D->words = (D->words / 8 + 1) * 8;
    int rc = -1;
    if (dense > 0) {
        D->id2v = (int32_t*)malloc((size_t)dense * 4);
        D->id2cnt = (int32_t*)malloc((size_t)dense * 4);
        D->bits = (uint32_t*)calloc((size_t)dense * (size_t)D->words, 4);
        if (!D->id2v || !D->id2cnt || !D->bits) goto out;
        for (int z = 0; z < nz; z++)
            if (z2d[z] != -1) {
                D->id2v[z2d[z]] = z;
                D->id2cnt[z2d[z]] = zcnt[z];
            }
    }
    if (dense == nz) {
        for (uint32_t i = 0; i < Sm->n; i++) {
            uint32_t* w = D->bits + (size_t)Sm->a[i] * D->words;
            w[Sm->b[i] >> 5] |= 1u << (Sm->b[i] & 31);
        }
        rc = 0;
        goto out;
    }
    {
        /* Keep sparse tuples in their order, set dense bits. */
        uint32_t ns = 0;
        uint32_t* ry = (uint32_t*)malloc((size_t)(Sm->n ? Sm->n : 1) * 4);
        uint32_t* rz = (uint32_t*)malloc((size_t)(Sm->n ? Sm->n : 1) * 4);
        if (!ry || !rz) { free(ry); free(rz); goto out; }
        for (uint32_t i = 0; i < Sm->n; i++) {
            int32_t d = z2d[Sm->a[i]];
            if (d != -1) {
                uint32_t* w = D->bits + (size_t)d * D->words;
                w[Sm->b[i] >> 5] |= 1u << (Sm->b[i] & 31);
            } else {
                ry[ns] = Sm->b[i];
                rz[ns] = Sm->a[i];
                ns++;
            }
        }
        int e = build_csr(ry, rz, NULL, ns, ny, Ssp);
        free(ry);
        free(rz);
        if (e) goto out;
    }
    rc = 0;
out:
    free(zcnt);
    free(z2d);
    free(rycnt);
    free(outj);
    return rc;
}

static void sdense_free(sdense_t* D) {
    free(D->id2v);
    free(D->id2cnt);
    free(D->bits);
    memset(D, 0, sizeof(*D));
}

/* ------------------------------------------------------------------ */
/* Hybrid_solution (dim3.hpp:889-974) for a range of x rows into one sink.
 * Dense block: per (x, dense z) either a 256-bit block AND test against a
 * lazily built x bitmap with early exit (AVX vptest in the reference,
 * dim3.hpp:916-934) or a probe of each y of the row (dim3.hpp:936-944),
 * chosen by f3.  Sparse block: Gustavson expansion with the SPA
 * last-writer array deduplicating z (dim3.hpp:952-973). */
typedef struct {
    const csr_t* R;
    const sdense_t* D;
    const csr_t* Ssp; /* JR == NULL when every z is dense */
    const uint32_t* id2x;
    const uint32_t* id2z;
    int nx, ny, nz;
    int f3len; /* length of each thread's f3 threshold cache */
} hybrid_t;

static int block_and_nonzero(const uint32_t* a, const uint32_t* b) {
    /* _mm256_testz_si256(a, b) == 0 over 8 words */
    uint32_t acc = 0;
    for (int i = 0; i < 8; i++) acc |= a[i] & b[i];
    return acc != 0;
}

static void hybrid_dense_rows(const hybrid_t* H, int x0, int x1, uint32_t* xbits, int32_t* f3cache, sink_t* out) {
    const csr_t* R = H->R;
    const sdense_t* D = H->D;
    for (int i = x0; i < x1; i++) {
        int len = R->JR[i + 1] - R->JR[i];
        if (len == 0) continue;
        uint32_t xv = H->id2x[i];
        int init = 0;
        int32_t thr = f3cache[len];
        if (thr == -1) {
            thr = f3_threshold(len, H->ny);
            f3cache[len] = thr;
        }
        for (int j = 0; j < D->size; j++) {
            const uint32_t* zb = D->bits + (size_t)j * D->words;
            uint32_t zv = H->id2z[D->id2v[j]];
            if (D->id2cnt[j] > thr) {
                if (!init) {
                    memset(xbits, 0, (size_t)D->words * 4);
                    for (int t = R->JR[i]; t < R->JR[i + 1]; t++) xbits[R->IC[t] >> 5] |= 1u << (R->IC[t] & 31);
                    init = 1;
                }
                for (int t = 0; t < D->words; t += 8)
                    if (block_and_nonzero(zb + t, xbits + t)) { emit_pair(out, xv, zv); break; }
            } else {
                for (int t = R->JR[i]; t < R->JR[i + 1]; t++) {
                    uint32_t y = (uint32_t)R->IC[t];
                    if (zb[y >> 5] & (1u << (y & 31))) { emit_pair(out, xv, zv); break; }
                }
            }
        }
    }
}

static void hybrid_sparse_rows(const hybrid_t* H, int x0, int x1, int32_t* spa, sink_t* out) {
    const csr_t* R = H->R;
    const csr_t* S = H->Ssp;
    for (int x = x0; x < x1; x++) {
        uint32_t xv = H->id2x[x];
        for (int i = R->JR[x]; i < R->JR[x + 1]; i++) {
            int y = R->IC[i];
            for (int j = S->JR[y]; j < S->JR[y + 1]; j++) {
                int z = S->IC[j];
                if (spa[z] != x) {
                    spa[z] = x;
                    emit_pair(out, xv, H->id2z[z]);
                }
            }
        }
    }
}

/* ------------------------------------------------------------------ */
/* Estimator (dim3.hpp:193-224) with the identity hash. */
int64_t dim3o_estimate(const uint32_t* R, uint64_t nR, const uint32_t* S, uint64_t nS) {
    int bits = 0;
    for (int ss = (int)nS; ss > 10000; ss /= 2) bits++;
    uint32_t mask = (1u << bits) - 1;
    u32map m;
    if (u32map_init(&m, 10000)) return 0;
    for (uint64_t i = 0; i < nS; i++) {
        uint32_t y = S[2 * i + 1];
        if ((y & mask) == 0) {
            int f;
            int64_t* p = u32map_slot(&m, y, &f);
            (*p)++;
        }
    }
    int64_t result = 0;
    for (uint64_t i = 0; i < nR; i++) {
        uint32_t y = R[2 * i + 1];
        if ((y & mask) == 0) {
            const int64_t* p = u32map_find(&m, y);
            if (p) result += *p;
        }
    }
    if (result == 0) {
        u32map_clear(&m);
        uint64_t kR = nR < 1000 ? nR : 1000, kS = nS < 1000 ? nS : 1000;
        for (uint64_t i = 0; i < kR; i++) {
            int f;
            int64_t* p = u32map_slot(&m, R[2 * i + 1], &f);
            (*p)++;
        }
        for (uint64_t i = 0; i < kS; i++) {
            const int64_t* p = u32map_find(&m, S[2 * i + 1]);
            if (p) result += *p;
        }
        u32map_free(&m);
        return (int64_t)(result * ((double)nR / 1e3) * ((double)nS / 1e3));
    }
    u32map_free(&m);
    return result << bits;
}

/* ------------------------------------------------------------------ */
/* Classical radix hash join + projection into a hash set (dim3.hpp:273-391). */
typedef struct {
    uint64_t* k;
    uint64_t cap, n;
} pairset;
#define PS_EMPTY 0xFFFFFFFFFFFFFFFFULL
static int pairset_init(pairset* s, uint64_t want) {
    uint64_t cap = 64;
    while (cap < 2 * want) cap <<= 1;
    s->k = (uint64_t*)malloc(cap * 8);
    if (!s->k) return -1;
    memset(s->k, 0xff, cap * 8);
    s->cap = cap;
    s->n = 0;
    return 0;
}
static int pairset_insert(pairset* s, uint64_t key, int* had_max);
static int pairset_rehash(pairset* s) {
    pairset o = *s;
    if (pairset_init(s, o.cap)) { *s = o; return -1; }
    int hm = 0;
    for (uint64_t i = 0; i < o.cap; i++)
        if (o.k[i] != PS_EMPTY) pairset_insert(s, o.k[i], &hm);
    free(o.k);
    return 0;
}
/* The all-ones key (x = z = 0xFFFFFFFF) is tracked outside the table. */
static int pairset_insert(pairset* s, uint64_t key, int* had_max) {
    if (key == PS_EMPTY) { *had_max = 1; return 0; }
    if (2 * (s->n + 1) > s->cap && pairset_rehash(s)) return -1;
    uint64_t mask = s->cap - 1, i = mix64(key) & mask;
    while (s->k[i] != PS_EMPTY) {
        if (s->k[i] == key) return 0;
        i = (i + 1) & mask;
    }
    s->k[i] = key;
    s->n++;
    return 0;
}

int dim3o_classical(const uint32_t* R, uint64_t nR, const uint32_t* S, uint64_t nS,
                    uint32_t** out, uint64_t* n_out, uint64_t* set_hash) {
    /* partition parameters (dim3.hpp:277-282, 292) */
    int para = (int)(L2_BYTES / 8 / 2);
    int bucket_bits = (int)ceil(log2((double)(L2_BYTES / 2 / LINE_BYTES)));
    int bmask = (1 << bucket_bits) - 1;
    int mx = (int)(nR > nS ? nR : nS);
    if (mx < (para << 1)) mx = para << 1;
    int pbits = (int)ceil(log2((double)(mx / para)));
    int nparts = 1 << pbits;
    rel_t r = {0}, s = {0}, pr = {0}, ps = {0};
    uint32_t* psR = (uint32_t*)malloc(((size_t)nparts + 1) * 4);
    uint32_t* psS = (uint32_t*)malloc(((size_t)nparts + 1) * 4);
    int32_t* head = (int32_t*)malloc(((size_t)bmask + 1) * 4);
    int32_t* next = (int32_t*)malloc((size_t)(nR ? nR : 1) * 4);
    pairset set = {0};
    int has_max = 0, rc = -1;
    if (!psR || !psS || !head || !next) goto done;
    if (rel_alloc(&r, (uint32_t)nR, 0) || rel_alloc(&s, (uint32_t)nS, 0)) goto done;
    for (uint64_t i = 0; i < nR; i++) { r.a[i] = R[2 * i]; r.b[i] = R[2 * i + 1]; }
    for (uint64_t i = 0; i < nS; i++) { s.a[i] = S[2 * i]; s.b[i] = S[2 * i + 1]; }
    if (partition_rel(&r, &pr, psR, nparts, 1) || partition_rel(&s, &ps, psS, nparts, 1)) goto done;
    if (pairset_init(&set, 1024)) goto done;
    for (int p = 0; p < nparts; p++) {
        memset(head, 0xff, ((size_t)bmask + 1) * 4);
        for (uint32_t i = psR[p]; i < psR[p + 1]; i++) {
            int b = (int)((pr.b[i] >> pbits) & (uint32_t)bmask);
            next[i] = head[b];
            head[b] = (int32_t)i;
        }
        for (uint32_t i = psS[p]; i < psS[p + 1]; i++) {
            int b = (int)((ps.b[i] >> pbits) & (uint32_t)bmask);
            for (int32_t e = head[b]; e != -1; e = next[e])
                if (pr.b[e] == ps.b[i] && pairset_insert(&set, ((uint64_t)pr.a[e] << 32) | ps.a[i], &has_max)) goto done;
        }
    }
    {
        uint64_t n = set.n + (uint64_t)has_max, h = 0, w = 0;
        uint32_t* o = out ? (uint32_t*)malloc((size_t)(n ? n : 1) * 8) : NULL;
        if (out && !o) goto done;
        for (uint64_t i = 0; i < set.cap; i++) {
            if (set.k[i] == PS_EMPTY) continue;
            uint32_t x = (uint32_t)(set.k[i] >> 32), z = (uint32_t)set.k[i];
            h += dim3o_pair_hash(x, z);
            if (o) { o[2 * w] = x; o[2 * w + 1] = z; }
            w++;
        }
        if (has_max) {
            h += dim3o_pair_hash(0xFFFFFFFFu, 0xFFFFFFFFu);
            if (o) { o[2 * w] = 0xFFFFFFFFu; o[2 * w + 1] = 0xFFFFFFFFu; }
        }
        if (out) *out = o;
        *n_out = n;
        if (set_hash) *set_hash = h;
    }
    rc = 0;
done:
    free(psR); free(psS); free(head); free(next); free(set.k);
    rel_free(&r); rel_free(&s); rel_free(&pr); rel_free(&ps);
    return rc;
}

/* ------------------------------------------------------------------ */
static int load_rel(const uint32_t* P, uint64_t n, const float* v, rel_t* r) {
    if (rel_alloc(r, (uint32_t)n, v != NULL)) return -1;
    for (uint64_t i = 0; i < n; i++) {
        r->a[i] = P[2 * i];
        r->b[i] = P[2 * i + 1];
    }
    if (v) memcpy(r->v, v, (size_t)n * 4);
    return 0;
}

static void sink_merge(sink_t* dst, sink_t* parts, int np) {
    uint64_t total = dst->n;
    for (int t = 0; t < np; t++) total += parts[t].n;
    if (dst->hash_only) {
        for (int t = 0; t < np; t++) dst->hash += parts[t].hash;
        dst->n = total;
        return;
    }
    while (dst->cap < total) if (sink_grow(dst)) return;
    for (int t = 0; t < np; t++) {
        if (parts[t].n) memcpy(dst->xz + 2 * dst->n, parts[t].xz, (size_t)parts[t].n * 8);
        dst->n += parts[t].n;
    }
}

/* DIM3::doJoinProject (dim3.hpp:987-1055) and
 * DIM3_parallel::doJoinProject_parallel (dim3_parallel.hpp:142-210). */
int dim3o_join_project(const uint32_t* R_in, uint64_t nR_in, const uint32_t* S_in, uint64_t nS_in,
                       int threads, int hash_only,
                       uint32_t** out, uint64_t* n_out, uint64_t* set_hash,
                       dim3o_stats* st) {
    dim3o_stats local;
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    /* R is the larger input (dim3.hpp:993-994). */
    const uint32_t *Rp = R_in, *Sp = S_in;
    uint64_t nR = nR_in, nS = nS_in;
    if (nR_in < nS_in) {
        Rp = S_in; Sp = R_in; nR = nS_in; nS = nR_in;
        st->swapped = 1;
    }
    sink_t sink = {0};
    sink.hash_only = hash_only;
    *n_out = 0;
    if (out) *out = NULL;
    if (set_hash) *set_hash = 0;
    if (nR == 0 || nS == 0) return 0;

    double t0 = now_s();
    st->out_j_hat = dim3o_estimate(Rp, nR, Sp, nS);
    double t1 = now_s();
    st->t_estimate = t1 - t0;
    if (threads <= 1 && f1_classical_better((int)nR, (int)nS, st->out_j_hat)) {
        st->used_classical = 1;
        uint64_t h = 0;
        int e = dim3o_classical(Rp, nR, Sp, nS, hash_only ? NULL : out, n_out, &h);
        if (set_hash) *set_hash = h;
        st->t_expand = now_s() - t1;
        return e;
    }

    rel_t R = {0}, S = {0};
    mapped_t M;
    csr_t Rall = {0}, Ssp = {0};
    sdense_t D = {0};
    int rc = -1;
    if (load_rel(Rp, nR, NULL, &R) || load_rel(Sp, nS, NULL, &S)) goto done;
    if (do_mapping(&R, &S, 8, &M)) goto done;
    double t2 = now_s();
    st->t_mapping = t2 - t1;
    if (M.Rm.n == 0 || M.Sm.n == 0) { rc = 0; mapped_free(&M); goto done; }
    st->nx = M.nx; st->ny = M.ny; st->nz = M.nz;

    if (build_csr(M.Rm.a, M.Rm.b, NULL, M.Rm.n, M.nx, &Rall)) { mapped_free(&M); goto done; }
    if (divide_S(&M.Sm, M.nx, M.ny, M.nz, &Rall, &D, &Ssp)) { mapped_free(&M); goto done; }
    st->n_dense_z = D.size;
    {
        /* exact OUT_J = sum_y degR(y) * degS(y) over the mapped relations */
        int64_t* dR = (int64_t*)calloc((size_t)M.ny, 8);
        int64_t* dS = (int64_t*)calloc((size_t)M.ny, 8);
        if (dR && dS) {
            for (uint32_t i = 0; i < M.Rm.n; i++) dR[M.Rm.b[i]]++;
            for (uint32_t i = 0; i < M.Sm.n; i++) dS[M.Sm.b[i]]++;
            uint64_t oj = 0;
            for (int y = 0; y < M.ny; y++) oj += (uint64_t)(dR[y] * dS[y]);
            st->out_j = oj;
        }
        free(dR);
        free(dS);
    }
    double t3 = now_s();
    st->t_divide = t3 - t2;
    {
        hybrid_t H;
        H.R = &Rall; H.D = &D; H.Ssp = Ssp.JR ? &Ssp : NULL;
        H.id2x = M.id2x; H.id2z = M.id2z;
        H.nx = M.nx; H.ny = M.ny; H.nz = M.nz;
        int maxlen = 0;
        for (int i = 0; i < M.nx; i++) {
            int l = Rall.JR[i + 1] - Rall.JR[i];
            if (l > maxlen) maxlen = l;
        }
        H.f3len = (M.ny > maxlen + 1 ? M.ny : maxlen + 1);
        int nt = threads < 1 ? 1 : threads;
        if (nt == 1) {
            uint32_t* xb = (uint32_t*)malloc((size_t)(D.words ? D.words : 8) * 4);
            int32_t* spa = H.Ssp ? (int32_t*)malloc((size_t)M.nz * 4) : NULL;
            int32_t* f3c = (int32_t*)malloc((size_t)H.f3len * 4);
            memset(f3c, 0xff, (size_t)H.f3len * 4);
            if (D.size > 0) hybrid_dense_rows(&H, 0, M.nx, xb, f3c, &sink);
            if (H.Ssp) {
                memset(spa, 0xff, (size_t)M.nz * 4);
                hybrid_sparse_rows(&H, 0, M.nx, spa, &sink);
            }
            free(xb);
            free(spa);
            free(f3c);
        } else {
            sink_t* parts = (sink_t*)calloc((size_t)nt, sizeof(sink_t));
            for (int t = 0; t < nt; t++) parts[t].hash_only = hash_only;
            /* dynamic schedule, chunk 30 (dim3_parallel.hpp:43, 102) */
#pragma omp parallel num_threads(nt)
            {
                int tid = 0;
#ifdef _OPENMP
                tid = omp_get_thread_num();
#endif
                uint32_t* xb = (uint32_t*)malloc((size_t)(D.words ? D.words : 8) * 4);
                int32_t* spa = H.Ssp ? (int32_t*)malloc((size_t)M.nz * 4) : NULL;
                int32_t* f3c = (int32_t*)malloc((size_t)H.f3len * 4);
                memset(f3c, 0xff, (size_t)H.f3len * 4);
                if (D.size > 0) {
#pragma omp for schedule(dynamic, 30)
                    for (int x = 0; x < M.nx; x++) hybrid_dense_rows(&H, x, x + 1, xb, f3c, &parts[tid]);
                }
                if (H.Ssp) {
                    memset(spa, 0xff, (size_t)M.nz * 4);
#pragma omp for schedule(dynamic, 30)
                    for (int x = 0; x < M.nx; x++) hybrid_sparse_rows(&H, x, x + 1, spa, &parts[tid]);
                }
                free(xb);
                free(spa);
                free(f3c);
            }
            sink_merge(&sink, parts, nt);
            for (int t = 0; t < nt; t++) {
                if (parts[t].oom) sink.oom = 1;
                free(parts[t].xz);
            }
            free(parts);
        }
    }
    st->t_expand = now_s() - t3;
    mapped_free(&M);
    rc = sink.oom ? -1 : 0;
done:
    rel_free(&R);
    rel_free(&S);
    csr_free(&Rall);
    csr_free(&Ssp);
    sdense_free(&D);
    if (rc == 0) {
        *n_out = sink.n;
        if (set_hash) *set_hash = hash_only ? sink.hash : 0;
        if (!hash_only && set_hash) {
            uint64_t h = 0;
            for (uint64_t i = 0; i < sink.n; i++) h += dim3o_pair_hash(sink.xz[2 * i], sink.xz[2 * i + 1]);
            *set_hash = h;
        }
        if (out) *out = sink.xz;
        else free(sink.xz);
    } else {
        free(sink.xz);
    }
    return rc;
}

/* ------------------------------------------------------------------ */
/* SpmmAggregate (dim3.hpp:1271-1310) with the COUNT plug-in
 * (insert -> 1, update -> +1, get -> count), emitting each x row's groups
 * in first-seen z order. */
static void spmm_count_rows(const csr_t* R, const csr_t* S, const uint32_t* id2x, const uint32_t* id2z,
                            int x0, int x1, int32_t* spa, int32_t* list, uint64_t* acc, sink_t* out) {
    for (int x = x0; x < x1; x++) {
        uint32_t xv = id2x[x];
        int nl = 0;
        for (int i = R->JR[x]; i < R->JR[x + 1]; i++) {
            int y = R->IC[i];
            for (int j = S->JR[y]; j < S->JR[y + 1]; j++) {
                int z = S->IC[j];
                if (spa[z] != x) {
                    spa[z] = x;
                    acc[z] = 1;
                    list[nl++] = z;
                } else {
                    acc[z]++;
                }
            }
        }
        for (int i = 0; i < nl; i++) emit_group(out, xv, id2z[list[i]], acc[list[i]]);
    }
}

/* Shared front half of DIM3JoinAggregate::doJoinAggregate (dim3.hpp:1318-1373):
 * swap, TUPLE mapping, divide_R with VAL (dim3.hpp:1376-1408) and an
 * all-sparse divide_S with VAL (dim3.hpp:1410-1450). */
static int agg_prepare(const uint32_t* R_in, const float* Rv_in, uint64_t nR_in,
                       const uint32_t* S_in, const float* Sv_in, uint64_t nS_in,
                       unsigned tuple_bytes, mapped_t* M, csr_t* Rall, csr_t* Ssp, dim3o_stats* st) {
    const uint32_t *Rp = R_in, *Sp = S_in;
    const float *Rv = Rv_in, *Sv = Sv_in;
    uint64_t nR = nR_in, nS = nS_in;
    if (nR_in < nS_in) {
        Rp = S_in; Sp = R_in; Rv = Sv_in; Sv = Rv_in; nR = nS_in; nS = nR_in;
        st->swapped = 1;
    }
    memset(M, 0, sizeof(*M));
    if (nR == 0 || nS == 0) return 0;
    double t0 = now_s();
    st->out_j_hat = dim3o_estimate(Rp, nR, Sp, nS);
    double t1 = now_s();
    st->t_estimate = t1 - t0;
    rel_t R = {0}, S = {0};
    int rc = -1;
    if (load_rel(Rp, nR, Rv, &R) || load_rel(Sp, nS, Sv, &S)) goto done;
    if (do_mapping(&R, &S, tuple_bytes, M)) goto done;
    double t2 = now_s();
    st->t_mapping = t2 - t1;
    if (M->Rm.n == 0 || M->Sm.n == 0) { rc = 0; goto done; }
    st->nx = M->nx; st->ny = M->ny; st->nz = M->nz;
    if (build_csr(M->Rm.a, M->Rm.b, M->Rm.v, M->Rm.n, M->nx, Rall)) goto done;
    if (build_csr(M->Sm.b, M->Sm.a, M->Sm.v, M->Sm.n, M->ny, Ssp)) goto done;
    st->t_divide = now_s() - t2;
    rc = 0;
done:
    rel_free(&R);
    rel_free(&S);
    return rc;
}

int dim3o_join_count(const uint32_t* R_in, uint64_t nR_in, const uint32_t* S_in, uint64_t nS_in,
                     int threads, int hash_only,
                     uint32_t** out_xz, uint64_t** out_cnt, uint64_t* n_out,
                     uint64_t* set_hash, dim3o_stats* st) {
    dim3o_stats local;
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    mapped_t M;
    csr_t Rall = {0}, Ssp = {0};
    sink_t sink = {0};
    sink.hash_only = hash_only;
    if (!hash_only) {
        sink.cnt = (uint64_t*)malloc(1024 * 8);
        sink.xz = (uint32_t*)malloc(1024 * 8);
        sink.cap = 1024;
        if (!sink.cnt || !sink.xz) return -1;
    }
    *n_out = 0;
    /* COUNT needs an integer Tv: TUPLE<int,int,long long> is 16 bytes. */
    int rc = agg_prepare(R_in, NULL, nR_in, S_in, NULL, nS_in, 16, &M, &Rall, &Ssp, st);
    if (rc == 0 && M.Rm.n && M.Sm.n) {
        double t3 = now_s();
        int nt = threads < 1 ? 1 : threads;
        if (nt == 1) {
            int32_t* spa = (int32_t*)malloc((size_t)M.nz * 4);
            int32_t* list = (int32_t*)malloc((size_t)M.nz * 4);
            uint64_t* acc = (uint64_t*)malloc((size_t)M.nz * 8);
            if (!spa || !list || !acc) rc = -1;
            else {
                memset(spa, 0xff, (size_t)M.nz * 4);
                spmm_count_rows(&Rall, &Ssp, M.id2x, M.id2z, 0, M.nx, spa, list, acc, &sink);
            }
            free(spa); free(list); free(acc);
        } else {
            sink_t* parts = (sink_t*)calloc((size_t)nt, sizeof(sink_t));
            for (int t = 0; t < nt; t++) {
                parts[t].hash_only = hash_only;
                if (!hash_only) {
                    parts[t].cnt = (uint64_t*)malloc(1024 * 8);
                    parts[t].xz = (uint32_t*)malloc(1024 * 8);
                    parts[t].cap = 1024;
                }
            }
#pragma omp parallel num_threads(nt)
            {
                int tid = 0;
#ifdef _OPENMP
                tid = omp_get_thread_num();
#endif
                int32_t* spa = (int32_t*)malloc((size_t)M.nz * 4);
                int32_t* list = (int32_t*)malloc((size_t)M.nz * 4);
                uint64_t* acc = (uint64_t*)malloc((size_t)M.nz * 8);
                memset(spa, 0xff, (size_t)M.nz * 4);
#pragma omp for schedule(dynamic, 30)
                for (int x = 0; x < M.nx; x++) spmm_count_rows(&Rall, &Ssp, M.id2x, M.id2z, x, x + 1, spa, list, acc, &parts[tid]);
                free(spa); free(list); free(acc);
            }
            for (int t = 0; t < nt; t++) {
                if (parts[t].oom) sink.oom = 1;
                if (hash_only) { sink.hash += parts[t].hash; sink.n += parts[t].n; continue; }
                for (uint64_t i = 0; i < parts[t].n; i++)
                    emit_group(&sink, parts[t].xz[2 * i], parts[t].xz[2 * i + 1], parts[t].cnt[i]);
                free(parts[t].xz);
                free(parts[t].cnt);
            }
            free(parts);
        }
        st->t_expand = now_s() - t3;
    }
    mapped_free(&M);
    csr_free(&Rall);
    csr_free(&Ssp);
    if (rc == 0 && sink.oom) rc = -1;
    if (rc != 0) { free(sink.xz); free(sink.cnt); return rc; }
    *n_out = sink.n;
    if (set_hash) {
        if (hash_only) *set_hash = sink.hash;
        else {
            uint64_t h = 0;
            for (uint64_t i = 0; i < sink.n; i++) h += dim3o_group_hash(sink.xz[2 * i], sink.xz[2 * i + 1], sink.cnt[i]);
            *set_hash = h;
        }
    }
    if (out_xz) *out_xz = sink.xz; else free(sink.xz);
    if (out_cnt) *out_cnt = sink.cnt; else free(sink.cnt);
    return 0;
}

/* AVG(R.v + S.v) with the reference's float accumulation order
 * (AggregateFunctionAvg, dim3.hpp:1453-1480). */
int dim3o_join_avg(const uint32_t* R_in, const float* Rv, uint64_t nR_in,
                   const uint32_t* S_in, const float* Sv, uint64_t nS_in,
                   uint32_t** out_xz, float** out_avg, uint64_t* n_out, dim3o_stats* st) {
    dim3o_stats local;
    if (!st) st = &local;
    memset(st, 0, sizeof(*st));
    mapped_t M;
    csr_t Rall = {0}, Ssp = {0};
    *n_out = 0;
    int rc = agg_prepare(R_in, Rv, nR_in, S_in, Sv, nS_in, 12, &M, &Rall, &Ssp, st);
    uint32_t* oxz = NULL;
    float* oav = NULL;
    uint64_t n = 0, cap = 0;
    if (rc == 0 && M.Rm.n && M.Sm.n) {
        int32_t* spa = (int32_t*)malloc((size_t)M.nz * 4);
        int32_t* list = (int32_t*)malloc((size_t)M.nz * 4);
        float* sum = (float*)malloc((size_t)M.nz * 4);
        int32_t* cnt = (int32_t*)malloc((size_t)M.nz * 4);
        if (!spa || !list || !sum || !cnt) rc = -1;
        else {
            memset(spa, 0xff, (size_t)M.nz * 4);
            for (int x = 0; x < M.nx && rc == 0; x++) {
                int nl = 0;
                for (int i = Rall.JR[x]; i < Rall.JR[x + 1]; i++) {
                    int y = Rall.IC[i];
                    float v1;
                    memcpy(&v1, &Rall.VAL[i], 4);
                    for (int j = Ssp.JR[y]; j < Ssp.JR[y + 1]; j++) {
                        int z = Ssp.IC[j];
                        float v2;
                        memcpy(&v2, &Ssp.VAL[j], 4);
                        if (spa[z] != x) {
                            spa[z] = x;
                            sum[z] = v1 + v2;
                            cnt[z] = 1;
                            list[nl++] = z;
                        } else {
                            sum[z] += v1 + v2;
                            cnt[z]++;
                        }
                    }
                }
                for (int i = 0; i < nl; i++) {
                    if (n == cap) {
                        cap = cap ? 2 * cap : 1024;
                        uint32_t* a = (uint32_t*)realloc(oxz, cap * 8);
                        float* b = (float*)realloc(oav, cap * 4);
                        if (!a || !b) { free(a ? a : oxz); free(b ? b : oav); oxz = NULL; oav = NULL; rc = -1; break; }
                        oxz = a; oav = b;
                    }
                    oxz[2 * n] = M.id2x[x];
                    oxz[2 * n + 1] = M.id2z[list[i]];
                    oav[n] = sum[list[i]] / cnt[list[i]];
                    n++;
                }
            }
        }
        free(spa); free(list); free(sum); free(cnt);
    }
    mapped_free(&M);
    csr_free(&Rall);
    csr_free(&Ssp);
    if (rc != 0) { free(oxz); free(oav); return rc; }
    *n_out = n;
    if (out_xz) *out_xz = oxz; else free(oxz);
    if (out_avg) *out_avg = oav; else free(oav);
    return 0;
}

void dim3o_free(void* p) { free(p); }

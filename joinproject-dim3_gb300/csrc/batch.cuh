// batch.cuh -- many joins per launch.
//
// Relation set: for every relation r of a set (tuples (f, y), f the first
// column) one segmented pass builds, for all relations at once,
//   TF, TY      value -> id tables (f and y), ids dense per relation
//   CSR by f    JRf over the global f-id space, ICf = global y ids
//               (the relation in the role of R)
//   CSR by (y, f tile)  JRy over a per-relation key space y*T + tile (plus
//               T empty sentinel keys), ICy = local f ids, VSy = f values
//               beside them (the relation in the role of S)
// Every relation's ids and keys are local; the set lays them out
// relation-major, so one prefix sum over a whole pool gives every
// relation's CSR at once (a relation's first global position is the tuple
// count of the relations before it).
//
// Query set: joins (P, Q) of relations of a set.  Per query a y map (P's y
// ids -> Q's y ids, or Q's empty sentinel row), P's CSR re-expressed in Q's
// y ids, per-row work and classes; then the row kernels of the single
// relation path run over the rows of all queries, each row fetching its
// query's context.  Kernels take their segment offsets from device memory,
// so a fixed launch sequence (capturable in a CUDA graph) serves any batch
// of a given shape.
#pragma once
#include "aggregate.cuh"
#include "common.cuh"
#include "expand.cuh"
#include "mapping.cuh"
#include "single.cuh"

namespace dim3g {

// Largest s in [0, n) with off[s] <= i (off[0..n] nondecreasing, off[0] = 0,
// i < off[n]): the segment holding element i, skipping empty segments.
__device__ __forceinline__ uint32_t seg_find(const uint64_t* __restrict__ off, uint32_t n, uint64_t i) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&off[mid]) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Per-thread cached segment lookup for loops over contiguous elements.
struct SegCursor {
    const uint64_t* off;
    uint32_t n;
    uint32_t s = 0;
    uint64_t lo = 1, hi = 0;
    __device__ __forceinline__ uint32_t at(uint64_t i) {
        if (i < lo || i >= hi) {
            s = seg_find(off, n, i);
            lo = __ldg(&off[s]);
            hi = __ldg(&off[s + 1]);
        }
        return s;
    }
};

// Grid-ordered element ranges: in round k CTA b takes the elements
// [(k * G + b) * blockDim, + blockDim), G the grid, so the whole grid works
// inside a window of about G * blockDim consecutive elements that moves
// through the relations in order.  The random-address updates of the index
// build (table slots, degree and cursor atomics, the CSR scatter) then fall
// in the few relations under the window, whose tables and CSR slices stay in
// L2, instead of in all of the set at once (CTA-contiguous ranges put the
// grid's CTAs in as many different relations).  The segment of an element is
// looked up again when a thread's next element lies in another relation.
#define DIM3G_FOR_CHUNK(i, n) \
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < (n); i += (uint64_t)gridDim.x * blockDim.x)

// Adds pred over the calling lanes to ctr[s], one atomic per group of lanes
// sharing s.
__device__ __forceinline__ void warp_count_by_seg(unsigned long long* ctr, uint32_t s, bool pred) {
    const unsigned act = __activemask();
    const unsigned grp = __match_any_sync(act, s);
    const unsigned b = __ballot_sync(act, pred) & grp;
    if (b && (int)lane_id() == __ffs(grp) - 1) atomicAdd(&ctr[s], (unsigned long long)__popc(b));
}

// ------------------------------------------------------------ relation set
struct RelIn {
    const uint2* pairs;  // (f, y) tuples, device
    uint64_t n;
};

// Per-relation layout, computed on the device once the id counts are known.
struct RelDev {
    uint64_t nt;        // tuples
    uint64_t tup_off;   // first position in the tuple-indexed pools
    uint64_t tab_off;   // first slot in TF / TY
    uint64_t tab_cap;   // slots per table (power of two)
    uint64_t nf, ny;    // distinct f, distinct y
    uint64_t fbase, ybase;  // first global f id / y id
    uint64_t yt_base;   // first key of the (y, f tile) key space
    uint32_t T, tile_shift, tile_width;
    uint32_t probe_lim; // longest probe of the tables (0: the whole table)
};

// The CSRs a relation's queries read: kRoleRows, by first value (the
// relation drives the rows of a join); kRoleCols, by (y, z tile) (its first
// values are a join's output column).
enum RelRole : uint8_t { kRoleRows = 1, kRoleCols = 2 };

// Pools of one relation set (device pointers).
struct RelPools {
    const RelIn* in;
    RelDev* rel;
    const uint64_t* tup_off;  // nrel + 1
    const uint64_t* tab_off;  // nrel + 1
    uint32_t nrel;
    uint32_t probe_lim;       // sketch-sized tables: longest probe (0: tuple-sized tables)
    uint64_t ntot;            // sum of tuples
    unsigned long long* TF;
    unsigned long long* TY;
    unsigned long long* nf_cnt;  // nrel
    unsigned long long* ny_cnt;  // nrel
    uint32_t* id2f;           // by global f id
    uint32_t* id2y;           // by global y id
    uint2* Pm;                // (global f id, global y id) per tuple
    uint32_t* degF;           // ntot + 1
    uint32_t* JRf;            // ntot + 1, global positions
    uint32_t* curF;
    uint32_t* ICf;            // global y ids
    uint32_t* ICr;            // the row (local f id) of each ICf entry
    uint32_t* cnt_yt;         // yt_cap
    uint32_t* JRy;            // yt_cap, global positions
    uint32_t* curY;
    uint64_t yt_cap;
    uint32_t* ICy;            // local f ids
    uint32_t* VSy;            // f values
    uint32_t* err;            // device error flags of the set
    unsigned long long* yt_need;  // keys the layout needs (+1)
    unsigned long long* f_need;   // first-value ids of the set (+1): the by-first-value row pointers scanned
    uint64_t* yoff;           // nrel + 1: first global y id of each relation
    const uint8_t* roles;     // nrel: RelRole bits (CSRs built for the relation)
};

__device__ __forceinline__ DevTable rel_table(unsigned long long* pool, const RelDev& r) {
    return DevTable{pool + r.tab_off, r.tab_cap - 1, r.probe_lim};
}

static __global__ void k_ix_insert(RelPools P) {
    SegCursor sc{P.tup_off, P.nrel};
    DIM3G_FOR_CHUNK(i, P.ntot) {
        const uint32_t r = sc.at(i);
        const uint2 t = P.in[r].pairs[i - sc.lo];
        const uint64_t to = __ldg(&P.tab_off[r]), cap = __ldg(&P.tab_off[r + 1]) - to;
        const bool nf = table_insert(DevTable{P.TF + to, cap - 1, P.probe_lim}, t.x, P.err);
        const bool ny = table_insert(DevTable{P.TY + to, cap - 1, P.probe_lim}, t.y, P.err);
        warp_count_by_seg(P.nf_cnt, r, nf);
        warp_count_by_seg(P.ny_cnt, r, ny);
    }
}

// Distinct-key sketches of every relation's two columns (kSketchRegs
// registers per column, zeroed by the caller): relation r's first column at
// regs + 2 r kSketchRegs, its y column after it.  Grid-ordered, so a warp's
// updates fall in one or two relations' registers.
static __global__ void k_rel_sketch(RelPools P, uint32_t* regs) {
    SegCursor sc{P.tup_off, P.nrel};
    DIM3G_FOR_CHUNK(i, P.ntot) {
        const uint32_t r = sc.at(i);
        const uint2 t = P.in[r].pairs[i - sc.lo];
        uint32_t* rr = regs + (uint64_t)2 * r * kSketchRegs;
        sketch_add_if_larger(rr, t.x);
        sketch_add_if_larger(rr + kSketchRegs, t.y);
    }
}

// One warp per column: (sum of 2^-register, zero registers).
static __global__ void k_rel_sketch_sum(const uint32_t* __restrict__ regs, uint32_t ncol, double2* out) {
    const uint32_t col = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32, lane = threadIdx.x & 31;
    if (col >= ncol) return;
    const uint32_t* r = regs + (uint64_t)col * kSketchRegs;
    double sum = 0;
    uint32_t zeros = 0;
    for (uint32_t k = lane; k < kSketchRegs; k += 32) {
        const uint32_t v = r[k];
        sum += ldexp(1.0, -(int)v);
        zeros += v == 0;
    }
    for (int o = 16; o; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        zeros += __shfl_xor_sync(0xffffffffu, zeros, o);
    }
    if (lane == 0) out[col] = make_double2(sum, (double)zeros);
}

// One CTA: per-relation id bases, z tiling and (y, tile) key ranges.
static __global__ void __launch_bounds__(1024) k_ix_layout(RelPools P, uint32_t tile_lg) {
    __shared__ uint64_t sm[1024 / 32 + 1];
    uint64_t cf = 0, cy = 0, ck = 0;
    for (uint32_t b = 0; b < P.nrel; b += 1024) {
        const uint32_t r = b + threadIdx.x;
        uint64_t nf = 0, ny = 0, T = 1, keys = 0;
        if (r < P.nrel) {
            nf = P.nf_cnt[r];
            ny = P.ny_cnt[r];
            T = nf > (1ull << tile_lg) ? (nf + (1ull << tile_lg) - 1) >> tile_lg : 1;
            keys = ny * T + T;  // T sentinel keys: y id ny has no tuples
        }
        uint64_t tf, ty, tk;
        const uint64_t ef = block_excl_scan<1024>(nf, sm, &tf);
        const uint64_t ey = block_excl_scan<1024>(ny, sm, &ty);
        const uint64_t ek = block_excl_scan<1024>(keys, sm, &tk);
        if (r < P.nrel) {
            RelDev d;
            d.nt = P.in[r].n;
            d.tup_off = P.tup_off[r];
            d.tab_off = P.tab_off[r];
            d.tab_cap = P.tab_off[r + 1] - P.tab_off[r];
            d.nf = nf;
            d.ny = ny;
            d.fbase = cf + ef;
            d.ybase = cy + ey;
            d.yt_base = ck + ek;
            d.T = (uint32_t)T;
            d.tile_shift = T > 1 ? tile_lg : 31;
            d.tile_width = T > 1 ? (1u << tile_lg) : (uint32_t)(nf > 0 ? nf : 1);
            d.probe_lim = P.probe_lim;
            P.rel[r] = d;
            P.yoff[r] = d.ybase;
            // a relation without the by-first-value CSR still takes its
            // tuples' positions in that CSR's global prefix (at its first
            // id, in one add), so every relation's positions stay
            // [tup_off, tup_off + nt) for the ones that have it
            if (!(P.roles[r] & kRoleRows) && d.nt) atomicAdd(&P.degF[d.fbase], (uint32_t)d.nt);
        }
        cf += tf;
        cy += ty;
        ck += tk;
    }
    if (threadIdx.x == 0) {
        P.yoff[P.nrel] = cy;
        *P.f_need = cf + 1;
        *P.yt_need = ck + 1;
        if (ck + 1 > P.yt_cap) raise_error(P.err, kErrTableFull);
        // a sketch-sized table overflowed its probe bound: some ids are
        // missing, so no later kernel may use the tables (the host rebuilds
        // with tuple-sized tables)
        if (*(volatile uint32_t*)P.err & kErrProbeLimit) *P.yt_need = ~0ull;
    }
}

// Tuples -> (global f id, global y id); degree of f; count of (y, f tile).
static __global__ void k_ix_map(RelPools P) {
    if (*P.yt_need > P.yt_cap) return;  // layout overflow: the host regrows
    SegCursor sc{P.tup_off, P.nrel};
    DIM3G_FOR_CHUNK(i, P.ntot) {
        const uint32_t r = sc.at(i);
        const RelDev& d = P.rel[r];
        const uint2 t = P.in[r].pairs[i - sc.lo];
        const uint32_t fid = table_find(rel_table(P.TF, d), t.x);
        const uint32_t yid = table_find(rel_table(P.TY, d), t.y);
        P.Pm[i] = make_uint2(fid, yid);
        const uint8_t ro = P.roles[r];
        if (ro & kRoleRows) atomicAdd(&P.degF[fid], 1u);
        if (ro & kRoleCols) {
            const uint64_t key = d.yt_base + (uint64_t)(yid - d.ybase) * d.T + ((fid - d.fbase) >> d.tile_shift);
            atomic_inc_agg(P.cnt_yt, key);  // heavy y keys repeat within a warp
        }
    }
}

static __global__ void k_ix_scatter(RelPools P) {
    if (*P.yt_need > P.yt_cap) return;
    SegCursor sc{P.tup_off, P.nrel};
    DIM3G_FOR_CHUNK(i, P.ntot) {
        const uint32_t r = sc.at(i);
        const RelDev& d = P.rel[r];
        const uint2 pm = P.Pm[i];
        const uint8_t ro = P.roles[r];
        const uint32_t fl = pm.x - (uint32_t)d.fbase;
        if (ro & kRoleRows) {
            const uint32_t pos = atomicAdd(&P.curF[pm.x], 1u);
            P.ICf[pos] = pm.y;
            P.ICr[pos] = fl;
        }
        if (ro & kRoleCols) {
            const uint64_t key = d.yt_base + (uint64_t)(pm.y - d.ybase) * d.T + (fl >> d.tile_shift);
            const uint32_t p2 = atomic_inc_agg(P.curY, key);
            P.ICy[p2] = fl;
            P.VSy[p2] = P.in[r].pairs[i - sc.lo].x;
        }
    }
}

// Exact join size of every ordered relation pair (r, s):
// outj[r * nrel + s] = sum over y of deg_r(y) * deg_s(y).  One thread per y
// of the set (global y ids), probing every relation's y table.
static __global__ void k_pair_outj(RelPools P, unsigned long long* outj) {
    if (*P.yt_need > P.yt_cap) return;
    const uint64_t ny_all = P.yoff[P.nrel];
    SegCursor sc{P.yoff, P.nrel};
    DIM3G_FOR_CHUNK(g, ny_all) {
        const uint32_t r = sc.at(g);
        const RelDev& d = P.rel[r];
        const uint32_t* jr = P.JRy + d.yt_base + (g - sc.lo) * d.T;
        const unsigned long long deg_r = jr[d.T] - jr[0];
        const uint32_t v = P.id2y[g];
        for (uint32_t s = 0; s < P.nrel; s++) {
            const RelDev& e = P.rel[s];
            const uint32_t t = table_find(rel_table(P.TY, e), v);
            if (t == kNotFound) continue;
            const uint32_t* js = P.JRy + e.yt_base + (uint64_t)(t - e.ybase) * e.T;
            const uint64_t key = (uint64_t)r * P.nrel + s;
            atomic_add_grouped(&outj[key], key, deg_r * (js[e.T] - js[0]));
        }
    }
}

// --------------------------------------------------------------- query set
enum QueryOp : uint32_t { kOpProject = 0, kOpCount = 1 };

struct QueryIn {
    uint32_t p, q;        // relation ids: P drives the rows, Q is probed
    uint32_t op;          // QueryOp
    uint32_t pad;
    uint2* out;           // (P.f, Q.f) pairs
    unsigned long long* out_cnt;  // counts (kOpCount)
    uint64_t cap;         // pairs the output holds
};

// Per-query results, copied back after the batch.
struct QueryRes {
    unsigned long long n_out;   // pairs written (or needed when > cap)
    unsigned long long out_j;   // candidates
    uint32_t err;
    uint32_t nx, ny, nz;        // rows (distinct P.f; 0 when a side is empty), P.y, Q.f
};

struct QueryPools {
    const RelDev* rel;
    const QueryIn* qin;
    uint32_t nq;
    const uint64_t* qt_off;    // nq + 1: prefix of P tuple counts (y map, P entries)
    const uint64_t* qrow_off;  // nq + 1: prefix of P tuple counts + 1 (rows)
    uint64_t ntot, nrows;
    const unsigned long long* TY;
    const uint32_t* id2f;
    const uint32_t* id2y;
    const uint32_t* JRf;
    const uint32_t* ICf;
    const uint32_t* ICr;
    const uint32_t* JRy;
    const uint32_t* ICy;
    const uint32_t* VSy;
    uint32_t* ymap;   // ntot
    uint32_t* ICq;    // ntot: P entries as Q y ids
    uint32_t* JRq;    // nrows: P row pointers, relative
    uint32_t* ucap;   // nrows
    uint8_t* cls;     // nrows
    unsigned long long* wrow;  // nrows: candidates per row
    RowCtx* rc;       // nq
    Reserve* rs;      // nq
    QueryRes* res;    // nq
    const unsigned long long* yt_need;  // the relation set's key-space check
    uint64_t yt_cap;
    uint32_t cta_rr;  // the context's CTA-row walk (RowCtx::cta_rr)
};

// False when the relation set's (y, f tile) key space outgrew its pool: its
// CSR was not built, and the query kernels must not read it.
__device__ __forceinline__ bool layout_ok(const QueryPools& Q) { return *Q.yt_need <= Q.yt_cap; }

// y map: y id of P -> y id of Q, or Q's sentinel y id (no tuples).
static __global__ void k_q_ymap(QueryPools Q) {
    if (!layout_ok(Q)) return;
    SegCursor sc{Q.qt_off, Q.nq};
    DIM3G_FOR_CHUNK(i, Q.ntot) {
        const uint32_t qi = sc.at(i);
        const QueryIn qn = Q.qin[qi];
        const RelDev& p = Q.rel[qn.p];
        const RelDev& q = Q.rel[qn.q];
        const uint64_t y = i - sc.lo;
        if (y >= p.ny) continue;
        const uint32_t g = table_find(rel_table((unsigned long long*)Q.TY, q), Q.id2y[p.ybase + y]);
        Q.ymap[i] = g == kNotFound ? (uint32_t)q.ny : g - (uint32_t)q.ybase;
    }
}

// P's CSR entries as Q y ids.
static __global__ void k_q_entries(QueryPools Q) {
    if (!layout_ok(Q)) return;
    SegCursor sc{Q.qt_off, Q.nq};
    DIM3G_FOR_CHUNK(i, Q.ntot) {
        const uint32_t qi = sc.at(i);
        const RelDev& p = Q.rel[Q.qin[qi].p];
        const uint64_t e = i - sc.lo;
        const uint32_t yg = Q.ICf[p.tup_off + e];
        const uint32_t yq = Q.ymap[sc.lo + (yg - p.ybase)];
        Q.ICq[i] = yq;
        // candidates of the entry: its S segment over all z tiles
        const RelDev& q = Q.rel[Q.qin[qi].q];
        const uint32_t* jr = Q.JRy + q.yt_base + (uint64_t)yq * q.T;
        const uint32_t len = jr[q.T] - jr[0];
        // entries of one row are contiguous: one atomic per run of a row
        const uint64_t g = Q.qrow_off[qi] + Q.ICr[p.tup_off + e];
        atomic_add_grouped(&Q.wrow[g], g, len);
    }
}

// P's row pointers relative to P's first entry.
static __global__ void k_q_rows(QueryPools Q) {
    if (!layout_ok(Q)) return;
    SegCursor sc{Q.qrow_off, Q.nq};
    DIM3G_FOR_CHUNK(i, Q.nrows) {
        const uint32_t qi = sc.at(i);
        const RelDev& p = Q.rel[Q.qin[qi].p];
        const uint64_t x = i - sc.lo;
        if (x <= Q.res[qi].nx) Q.JRq[i] = Q.JRf[p.fbase + x] - (uint32_t)p.tup_off;
    }
}

// One thread per query: its row context and output reservation.
static __global__ void k_q_setup(QueryPools Q) {
    const uint32_t qi = blockIdx.x * blockDim.x + threadIdx.x;
    if (qi >= Q.nq) return;
    const QueryIn qn = Q.qin[qi];
    const RelDev& p = Q.rel[qn.p];
    const RelDev& q = Q.rel[qn.q];
    RowCtx c{};
    c.JR_R = Q.JRq + Q.qrow_off[qi];
    c.IC_R = Q.ICq + Q.qt_off[qi];
    c.JR_S = Q.JRy + q.yt_base;
    c.IC_S = Q.ICy;
    c.VS = Q.VSy;
    c.T = q.T;
    c.tile_width = q.tile_width;
    c.m = (uint32_t)q.nf;
    c.cta_rr = Q.cta_rr;
    c.ucap = Q.ucap + Q.qrow_off[qi];
    c.cnt = nullptr;
    c.off = nullptr;
    c.id2x = Q.id2f + p.fbase;
    c.id2z = Q.id2f + q.fbase;
    c.out = qn.out;
    c.err = &Q.res[qi].err;
    c.next_row = nullptr;
    Q.rc[qi] = c;
    Q.rs[qi] = Reserve{&Q.res[qi].n_out, qn.cap};
    QueryRes r{};
    const bool ok = layout_ok(Q);
    const bool live = ok && Q.qt_off[qi + 1] > Q.qt_off[qi];  // both sides nonempty
    r.nx = live ? (uint32_t)p.nf : 0u;
    r.err = ok ? 0u : (uint32_t)kErrTableFull;
    r.ny = (uint32_t)p.ny;
    r.nz = (uint32_t)q.nf;
    Q.res[qi] = r;
}

// Per-row class (1..5 project, 9..13 COUNT) from the candidates counted per
// row by k_q_entries; one thread per row of the row space.
static __global__ void k_q_row_work(QueryPools Q, uint32_t cap_w, uint32_t cap_b) {
    if (!layout_ok(Q)) return;
    SegCursor sc{Q.qrow_off, Q.nq};
    DIM3G_FOR_CHUNK(g, Q.nrows) {
        const uint32_t qi = sc.at(g);
        const uint64_t x = g - sc.lo;
        if (x >= Q.res[qi].nx) continue;
        const unsigned long long w = Q.wrow[g];
        const uint32_t m = Q.res[qi].nz;
        const uint32_t u = (uint32_t)(w < m ? w : m);
        Q.ucap[g] = u;
        uint32_t k = row_class(w, u, cap_w, cap_b, true);
        if (k && Q.qin[qi].op == kOpCount) {
            k += 8;
            if (w >= 0xFFFFFFFFull) raise_error(&Q.res[qi].err, kErrCountRange);
        }
        Q.cls[g] = (uint8_t)k;
        atomic_add_grouped(&Q.res[qi].out_j, qi, w);  // one atomic per query run
    }
}

// ---- class lists in one partition of the row space (instead of one
// prefix sum per class).  A row's bucket: 0 warp class (k0+1); 1..3 CTA
// class (k0+2), by distinct bound u <= capS, u <= capM, larger when split
// (else all 1); 4 huge bitmap rows (k0+4); 5 bitmap rows (k0+3); 6 tiny
// rows (k0+5); 7 none.  Three launches: per-tile bucket counts, their
// prefix per bucket (one CTA), the scatter into the lists.  Order within a
// list is unspecified (rows are claimed dynamically anyway).
constexpr uint32_t kPartItems = 16;
constexpr uint32_t kPartTile = 256 * kPartItems;  // rows a CTA tile
constexpr uint32_t kPartBuckets = 7;
struct PartSpec {
    uint32_t k0, split, capS, capM;
};
__device__ __forceinline__ uint32_t row_bucket(const uint8_t* __restrict__ cls, const uint32_t* __restrict__ ucap,
                                               uint64_t i, const PartSpec& ps) {
    const uint32_t c = cls[i];
    if (c == ps.k0 + 1u) return 0;
    if (c == ps.k0 + 2u) {
        if (!ps.split) return 1;
        const uint32_t u = ucap[i];
        return u <= ps.capS ? 1u : (u <= ps.capM ? 2u : 3u);
    }
    if (c == ps.k0 + 4u) return 4;
    if (c == ps.k0 + 3u) return 5;
    if (c == ps.k0 + 5u) return 6;
    return 7;
}

// hist[tile * 8 + b] = rows of bucket b in the tile.
static __global__ void __launch_bounds__(256) k_part_count(const uint8_t* __restrict__ cls,
                                                           const uint32_t* __restrict__ ucap, uint64_t n, PartSpec ps,
                                                           uint32_t* __restrict__ hist) {
    __shared__ uint32_t s[8];
    if (threadIdx.x < 8) s[threadIdx.x] = 0;
    __syncthreads();
    const uint64_t base = (uint64_t)blockIdx.x * kPartTile;
    uint32_t c[kPartBuckets];
#pragma unroll
    for (uint32_t b = 0; b < kPartBuckets; b++) c[b] = 0;
#pragma unroll 4
    for (uint32_t k = 0; k < kPartItems; k++) {
        const uint64_t i = base + (uint64_t)k * 256 + threadIdx.x;
        const uint32_t b = i < n ? row_bucket(cls, ucap, i, ps) : 7u;
#pragma unroll
        for (uint32_t q = 0; q < kPartBuckets; q++) c[q] += b == q ? 1u : 0u;
    }
#pragma unroll
    for (uint32_t q = 0; q < kPartBuckets; q++) {
        const uint32_t v = warp_sum(c[q]);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(&s[q], v);
    }
    __syncthreads();
    if (threadIdx.x < kPartBuckets) hist[(uint64_t)blockIdx.x * 8 + threadIdx.x] = s[threadIdx.x];
}

// One CTA: hist becomes each tile's first position in its bucket; the
// bucket totals go to the class counts (n[1..5] as the class prefix sums
// gave them; nb[0..2] the split CTA class), base[b] = where bucket b starts
// in its list.
static __global__ void __launch_bounds__(1024) k_part_offsets(uint32_t* __restrict__ hist, uint32_t ntiles,
                                                              unsigned long long* n, unsigned long long* nb,
                                                              unsigned long long* base) {
    __shared__ uint64_t sm[1024 / 32 + 1];
    __shared__ unsigned long long tot[8];
    for (uint32_t b = 0; b < kPartBuckets; b++) {
        uint64_t carry = 0;
        for (uint32_t t0 = 0; t0 < ntiles; t0 += 1024) {
            const uint32_t t = t0 + threadIdx.x;
            const uint64_t v = t < ntiles ? hist[(uint64_t)t * 8 + b] : 0u;
            uint64_t sum;
            const uint64_t e = block_excl_scan<1024>(v, sm, &sum);
            if (t < ntiles) hist[(uint64_t)t * 8 + b] = (uint32_t)(carry + e);
            carry += sum;
        }
        if (threadIdx.x == 0) tot[b] = carry;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        n[1] = tot[0];
        n[2] = tot[1] + tot[2] + tot[3];
        if (nb) {
            nb[0] = tot[1];
            nb[1] = tot[2];
            nb[2] = tot[3];
        }
        n[4] = tot[4];
        n[3] = tot[5];
        n[5] = tot[6];
        base[0] = 0;
        base[1] = 0;
        base[2] = tot[1];
        base[3] = tot[1] + tot[2];
        base[4] = 0;
        base[5] = tot[4];
        base[6] = 0;
    }
}

// Each row of a bucket to list[base[b] + its tile's offset + its rank in the
// tile] (one shared atomic per group of lanes with the same bucket).
static __global__ void __launch_bounds__(256) k_part_scatter(const uint8_t* __restrict__ cls,
                                                             const uint32_t* __restrict__ ucap, uint64_t n,
                                                             PartSpec ps, const uint32_t* __restrict__ off,
                                                             const unsigned long long* __restrict__ base,
                                                             uint32_t* lw, uint32_t* lb, uint32_t* lm,
                                                             uint32_t* lt) {
    __shared__ uint32_t s[8];
    __shared__ unsigned long long s_at[8];
    if (threadIdx.x < kPartBuckets) {
        s[threadIdx.x] = 0;
        s_at[threadIdx.x] = base[threadIdx.x] + off[(uint64_t)blockIdx.x * 8 + threadIdx.x];
    }
    __syncthreads();
    const uint64_t t0 = (uint64_t)blockIdx.x * kPartTile;
    const uint32_t lane = lane_id();
    for (uint32_t k = 0; k < kPartItems; k++) {
        const uint64_t i = t0 + (uint64_t)k * 256 + threadIdx.x;
        const uint32_t b = i < n ? row_bucket(cls, ucap, i, ps) : 7u;
        const unsigned grp = __match_any_sync(0xffffffffu, b);
        const int leader = __ffs(grp) - 1;
        uint32_t r0 = 0;
        if ((int)lane == leader && b < kPartBuckets) r0 = atomicAdd(&s[b], (uint32_t)__popc(grp));
        r0 = __shfl_sync(0xffffffffu, r0, leader);
        if (b < kPartBuckets) {
            const unsigned long long pos = s_at[b] + r0 + __popc(grp & lanemask_lt());
            uint32_t* list = b == 0 ? lw : (b <= 3 ? lb : (b <= 5 ? lm : lt));
            list[pos] = (uint32_t)i;
        }
    }
}

// Row g of the row space -> (query, local row).
__device__ __forceinline__ uint32_t query_of_row(const QueryPools& Q, uint32_t g, uint32_t* x) {
    const uint32_t qi = seg_find(Q.qrow_off, Q.nq, g);
    *x = g - (uint32_t)Q.qrow_off[qi];
    return qi;
}

struct BatchRows {
    const uint32_t* list;
    const unsigned long long* n_a;  // rows of the list (or its first part)
    const unsigned long long* n_b;  // second part (or nullptr)
    uint32_t* next;                 // dynamic row counter of CTA classes
    const unsigned long long* skip0 = nullptr;  // the rows start past these counts (device; null: 0)
    const unsigned long long* skip1 = nullptr;
    __device__ __forceinline__ const uint32_t* rows() const {
        return list + (skip0 ? *skip0 : 0ull) + (skip1 ? *skip1 : 0ull);
    }
};

// ---- project, single pass: rows of many queries, each CTA (or warp) copying
// its row's query context into shared memory; the row bodies of single.cuh.
static __global__ void __launch_bounds__(1024) k_b_single_bitmap(QueryPools Q, BatchRows L, uint32_t bitmap_words) {
    extern __shared__ uint32_t bm[];
    __shared__ uint32_t s_row, s_x, s_q;
    __shared__ RowCtx s_c;
    __shared__ CtaChunks s_cc;
    if (threadIdx.x == 0) s_cc.n = 0;
    uint32_t* stage = bm + bitmap_words + (threadIdx.x >> 5) * kStage;
    const uint32_t nrows = (uint32_t)(*L.n_a + *L.n_b);
    for (uint32_t ri = cta_next_row(L.next, &s_row); ri < nrows; ri = cta_next_row(L.next, &s_row)) {
        if (threadIdx.x == 0) {
            uint32_t x;
            s_q = query_of_row(Q, L.list[ri], &x);
            s_x = x;
            s_c = Q.rc[s_q];
        }
        __syncthreads();
        StageSink sink{stage, s_c.out, Q.rs[s_q], s_c.id2x[s_x]};
        single_bitmap_row(s_c, s_x, bm, sink, &s_cc);
        sink.flush();
    }
}

static __global__ void __launch_bounds__(1024) k_b_single_block(QueryPools Q, BatchRows L, uint32_t block_lg) {
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t s_row, s_x, s_q;
    __shared__ RowCtx s_c;
    __shared__ CtaChunks s_cc;
    if (threadIdx.x == 0) s_cc.n = 0;
    uint32_t* stage = smem + (1u << block_lg) + (threadIdx.x >> 5) * kStage;
    const uint32_t nrows = (uint32_t)*L.n_a;
    const uint32_t* rows = L.rows();
    for (uint32_t ri = cta_next_row(L.next, &s_row); ri < nrows; ri = cta_next_row(L.next, &s_row)) {
        if (threadIdx.x == 0) {
            uint32_t x;
            s_q = query_of_row(Q, rows[ri], &x);
            s_x = x;
            s_c = Q.rc[s_q];
        }
        __syncthreads();
        StageSink sink{stage, s_c.out, Q.rs[s_q], s_c.id2x[s_x]};
        single_block_row(s_c, s_x, smem, sink, block_lg, &s_cc);
        sink.flush();
    }
}

// Warp class: at most 8 warps per CTA, one context slot each.
static __global__ void __launch_bounds__(256) k_b_single_warp(QueryPools Q, BatchRows L, uint32_t warp_lg,
                                                              uint32_t stage) {
    extern __shared__ uint32_t smem[];
    __shared__ RowCtx s_c[8];
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = lane_id();
    uint32_t* tab = smem + (size_t)wib * warp_row_words(warp_lg, stage);
    // the warp's pairs are staged across its rows and flushed when the
    // query (cursor and output) changes
    PairStageSink sink{reinterpret_cast<uint2*>(tab + (1u << warp_lg)), nullptr, Reserve{nullptr, 0}, 0, stage};
    uint32_t cur_q = 0xFFFFFFFFu, q_lo = 1, q_hi = 0;
    const uint32_t nrows = (uint32_t)*L.n_a;
    for (uint32_t ri = blockIdx.x * nw + wib; ri < nrows; ri += gridDim.x * nw) {
        // rows of one query are contiguous in the list: look the query up
        // only when the row leaves the current query's row range
        const uint32_t g = L.list[ri];
        uint32_t qi = cur_q;
        if (g < q_lo || g >= q_hi) {
            qi = seg_find(Q.qrow_off, Q.nq, g);
            q_lo = (uint32_t)Q.qrow_off[qi];
            q_hi = (uint32_t)Q.qrow_off[qi + 1];
        }
        const uint32_t x = g - q_lo;
        if (qi != cur_q) {
            sink.flush();
            __syncwarp();
            if (lane == 0) s_c[wib] = Q.rc[qi];
            __syncwarp();
            sink.rs = Q.rs[qi];
            sink.out = s_c[wib].out;
            cur_q = qi;
        }
        single_warp_row(s_c[wib], x, tab, sink, warp_lg);
    }
    sink.flush();
}

// ---- COUNT, single pass: rows reserve output ranges from their query's
// cursor, one atomic per 32 emitted groups.
__device__ __forceinline__ void emit_groups(const RowCtx& c, const Reserve& rs, unsigned long long* out_cnt,
                                            bool have, uint32_t xv, uint32_t zv, uint32_t cnt) {
    const uint32_t b = __ballot_sync(0xffffffffu, have);
    if (!b) return;
    unsigned long long base = 0;
    if (lane_id() == 0) base = atomicAdd(rs.cursor, (unsigned long long)__popc(b));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (have) {
        const unsigned long long pos = base + __popc(b & lanemask_lt());
        if (pos < rs.cap) {
            c.out[pos] = make_uint2(xv, zv);
            out_cnt[pos] = cnt;
        }
    }
}

// (x, z, count) groups staged across the rows of one warp and one query,
// reserved once per kStage groups (see PairStageSink).
struct GroupStage {
    uint2* pairs;      // cap (x value, z value)
    uint32_t* counts;  // cap counts
    uint2* out;
    unsigned long long* out_cnt;
    Reserve rs;
    uint32_t cap;      // at least 32
    uint32_t n = 0;
    __device__ __forceinline__ void flush() {
        if (n == 0) return;
        unsigned long long base = 0;
        if (lane_id() == 0) base = atomicAdd(rs.cursor, (unsigned long long)n);
        base = __shfl_sync(0xffffffffu, base, 0);
        __syncwarp();
        if (base + n <= rs.cap)
            for (uint32_t i = lane_id(); i < n; i += 32) {
                out[base + i] = pairs[i];
                out_cnt[base + i] = counts[i];
            }
        __syncwarp();
        n = 0;
    }
    // warp-collective: the lanes with `have` add one group each
    __device__ __forceinline__ void add(bool have, uint32_t xv, uint32_t zv, uint32_t cnt) {
        const uint32_t b = __ballot_sync(0xffffffffu, have);
        if (!b) return;
        if (n + __popc(b) > cap) flush();
        if (have) {
            const uint32_t pos = n + __popc(b & lanemask_lt());
            pairs[pos] = make_uint2(xv, zv);
            counts[pos] = cnt;
        }
        n += __popc(b);
        __syncwarp();
    }
};

// Per-warp shared memory of the COUNT warp classes: 2^(warp_lg+1) map
// words, then `stage` staged groups (3 words each).
__host__ __device__ constexpr size_t agg_warp_words(uint32_t warp_lg, uint32_t stage) {
    return ((size_t)2 << warp_lg) + 3 * (size_t)stage;
}

static __global__ void __launch_bounds__(256) k_b_agg_warp(QueryPools Q, BatchRows L, uint32_t warp_lg,
                                                           uint32_t stage) {
    extern __shared__ uint32_t smem[];
    __shared__ RowCtx s_c[8];
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = lane_id();
    uint32_t* keys = smem + (size_t)wib * agg_warp_words(warp_lg, stage);
    uint32_t* vals = keys + (1u << warp_lg);
    GroupStage gs{reinterpret_cast<uint2*>(keys + (2u << warp_lg)), keys + (2u << warp_lg) + 2 * stage, nullptr,
                  nullptr, Reserve{nullptr, 0}, stage};
    uint32_t cur_q = 0xFFFFFFFFu, q_lo = 1, q_hi = 0;
    const uint32_t nrows = (uint32_t)*L.n_a;
    for (uint32_t ri = blockIdx.x * nw + wib; ri < nrows; ri += gridDim.x * nw) {
        // rows of one query are contiguous in the list: look the query up
        // only when the row leaves the current query's row range
        const uint32_t g = L.list[ri];
        uint32_t qi = cur_q;
        if (g < q_lo || g >= q_hi) {
            qi = seg_find(Q.qrow_off, Q.nq, g);
            q_lo = (uint32_t)Q.qrow_off[qi];
            q_hi = (uint32_t)Q.qrow_off[qi + 1];
        }
        const uint32_t x = g - q_lo;
        if (qi != cur_q) {
            gs.flush();
            __syncwarp();
            if (lane == 0) s_c[wib] = Q.rc[qi];
            __syncwarp();
            gs.rs = Q.rs[qi];
            gs.out = s_c[wib].out;
            gs.out_cnt = Q.qin[qi].out_cnt;
            cur_q = qi;
        }
        const RowCtx& c = s_c[wib];
        const uint32_t u = c.ucap[x];
        const uint32_t xv = c.id2x[x];
        NullSink sink;
        if (use_row_counters(c.m, u, warp_lg + 1)) {
            for (uint32_t s = lane; s < c.m; s += 32) keys[s] = 0;
            __syncwarp();
            CountTile set{keys, 0};
            warp_expand(c, c.JR_R[x], c.JR_R[x + 1], 0, 0, 0, c.T, set, sink);
            __syncwarp();
            for (uint32_t sb = 0; sb < c.m; sb += 32) {
                const uint32_t z = sb + lane;
                const uint32_t v = z < c.m ? keys[z] : 0u;
                gs.add(v != 0, xv, v ? __ldg(&c.id2z[z]) : 0u, v);
            }
            __syncwarp();
            continue;
        }
        uint32_t lg = ceil_log2(2 * u);
        lg = lg < 5 ? 5 : (lg > warp_lg ? warp_lg : lg);
        for (uint32_t s = lane; s < (1u << lg); s += 32) {
            keys[s] = kEmpty32;
            vals[s] = 0;
        }
        __syncwarp();
        CountMap set{keys, vals, lg, c.err};
        warp_expand(c, c.JR_R[x], c.JR_R[x + 1], 0, 0, 0, c.T, set, sink);
        __syncwarp();
        for (uint32_t sb = 0; sb < (1u << lg); sb += 32) {
            const uint32_t key = keys[sb + lane];
            const bool have = key != kEmpty32;
            gs.add(have, xv, have ? __ldg(&c.id2z[key]) : 0u, have ? vals[sb + lane] : 0u);
        }
        __syncwarp();
    }
    gs.flush();
}

static __global__ void __launch_bounds__(256) k_b_agg_block(QueryPools Q, BatchRows L, uint32_t block_lg) {
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t s_row, s_x, s_q;
    __shared__ RowCtx s_c;
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = lane_id();
    const uint32_t nw_lg = 31 - __clz(nw);
    uint32_t* keys = smem;
    uint32_t* vals = smem + (1u << block_lg);
    const uint32_t nrows = (uint32_t)*L.n_a;
    for (uint32_t ri = cta_next_row(L.next, &s_row); ri < nrows; ri = cta_next_row(L.next, &s_row)) {
        if (threadIdx.x == 0) {
            uint32_t x;
            s_q = query_of_row(Q, L.list[ri], &x);
            s_x = x;
            s_c = Q.rc[s_q];
        }
        __syncthreads();
        const RowCtx& c = s_c;
        const uint32_t x = s_x;
        const uint32_t u = c.ucap[x];
        const bool direct = use_row_counters(c.m, u, block_lg + 1);
        uint32_t lg = ceil_log2(2 * u);
        lg = lg < 5 ? 5 : (lg > block_lg ? block_lg : lg);
        if (direct) {
            for (uint32_t s = threadIdx.x; s < c.m; s += blockDim.x) keys[s] = 0;
        } else {
            for (uint32_t s = threadIdx.x; s < (1u << lg); s += blockDim.x) {
                keys[s] = kEmpty32;
                vals[s] = 0;
            }
        }
        __syncthreads();
        NullSink sink;
        if (direct) {
            CountTile set{keys, 0};
            warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, 0, c.T, set, sink);
        } else {
            CountMap set{keys, vals, lg, c.err};
            warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, 0, c.T, set, sink);
        }
        __syncthreads();
        const Reserve rs = Q.rs[s_q];
        const uint32_t xv = c.id2x[x];
        unsigned long long* oc = Q.qin[s_q].out_cnt;
        const uint32_t span = direct ? c.m : (1u << lg);
        for (uint32_t sb = wib * 32; sb < span; sb += nw * 32) {
            const uint32_t s = sb + lane;
            uint32_t zid = kEmpty32, v = 0;
            if (s < span) {
                if (direct) {
                    v = keys[s];
                    zid = v ? s : kEmpty32;
                } else {
                    zid = keys[s];
                    v = vals[s];
                }
            }
            const bool have = zid != kEmpty32;
            emit_groups(c, rs, oc, have, xv, have ? __ldg(&c.id2z[zid]) : 0u, have ? v : 0u);
        }
    }
}

// Classes 3/4 of COUNT: one CTA per row with a private counter array over
// one z tile in global memory (L2-resident), plus a list of the z touched
// in the tile, so emission and reset cost O(distinct z).
struct TouchCountTile {
    uint32_t* ctr;
    uint32_t* touched;
    uint32_t* n_touched;  // shared
    uint32_t lo;
    __device__ __forceinline__ bool insert(uint32_t z, bool act) {
        if (act) {
            const uint32_t zl = z - lo;
            if (atomicAdd(&ctr[zl], 1u) == 0) touched[atomicAdd(n_touched, 1u)] = zl;
        }
        return false;
    }
};

static __global__ void __launch_bounds__(512) k_b_agg_tile(QueryPools Q, BatchRows L, uint32_t* scratch, uint32_t tile_cap) {
    __shared__ uint32_t s_row, s_x, s_q, s_nt;
    __shared__ RowCtx s_c;
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = lane_id();
    const uint32_t nw_lg = 31 - __clz(nw);
    uint32_t* ctr = scratch + (size_t)blockIdx.x * 2 * tile_cap;
    uint32_t* touched = ctr + tile_cap;
    const uint32_t nrows = (uint32_t)(*L.n_a + *L.n_b);
    for (uint32_t ri = cta_next_row(L.next, &s_row); ri < nrows; ri = cta_next_row(L.next, &s_row)) {
        if (threadIdx.x == 0) {
            uint32_t x;
            s_q = query_of_row(Q, L.list[ri], &x);
            s_x = x;
            s_c = Q.rc[s_q];
        }
        __syncthreads();
        const RowCtx& c = s_c;
        const uint32_t x = s_x;
        const Reserve rs = Q.rs[s_q];
        const uint32_t xv = c.id2x[x];
        unsigned long long* oc = Q.qin[s_q].out_cnt;
        for (uint32_t t = 0; t < c.T; t++) {
            const uint32_t lo = t * c.tile_width;
            if (threadIdx.x == 0) s_nt = 0;
            __syncthreads();
            TouchCountTile set{ctr, touched, &s_nt, lo};
            NullSink sink;
            warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, t, t + 1, set, sink);
            __threadfence_block();
            __syncthreads();
            const uint32_t nt = s_nt;
            for (uint32_t jb = wib * 32; jb < nt; jb += nw * 32) {
                const uint32_t j = jb + lane;
                const bool have = j < nt;
                uint32_t zl = 0, v = 0;
                if (have) {
                    zl = __ldcg(&touched[j]);
                    v = __ldcg(&ctr[zl]);
                    ctr[zl] = 0;
                }
                emit_groups(c, rs, oc, have, xv, have ? __ldg(&c.id2z[lo + zl]) : 0u, v);
            }
            __syncthreads();
        }
    }
}

}  // namespace dim3g

// batch.cu -- resident relation sets, many-query passes, and batches of
// independent joins run as one CUDA graph, and a serving loop with
// continuous batching over a resident set (host side; kernels in batch.cuh).
//
// Relation set creation: a distinct-key sketch of every relation's columns
// sizes its value -> id tables (k_rel_sketch, synchronised once).
// Relation set build (one stream, no host synchronisation inside):
//   memsets -> k_ix_insert -> k_ix_layout -> id scans (TF, TY) -> k_ix_map
//   -> CSR scans (by f, by (y, f tile); bounded by the layout's counts)
//   -> k_ix_scatter (a batch builds only the CSR each relation's query reads)
// Query pass over queries (P, Q) of a set:
//   k_q_setup -> k_q_ymap -> k_q_entries -> k_q_rows -> k_q_row_work
//   -> class lists (one partition) -> project row kernels -> COUNT row
//   kernels -> per-query results to pinned host memory
// Every size the launches depend on is known on the host from the tuple
// counts; counts that depend on the data (distinct values, rows per class,
// output sizes) stay on the device.  The data-dependent bounds -- the
// (y, f tile) key space and the probe bound of the sketch-sized tables --
// are checked on the device; on overflow the host regrows that pool (or
// falls back to tuple-sized tables) and runs again.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/dim3gpu.h"
#include "batch.cuh"
#include "internal.h"
#include "scan.cuh"

using namespace dim3g;
namespace I = dim3g_internal;

namespace {

#define BCU(call)                                                                                             \
    do {                                                                                                      \
        cudaError_t e_ = (call);                                                                              \
        if (e_ != cudaSuccess) return I::fail(ctx, DIM3G_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)
#define BLAUNCH()                          \
    do {                                   \
        BCU(cudaGetLastError());           \
        launches++;                        \
    } while (0)

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// Offsets of typed arrays inside one device allocation.
struct Layout {
    size_t total = 0;
    template <class T>
    size_t add(uint64_t count) {
        size_t o = total;
        total += align256((size_t)(count ? count : 1) * sizeof(T));
        return o;
    }
};

template <class K>
unsigned resident(K kernel, int block, size_t smem, int sm) {
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, smem) != cudaSuccess || per < 1) {
        cudaGetLastError();
        per = 1;
    }
    return (unsigned)(per * sm);
}
unsigned elem_grid(uint64_t n, int sm) {
    uint64_t b = (n + 255) / 256;
    uint64_t cap = (uint64_t)sm * 8;
    return (unsigned)(b < 1 ? 1 : (b > cap ? cap : b));
}

struct Tuning {
    uint32_t warp_lg, block_lg, block_threads, tile_lg, cta_rr, block_split;
};
Tuning tuning_of(const dim3g_ctx* ctx) {
    int64_t w = 11, b = 14, t = 512, tl = 19, rr = 2, bs = 1;
    dim3g_get_param(ctx, "block_split", &bs);
    dim3g_get_param(ctx, "warp_slots_log2", &w);
    dim3g_get_param(ctx, "block_slots_log2", &b);
    dim3g_get_param(ctx, "block_threads", &t);
    dim3g_get_param(ctx, "tile_bits_log2", &tl);
    dim3g_get_param(ctx, "cta_walk", &rr);
    if (tl > 19) tl = 19;  // the batch bitmap kernel runs 512-thread CTAs
    return Tuning{(uint32_t)w, (uint32_t)b, (uint32_t)t, (uint32_t)tl, (uint32_t)rr, (uint32_t)bs};
}

// Warps per CTA of the warp-class kernels (about half an SM's shared memory).
uint32_t warps_for(size_t per_warp) {
    size_t w = (size_t)112 * 1024 / per_warp;
    return (uint32_t)(w < 1 ? 1 : (w > 8 ? 8 : w));
}

}  // namespace

// ============================================================ relation set
// Device scratch of one query pass (a relation set has one; every lane of a
// server has its own, so passes can run concurrently).
struct QueryScratch {
    char* qmem = nullptr;
    size_t qmem_bytes = 0;
    uint32_t* agg = nullptr;  // COUNT tile counters + touched lists
    size_t agg_bytes = 0;
    QueryRes* h_res = nullptr;  // pinned
    uint32_t h_res_n = 0;
    QueryScratch() = default;
    QueryScratch(const QueryScratch&) = delete;
    QueryScratch& operator=(const QueryScratch&) = delete;
    ~QueryScratch() {
        if (qmem) cudaFree(qmem);
        if (agg) cudaFree(agg);
        if (h_res) cudaFreeHost(h_res);
    }
};

struct dim3g_relset {
    dim3g_ctx* ctx = nullptr;
    uint32_t nrel = 0;
    std::vector<RelIn> h_in;
    std::vector<uint64_t> h_tup_off, h_tab_off;
    std::vector<uint64_t> h_cap;  // sketch-sized table slots per relation (when sized)
    std::vector<uint8_t> h_roles; // CSRs each relation needs (RelRole bits; empty: both for every relation)
    bool sized = false;           // tables from h_cap (else from the tuple counts)
    uint64_t ntot = 0, tabtot = 0, yt_cap = 0;
    uint32_t tile_lg = 19;
    char* mem = nullptr;
    size_t mem_bytes = 0;
    RelPools P{};
    uint64_t* bsum = nullptr;
    uint64_t bsum_n = 0;
    QueryScratch qs;  // scratch of dim3g_relset_join (grow-only)
    unsigned long long* h_need = nullptr;  // pinned: yt keys needed, err
    uint64_t launches_build = 0;

    ~dim3g_relset() {
        if (mem) cudaFree(mem);
        if (h_need) cudaFreeHost(h_need);
    }
};

namespace {

// Host layout of a relation set from its tuple counts.
int relset_plan(dim3g_relset* s, const dim3g_relation* rels, uint32_t n, uint64_t yt_cap) {
    dim3g_ctx* ctx = s->ctx;
    s->nrel = n;
    s->h_in.resize(n);
    s->h_tup_off.assign(n + 1, 0);
    s->h_tab_off.assign(n + 1, 0);
    uint64_t yt_guess = 1;
    for (uint32_t r = 0; r < n; r++) {
        if (!rels[r].d_pairs && rels[r].n) return I::fail(ctx, DIM3G_ERR_INVALID, "relation %u: null pairs", r);
        if ((uintptr_t)rels[r].d_pairs & 7u) return I::fail(ctx, DIM3G_ERR_INVALID, "relation %u: pairs not 8-byte aligned", r);
        s->h_in[r] = RelIn{(const uint2*)rels[r].d_pairs, rels[r].n};
        s->h_tup_off[r + 1] = s->h_tup_off[r] + rels[r].n;
        const uint64_t full = next_pow2(rels[r].n * 2 < 1024 ? 1024 : rels[r].n * 2);
        const uint64_t cap = s->sized && s->h_cap[r] < full ? s->h_cap[r] : full;
        s->h_tab_off[r + 1] = s->h_tab_off[r] + cap;
        yt_guess += 2 * rels[r].n + 2;
    }
    s->ntot = s->h_tup_off[n];
    if (s->ntot >= 0xFFFFFFFFull)
        return I::fail(ctx, DIM3G_ERR_UNSUPPORTED, "a relation set holds fewer than 2^32-1 tuples in total");
    s->tabtot = s->h_tab_off[n];
    s->yt_cap = yt_cap ? yt_cap : yt_guess;

    Layout L;
    const size_t o_in = L.add<RelIn>(n), o_rel = L.add<RelDev>(n), o_tup = L.add<uint64_t>(n + 1),
                 o_tab = L.add<uint64_t>(n + 1), o_TF = L.add<unsigned long long>(s->tabtot),
                 o_TY = L.add<unsigned long long>(s->tabtot), o_nf = L.add<unsigned long long>(n),
                 o_ny = L.add<unsigned long long>(n), o_id2f = L.add<uint32_t>(s->ntot),
                 o_id2y = L.add<uint32_t>(s->ntot), o_Pm = L.add<uint2>(s->ntot), o_deg = L.add<uint32_t>(s->ntot + 1),
                 o_JRf = L.add<uint32_t>(s->ntot + 1), o_curF = L.add<uint32_t>(s->ntot + 1),
                 o_ICf = L.add<uint32_t>(s->ntot), o_ICr = L.add<uint32_t>(s->ntot), o_cyt = L.add<uint32_t>(s->yt_cap),
                 o_JRy = L.add<uint32_t>(s->yt_cap), o_curY = L.add<uint32_t>(s->yt_cap),
                 o_ICy = L.add<uint32_t>(s->ntot), o_VSy = L.add<uint32_t>(s->ntot), o_err = L.add<uint32_t>(4),
                 o_need = L.add<unsigned long long>(2), o_yoff = L.add<uint64_t>(n + 1),
                 o_roles = L.add<uint8_t>(n), o_fneed = L.add<unsigned long long>(1);
    uint64_t sn = scan_storage(s->tabtot);
    const uint64_t s2 = scan_storage(s->ntot + 1), s3 = scan_storage(s->yt_cap);
    if (s2 > sn) sn = s2;
    if (s3 > sn) sn = s3;
    const size_t o_bsum = L.add<uint64_t>(sn);
    if (s->mem && s->mem_bytes < L.total) {
        cudaFree(s->mem);
        s->mem = nullptr;
        s->mem_bytes = 0;
    }
    if (!s->mem) {
        if (cudaMalloc(&s->mem, L.total) != cudaSuccess) {
            cudaGetLastError();
            return I::fail(ctx, DIM3G_ERR_NOMEM, "relation set: device allocation of %zu bytes failed", L.total);
        }
        s->mem_bytes = L.total;
    }
    char* m = s->mem;
    RelPools& P = s->P;
    P.in = (const RelIn*)(m + o_in);
    P.rel = (RelDev*)(m + o_rel);
    P.tup_off = (const uint64_t*)(m + o_tup);
    P.tab_off = (const uint64_t*)(m + o_tab);
    P.nrel = n;
    P.probe_lim = s->sized ? (uint32_t)kSizedProbeLimit : 0u;
    P.ntot = s->ntot;
    P.TF = (unsigned long long*)(m + o_TF);
    P.TY = (unsigned long long*)(m + o_TY);
    P.nf_cnt = (unsigned long long*)(m + o_nf);
    P.ny_cnt = (unsigned long long*)(m + o_ny);
    P.id2f = (uint32_t*)(m + o_id2f);
    P.id2y = (uint32_t*)(m + o_id2y);
    P.Pm = (uint2*)(m + o_Pm);
    P.degF = (uint32_t*)(m + o_deg);
    P.JRf = (uint32_t*)(m + o_JRf);
    P.curF = (uint32_t*)(m + o_curF);
    P.ICf = (uint32_t*)(m + o_ICf);
    P.ICr = (uint32_t*)(m + o_ICr);
    P.cnt_yt = (uint32_t*)(m + o_cyt);
    P.JRy = (uint32_t*)(m + o_JRy);
    P.curY = (uint32_t*)(m + o_curY);
    P.yt_cap = s->yt_cap;
    P.ICy = (uint32_t*)(m + o_ICy);
    P.VSy = (uint32_t*)(m + o_VSy);
    P.err = (uint32_t*)(m + o_err);
    P.yt_need = (unsigned long long*)(m + o_need);
    P.yoff = (uint64_t*)(m + o_yoff);
    P.roles = (const uint8_t*)(m + o_roles);
    P.f_need = (unsigned long long*)(m + o_fneed);
    s->bsum = (uint64_t*)(m + o_bsum);
    s->bsum_n = sn;
    BCU(cudaMemcpy((void*)P.in, s->h_in.data(), n * sizeof(RelIn), cudaMemcpyHostToDevice));
    BCU(cudaMemcpy((void*)P.tup_off, s->h_tup_off.data(), (n + 1) * 8, cudaMemcpyHostToDevice));
    BCU(cudaMemcpy((void*)P.tab_off, s->h_tab_off.data(), (n + 1) * 8, cudaMemcpyHostToDevice));
    if (s->h_roles.size() != n) s->h_roles.assign(n, (uint8_t)(kRoleRows | kRoleCols));
    BCU(cudaMemcpy((void*)P.roles, s->h_roles.data(), n, cudaMemcpyHostToDevice));
    return DIM3G_OK;
}

// Table sizes from a distinct-key sketch of every relation's two columns
// (mapping.cuh): relation r's value -> id tables get s->h_cap[r] slots, about
// table_slack_pct percent of its larger column's distinct keys, instead of
// twice its tuple count.  The tables of a set whose relations repeat keys --
// 1e3..1e6 distinct values over up to 4e6 tuples in a mixed batch -- then
// shrink several times, and with them the build's memsets and id scans.  One
// pass, synchronised, at creation; a build whose tables overflow the probe
// bound (the data changed, or the estimate was low) is redone with
// tuple-sized tables by the caller.
int relset_sketch(dim3g_relset* s, const dim3g_relation* rels, uint32_t n) {
    dim3g_ctx* ctx = s->ctx;
    int64_t on = 1, slack = 150;
    dim3g_get_param(ctx, "sized_tables", &on);
    dim3g_get_param(ctx, "table_slack_pct", &slack);
    s->sized = false;
    s->h_cap.assign(n, 0);
    if (!on || n == 0) return DIM3G_OK;
    std::vector<RelIn> in(n);
    std::vector<uint64_t> off(n + 1, 0);
    for (uint32_t r = 0; r < n; r++) {
        if (!rels[r].d_pairs && rels[r].n) return I::fail(ctx, DIM3G_ERR_INVALID, "relation %u: null pairs", r);
        if ((uintptr_t)rels[r].d_pairs & 7u) return I::fail(ctx, DIM3G_ERR_INVALID, "relation %u: pairs not 8-byte aligned", r);
        in[r] = RelIn{(const uint2*)rels[r].d_pairs, rels[r].n};
        off[r + 1] = off[r] + rels[r].n;
    }
    if (off[n] == 0 || off[n] >= 0xFFFFFFFFull) return DIM3G_OK;  // nothing to size / refused by the plan
    Layout L;
    const size_t o_in = L.add<RelIn>(n), o_off = L.add<uint64_t>(n + 1), o_regs = L.add<uint32_t>((uint64_t)2 * n * kSketchRegs),
                 o_sum = L.add<double2>(2 * (uint64_t)n);
    char* m = nullptr;
    if (cudaMalloc(&m, L.total) != cudaSuccess) {
        cudaGetLastError();
        return DIM3G_OK;  // no room for the sketch: tuple-sized tables
    }
    cudaStream_t st = I::stream(ctx);
    RelPools P{};
    P.in = (const RelIn*)(m + o_in);
    P.tup_off = (const uint64_t*)(m + o_off);
    P.nrel = n;
    P.ntot = off[n];
    uint32_t* regs = (uint32_t*)(m + o_regs);
    double2* sums = (double2*)(m + o_sum);
    std::vector<double2> h(2 * (size_t)n);
    cudaError_t e = cudaMemcpyAsync((void*)P.in, in.data(), n * sizeof(RelIn), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync((void*)P.tup_off, off.data(), (n + 1) * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(regs, 0, (size_t)2 * n * kSketchRegs * 4, st);
    if (e == cudaSuccess) {
        k_rel_sketch<<<elem_grid(P.ntot, I::sm_count(ctx)), 256, 0, st>>>(P, regs);
        k_rel_sketch_sum<<<(2 * n + 7) / 8, 256, 0, st>>>(regs, 2 * n, sums);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data(), sums, h.size() * sizeof(double2), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(m);
    if (e != cudaSuccess) return I::fail(ctx, DIM3G_ERR_CUDA, "relation set sketch: %s", cudaGetErrorString(e));
    I::add_launches(ctx, 2);
    for (uint32_t r = 0; r < n; r++) {
        const double ef = sketch_estimate(h[2 * r].x, (uint32_t)h[2 * r].y);
        const double ey = sketch_estimate(h[2 * r + 1].x, (uint32_t)h[2 * r + 1].y);
        const uint64_t full = next_pow2(rels[r].n * 2 < 1024 ? 1024 : rels[r].n * 2);
        s->h_cap[r] = sketch_capacity(ef > ey ? ef : ey, full, (uint32_t)slack);
        if (s->h_cap[r] < full) s->sized = true;
    }
    return DIM3G_OK;
}

// After a build: a sketch-sized table overflowed its probe bound.  Returns
// true when the set was re-planned with tuple-sized tables (build again).
bool relset_unsize(dim3g_relset* s, const dim3g_relation* rels, int* rc) {
    *rc = DIM3G_OK;
    if (!((uint32_t)s->h_need[1] & kErrProbeLimit)) return false;
    if (!s->sized) {
        // a tuple-sized table (twice the tuples) cannot fill: a device fault
        *rc = I::fail(s->ctx, DIM3G_ERR_DEVICE, "relation set build: a tuple-sized table overflowed");
        return true;
    }
    s->sized = false;
    *rc = relset_plan(s, rels, s->nrel, s->yt_cap);
    return true;
}

// The build launches (stream ordered; capturable).
int relset_enqueue_build(dim3g_relset* s, cudaStream_t st, uint64_t& launches) {
    dim3g_ctx* ctx = s->ctx;
    const RelPools& P = s->P;
    const int sm = I::sm_count(ctx);
    BCU(cudaMemsetAsync(P.TF, 0xff, s->tabtot * 8, st));
    BCU(cudaMemsetAsync(P.TY, 0xff, s->tabtot * 8, st));
    BCU(cudaMemsetAsync(P.nf_cnt, 0, s->nrel * 8, st));
    BCU(cudaMemsetAsync(P.ny_cnt, 0, s->nrel * 8, st));
    BCU(cudaMemsetAsync(P.degF, 0, (s->ntot + 1) * 4, st));
    BCU(cudaMemsetAsync(P.cnt_yt, 0, s->yt_cap * 4, st));
    BCU(cudaMemsetAsync(P.err, 0, 16, st));
    if (s->ntot) {
        k_ix_insert<<<elem_grid(s->ntot, sm), 256, 0, st>>>(P);
        BLAUNCH();
    }
    k_ix_layout<<<1, 1024, 0, st>>>(P, s->tile_lg);
    BLAUNCH();
    device_scan(OccupiedSrc{P.TF}, AssignIdDst{P.TF, P.id2f}, s->tabtot, s->bsum, nullptr, st);
    launches += scan_launches(s->tabtot);
    device_scan(OccupiedSrc{P.TY}, AssignIdDst{P.TY, P.id2y}, s->tabtot, s->bsum, nullptr, st);
    launches += scan_launches(s->tabtot);
    BCU(cudaGetLastError());
    if (s->ntot) {
        k_ix_map<<<elem_grid(s->ntot, sm), 256, 0, st>>>(P);
        BLAUNCH();
    }
    // row pointers up to the id / key counts the layout found (the launch
    // covers the tuple-count bounds; past the counts nothing is read or written)
    device_scan(BoundSrc<U32Src>{U32Src{P.degF}, P.f_need}, BoundDst<RowPtrDst>{RowPtrDst{P.JRf, P.curF}, P.f_need},
                s->ntot + 1, s->bsum, nullptr, st);
    launches += scan_launches(s->ntot + 1);
    device_scan(BoundSrc<U32Src>{U32Src{P.cnt_yt}, P.yt_need}, BoundDst<RowPtrDst>{RowPtrDst{P.JRy, P.curY}, P.yt_need},
                s->yt_cap, s->bsum, nullptr, st);
    launches += scan_launches(s->yt_cap);
    BCU(cudaGetLastError());
    if (s->ntot) {
        k_ix_scatter<<<elem_grid(s->ntot, sm), 256, 0, st>>>(P);
        BLAUNCH();
    }
    BCU(cudaMemcpyAsync(s->h_need, P.yt_need, 8, cudaMemcpyDeviceToHost, st));
    BCU(cudaMemcpyAsync(s->h_need + 1, P.err, 4, cudaMemcpyDeviceToHost, st));
    return DIM3G_OK;
}

// ---------------------------------------------------------------- queries
struct QueryPlan {
    uint32_t nq = 0;
    std::vector<QueryIn> h_qin;
    std::vector<uint64_t> h_qt_off, h_qrow_off;
    std::vector<uint32_t> swapped;
    uint64_t ntot = 0, nrows = 0;
    bool has_project = false, has_count = false;
    QueryPools Q{};
    uint32_t* lists = nullptr;             // 3 x nrows
    unsigned long long* ncls = nullptr;    // rows per class 0..8
    uint32_t* next_row = nullptr;          // 8 dynamic counters (4..6: split block launches)
    uint64_t* bsum = nullptr;
    uint32_t* part = nullptr;              // class-list partition: per-tile bucket offsets
    unsigned long long* pbase = nullptr;   // its bucket starts (8)
};

// Device layout of a query pass's scratch (every size monotone in the
// arguments, so scratch laid out for maxima fits every smaller pass).
struct QLayout {
    size_t qin, qt, qr, ymap, ICq, JRq, ucap, cls, wrow, rc, rs, res, lists, ncls, next, bsum, part, pbase, total;
};
QLayout query_layout(uint32_t nq, uint64_t ntot, uint64_t nrows) {
    Layout L;
    QLayout o;
    o.qin = L.add<QueryIn>(nq);
    o.qt = L.add<uint64_t>(nq + 1);
    o.qr = L.add<uint64_t>(nq + 1);
    o.ymap = L.add<uint32_t>(ntot);
    o.ICq = L.add<uint32_t>(ntot);
    o.JRq = L.add<uint32_t>(nrows);
    o.ucap = L.add<uint32_t>(nrows);
    o.cls = L.add<uint8_t>(nrows);
    o.wrow = L.add<unsigned long long>(nrows);
    o.rc = L.add<RowCtx>(nq);
    o.rs = L.add<Reserve>(nq);
    o.res = L.add<QueryRes>(nq);
    o.lists = L.add<uint32_t>(4 * nrows);
    o.ncls = L.add<unsigned long long>(24);  // [16..18]: block-class rows by hash-set size
    o.next = L.add<uint32_t>(8);
    o.bsum = L.add<uint64_t>(scan_storage(nrows));
    o.part = L.add<uint32_t>(8 * ((nrows + kPartTile - 1) / kPartTile));
    o.pbase = L.add<unsigned long long>(8);
    o.total = L.total;
    return o;
}

int query_plan(dim3g_relset* s, QueryScratch& qs, const dim3g_query* q, uint32_t nq, QueryPlan& qp) {
    dim3g_ctx* ctx = s->ctx;
    qp.nq = nq;
    qp.h_qin.resize(nq);
    qp.swapped.resize(nq);
    qp.h_qt_off.assign(nq + 1, 0);
    qp.h_qrow_off.assign(nq + 1, 0);
    for (uint32_t i = 0; i < nq; i++) {
        if (q[i].r >= s->nrel || q[i].s >= s->nrel)
            return I::fail(ctx, DIM3G_ERR_INVALID, "query %u: relation index out of range", i);
        if (q[i].op != DIM3G_OP_PROJECT && q[i].op != DIM3G_OP_COUNT)
            return I::fail(ctx, DIM3G_ERR_INVALID, "query %u: unknown op %u", i, q[i].op);
        if (q[i].capacity && (!q[i].d_out || (q[i].op == DIM3G_OP_COUNT && !q[i].d_cnt)))
            return I::fail(ctx, DIM3G_ERR_INVALID, "query %u: null output with nonzero capacity", i);
        if (((uintptr_t)q[i].d_out & 7u) || ((uintptr_t)q[i].d_cnt & 7u))
            return I::fail(ctx, DIM3G_ERR_INVALID, "query %u: outputs not 8-byte aligned", i);
        const uint64_t nr = s->h_in[q[i].r].n, ns = s->h_in[q[i].s].n;
        const bool sw = nr < ns;  // the larger relation drives the rows
        QueryIn qi{};
        qi.p = sw ? q[i].s : q[i].r;
        qi.q = sw ? q[i].r : q[i].s;
        qi.op = q[i].op == DIM3G_OP_COUNT ? kOpCount : kOpProject;
        qi.out = (uint2*)q[i].d_out;
        qi.out_cnt = (unsigned long long*)q[i].d_cnt;
        qi.cap = q[i].capacity;
        // an empty side gives an empty result: no rows
        const uint64_t np = (nr == 0 || ns == 0) ? 0 : s->h_in[qi.p].n;
        qp.h_qin[i] = qi;
        qp.swapped[i] = sw;
        qp.h_qt_off[i + 1] = qp.h_qt_off[i] + np;
        qp.h_qrow_off[i + 1] = qp.h_qrow_off[i] + np + 1;
        if (qi.op == kOpCount) qp.has_count = true;
        else qp.has_project = true;
    }
    qp.ntot = qp.h_qt_off[nq];
    qp.nrows = qp.h_qrow_off[nq];
    if (qp.nrows >= 0xFFFFFFFFull)
        return I::fail(ctx, DIM3G_ERR_UNSUPPORTED, "a query pass covers fewer than 2^32-1 rows in total");

    const QLayout o = query_layout(nq, qp.ntot, qp.nrows);
    if (qs.qmem && qs.qmem_bytes < o.total) {
        cudaFree(qs.qmem);
        qs.qmem = nullptr;
        qs.qmem_bytes = 0;
    }
    if (!qs.qmem) {
        if (cudaMalloc(&qs.qmem, o.total) != cudaSuccess) {
            cudaGetLastError();
            return I::fail(ctx, DIM3G_ERR_NOMEM, "query pass: device allocation of %zu bytes failed", o.total);
        }
        qs.qmem_bytes = o.total;
    }
    if (qs.h_res_n < nq) {
        if (qs.h_res) cudaFreeHost(qs.h_res);
        qs.h_res = nullptr;
        qs.h_res_n = 0;
        if (cudaMallocHost((void**)&qs.h_res, (size_t)nq * sizeof(QueryRes)) != cudaSuccess) {
            cudaGetLastError();
            return I::fail(ctx, DIM3G_ERR_NOMEM, "query pass: pinned allocation failed");
        }
        qs.h_res_n = nq;
    }
    char* m = qs.qmem;
    QueryPools& Q = qp.Q;
    const RelPools& P = s->P;
    Q.rel = P.rel;
    Q.qin = (const QueryIn*)(m + o.qin);
    Q.nq = nq;
    Q.qt_off = (const uint64_t*)(m + o.qt);
    Q.qrow_off = (const uint64_t*)(m + o.qr);
    Q.ntot = qp.ntot;
    Q.nrows = qp.nrows;
    Q.TY = P.TY;
    Q.id2f = P.id2f;
    Q.id2y = P.id2y;
    Q.JRf = P.JRf;
    Q.ICf = P.ICf;
    Q.ICr = P.ICr;
    Q.JRy = P.JRy;
    Q.ICy = P.ICy;
    Q.VSy = P.VSy;
    Q.yt_need = P.yt_need;
    Q.yt_cap = P.yt_cap;
    Q.ymap = (uint32_t*)(m + o.ymap);
    Q.ICq = (uint32_t*)(m + o.ICq);
    Q.JRq = (uint32_t*)(m + o.JRq);
    Q.ucap = (uint32_t*)(m + o.ucap);
    Q.cls = (uint8_t*)(m + o.cls);
    Q.wrow = (unsigned long long*)(m + o.wrow);
    Q.rc = (RowCtx*)(m + o.rc);
    Q.rs = (Reserve*)(m + o.rs);
    Q.res = (QueryRes*)(m + o.res);
    qp.lists = (uint32_t*)(m + o.lists);
    qp.ncls = (unsigned long long*)(m + o.ncls);
    qp.next_row = (uint32_t*)(m + o.next);
    qp.bsum = (uint64_t*)(m + o.bsum);
    qp.part = (uint32_t*)(m + o.part);
    qp.pbase = (unsigned long long*)(m + o.pbase);
    return DIM3G_OK;
}

// Uploads the query descriptors (outside any capture: pageable copies).
int query_upload(dim3g_relset* s, const QueryPlan& qp) {
    dim3g_ctx* ctx = s->ctx;
    BCU(cudaMemcpy((void*)qp.Q.qin, qp.h_qin.data(), qp.nq * sizeof(QueryIn), cudaMemcpyHostToDevice));
    BCU(cudaMemcpy((void*)qp.Q.qt_off, qp.h_qt_off.data(), (qp.nq + 1) * 8, cudaMemcpyHostToDevice));
    BCU(cudaMemcpy((void*)qp.Q.qrow_off, qp.h_qrow_off.data(), (qp.nq + 1) * 8, cudaMemcpyHostToDevice));
    return DIM3G_OK;
}

struct ClassList {
    uint32_t* list;
    unsigned long long* n;
};

// The query pass (stream ordered; capturable).
int query_enqueue(dim3g_relset* s, QueryScratch& qs, QueryPlan& qp, cudaStream_t st, uint64_t& launches) {
    dim3g_ctx* ctx = s->ctx;
    QueryPools& Q = qp.Q;
    const int sm = I::sm_count(ctx);
    const Tuning tu = tuning_of(ctx);
    const uint32_t nq = qp.nq;
    Q.cta_rr = tu.cta_rr;
    BCU(cudaMemsetAsync(qp.ncls, 0, 24 * 8, st));
    BCU(cudaMemsetAsync(Q.cls, 0, qp.nrows, st));
    BCU(cudaMemsetAsync(Q.wrow, 0, qp.nrows * 8, st));
    BCU(cudaMemsetAsync(qp.next_row, 0, 8 * 4, st));
    k_q_setup<<<(nq + 127) / 128, 128, 0, st>>>(Q);
    BLAUNCH();
    if (qp.ntot) {
        k_q_ymap<<<elem_grid(qp.ntot, sm), 256, 0, st>>>(Q);
        BLAUNCH();
        k_q_entries<<<elem_grid(qp.ntot, sm), 256, 0, st>>>(Q);
        BLAUNCH();
    }
    k_q_rows<<<elem_grid(qp.nrows, sm), 256, 0, st>>>(Q);
    BLAUNCH();
    const uint32_t cap_w = 1u << (tu.warp_lg - 1), cap_b = 1u << (tu.block_lg - 1);
    k_q_row_work<<<elem_grid(qp.nrows, sm), 256, 0, st>>>(Q, cap_w, cap_b);
    BLAUNCH();
    uint32_t* lw = qp.lists;
    uint32_t* lb = qp.lists + qp.nrows;
    uint32_t* lm = qp.lists + 2 * qp.nrows;
    uint32_t* lt = qp.lists + 3 * qp.nrows;
    const uint32_t bm_words = (1u << s->tile_lg) / 32;  // the tiling the set was built with
    for (int op = 0; op < 2; op++) {
        if (op == 0 && !qp.has_project) continue;
        if (op == 1 && !qp.has_count) continue;
        const uint8_t k0 = op ? 8 : 0;
        unsigned long long* n = qp.ncls + 8 * op;  // n[1..5]: rows of classes k0+1..k0+5
        unsigned long long* nb = qp.ncls + 16;  // block-class rows by hash-set size (project, split)
        const bool split = op == 0 && tu.block_split;
        {
            // the class lists (and the CTA class by hash-set size) in one partition
            const uint32_t b = tu.block_lg;
            const PartSpec ps{k0, split ? 1u : 0u, 1u << (b - 3), 1u << (b - 2)};
            const uint64_t ntiles = (qp.nrows + kPartTile - 1) / kPartTile;
            if (ntiles) {
                k_part_count<<<(unsigned)ntiles, 256, 0, st>>>(Q.cls, Q.ucap, qp.nrows, ps, qp.part);
                BLAUNCH();
                k_part_offsets<<<1, 1024, 0, st>>>(qp.part, (uint32_t)ntiles, n, split ? nb : nullptr, qp.pbase);
                BLAUNCH();
                k_part_scatter<<<(unsigned)ntiles, 256, 0, st>>>(Q.cls, Q.ucap, qp.nrows, ps, qp.part, qp.pbase, lw, lb,
                                                                 lm, lt);
                BLAUNCH();
            }
        }
        BCU(cudaGetLastError());
        BCU(cudaMemsetAsync(qp.next_row, 0, 8 * 4, st));
        if (op == 0) {
            const size_t ss_m = (size_t)bm_words * 4 + 16 * kStage * 4;
            k_b_single_bitmap<<<resident(k_b_single_bitmap, 512, ss_m, sm), 512, ss_m, st>>>(
                Q, BatchRows{lm, &n[4], &n[3], &qp.next_row[0]}, bm_words);
            BLAUNCH();
            const int blk_b = (int)tu.block_threads;
            if (split) {
                const unsigned long long* skip[3][2] = {{nullptr, nullptr}, {&nb[0], nullptr}, {&nb[0], &nb[1]}};
                for (uint32_t k = 0; k < 3; k++) {
                    const int thr = k < 2 ? (int)kBlockSplitThreads : blk_b;
                    const uint32_t lg = tu.block_lg - 2 + k;
                    const size_t ss = ((size_t)1 << lg) * 4 + (size_t)(thr / 32) * kStage * 4;
                    k_b_single_block<<<resident(k_b_single_block, thr, ss, sm), thr, ss, st>>>(
                        Q, BatchRows{lb, &nb[k], nullptr, &qp.next_row[4 + k], skip[k][0], skip[k][1]}, lg);
                    BLAUNCH();
                }
            } else {
                const size_t ss_b = ((size_t)1 << tu.block_lg) * 4 + (size_t)(blk_b / 32) * kStage * 4;
                k_b_single_block<<<resident(k_b_single_block, blk_b, ss_b, sm), blk_b, ss_b, st>>>(
                    Q, BatchRows{lb, &n[2], nullptr, &qp.next_row[1]}, tu.block_lg);
                BLAUNCH();
            }
            const uint32_t wps = warps_for(warp_row_words(tu.warp_lg, kStage) * 4);
            const size_t ss_w = (size_t)wps * warp_row_words(tu.warp_lg, kStage) * 4;
            k_b_single_warp<<<resident(k_b_single_warp, 32 * wps, ss_w, sm), 32 * wps, ss_w, st>>>(
                Q, BatchRows{lw, &n[1], nullptr, nullptr}, tu.warp_lg, kStage);
            BLAUNCH();
            const uint32_t wpt = warps_for(warp_row_words(kTinyLg, kTinyStage) * 4);
            const size_t ss_t = (size_t)wpt * warp_row_words(kTinyLg, kTinyStage) * 4;
            k_b_single_warp<<<resident(k_b_single_warp, 32 * wpt, ss_t, sm), 32 * wpt, ss_t, st>>>(
                Q, BatchRows{lt, &n[5], nullptr, nullptr}, kTinyLg, kTinyStage);
            BLAUNCH();
        } else {
            const unsigned g_t = (unsigned)(2 * sm);
            k_b_agg_tile<<<g_t, 512, 0, st>>>(Q, BatchRows{lm, &n[4], &n[3], &qp.next_row[2]}, qs.agg,
                                              1u << s->tile_lg);
            BLAUNCH();
            const size_t ss_b = (size_t)2 << tu.block_lg << 2;
            k_b_agg_block<<<resident(k_b_agg_block, 256, ss_b, sm), 256, ss_b, st>>>(
                Q, BatchRows{lb, &n[2], nullptr, &qp.next_row[3]}, tu.block_lg);
            BLAUNCH();
            const uint32_t wpa = warps_for(agg_warp_words(tu.warp_lg, kStage) * 4);
            const size_t ss_w = (size_t)wpa * agg_warp_words(tu.warp_lg, kStage) * 4;
            k_b_agg_warp<<<resident(k_b_agg_warp, 32 * wpa, ss_w, sm), 32 * wpa, ss_w, st>>>(
                Q, BatchRows{lw, &n[1], nullptr, nullptr}, tu.warp_lg, kStage);
            BLAUNCH();
            const uint32_t wpt = warps_for(agg_warp_words(kTinyLg, kTinyStage) * 4);
            const size_t ss_t = (size_t)wpt * agg_warp_words(kTinyLg, kTinyStage) * 4;
            k_b_agg_warp<<<resident(k_b_agg_warp, 32 * wpt, ss_t, sm), 32 * wpt, ss_t, st>>>(
                Q, BatchRows{lt, &n[5], nullptr, nullptr}, kTinyLg, kTinyStage);
            BLAUNCH();
        }
    }
    BCU(cudaMemcpyAsync(qs.h_res, Q.res, (size_t)nq * sizeof(QueryRes), cudaMemcpyDeviceToHost, st));
    return DIM3G_OK;
}

// Shared-memory limits of the batch kernels (per device, idempotent).
// Limits for the largest settings (tiles of 2^19 bits, 2^14-slot CTA sets,
// 1024-thread CTAs).
int set_batch_attributes(dim3g_ctx* ctx) {
    const int bm = (1 << 19) / 8 + 16 * (int)kStage * 4;
    const int blk = (1 << 14) * 4 + 32 * (int)kStage * 4;
    BCU(cudaFuncSetAttribute(k_b_single_bitmap, cudaFuncAttributeMaxDynamicSharedMemorySize, bm));
    BCU(cudaFuncSetAttribute(k_b_single_block, cudaFuncAttributeMaxDynamicSharedMemorySize, blk));
    BCU(cudaFuncSetAttribute(k_b_single_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    BCU(cudaFuncSetAttribute(k_b_agg_block, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 << 14 << 2));
    BCU(cudaFuncSetAttribute(k_b_agg_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024));
    return DIM3G_OK;
}

int ensure_agg_scratch(dim3g_relset* s, QueryScratch& qs) {
    dim3g_ctx* ctx = s->ctx;
    const size_t need = (size_t)2 * I::sm_count(ctx) * 2 * ((size_t)1 << s->tile_lg) * 4;
    if (qs.agg_bytes >= need) return DIM3G_OK;
    if (qs.agg) cudaFree(qs.agg);
    qs.agg = nullptr;
    qs.agg_bytes = 0;
    if (cudaMalloc(&qs.agg, need) != cudaSuccess) {
        cudaGetLastError();
        return I::fail(ctx, DIM3G_ERR_NOMEM, "COUNT scratch: device allocation of %zu bytes failed", need);
    }
    // counters start at zero; every row resets the counters it touched
    BCU(cudaMemset(qs.agg, 0, need));
    qs.agg_bytes = need;
    return DIM3G_OK;
}

// Results of a finished pass into the caller's query array.
int query_results(dim3g_relset* s, const QueryScratch& qs, const QueryPlan& qp, dim3g_query* q) {
    int first = DIM3G_OK;
    for (uint32_t i = 0; i < qp.nq; i++) {
        const QueryRes& r = qs.h_res[i];
        q[i].swapped = qp.swapped[i];
        q[i].n_out = r.n_out;
        q[i].out_j = r.out_j;
        int st = DIM3G_OK;
        if (r.err) st = DIM3G_ERR_DEVICE;
        else if (r.n_out > q[i].capacity) st = DIM3G_ERR_CAPACITY;
        q[i].status = st;
        if (st && !first) {
            first = st;
            I::fail(s->ctx, st, "query %u: %s", i,
                    st == DIM3G_ERR_DEVICE ? "device bound violated" : "output buffer too small");
        }
    }
    return first;
}

int relset_build_sync(dim3g_relset* s, const dim3g_relation* rels) {
    dim3g_ctx* ctx = s->ctx;
    cudaStream_t st = I::stream(ctx);
    for (int attempt = 0; attempt < 3; attempt++) {
        uint64_t launches = 0;
        int r = relset_enqueue_build(s, st, launches);
        I::add_launches(ctx, launches);
        if (r) return r;
        BCU(cudaStreamSynchronize(st));
        if (relset_unsize(s, rels, &r)) {
            if (r) return r;
            continue;
        }
        const uint64_t need = s->h_need[0];
        const uint32_t err = (uint32_t)s->h_need[1];
        if (need <= s->yt_cap) {
            if (err) return I::fail(ctx, DIM3G_ERR_DEVICE, "relation set build: device bound violated (flags %u)", err);
            return DIM3G_OK;
        }
        r = relset_plan(s, rels, s->nrel, need);  // regrow the (y, tile) pool
        if (r) return r;
    }
    return I::fail(ctx, DIM3G_ERR_DEVICE, "relation set build: key space did not converge");
}

}  // namespace

// ================================================================== batch
struct dim3g_batch {
    dim3g_relset set;
    QueryPlan qp;
    std::vector<dim3g_relation> rels;
    std::vector<dim3g_query> queries;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    uint64_t launches_per_run = 0;
    float ms_last = 0;
    ~dim3g_batch() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (ev0) cudaEventDestroy(ev0);
        if (ev1) cudaEventDestroy(ev1);
    }
};

namespace {

int batch_capture(dim3g_batch* b) {
    dim3g_ctx* ctx = b->set.ctx;
    cudaStream_t st = I::stream(ctx);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
    int r = query_upload(&b->set, b->qp);
    if (r) return r;
    BCU(cudaStreamSynchronize(st));
    uint64_t launches = 0;
    BCU(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    r = relset_enqueue_build(&b->set, st, launches);
    if (!r) r = query_enqueue(&b->set, b->set.qs, b->qp, st, launches);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(st, &g);
    if (r) {
        if (g) cudaGraphDestroy(g);
        return r;
    }
    if (e != cudaSuccess) return I::fail(ctx, DIM3G_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
    b->graph = g;
    BCU(cudaGraphInstantiate(&b->exec, g, 0));
    b->launches_per_run = launches;
    return DIM3G_OK;
}

}  // namespace

extern "C" {

int dim3g_relset_create(dim3g_ctx* ctx, const dim3g_relation* rels, uint32_t n, dim3g_relset** out) {
    if (!ctx || !out || (n && !rels)) return DIM3G_ERR_INVALID;
    *out = nullptr;
    if (n == 0) return I::fail(ctx, DIM3G_ERR_INVALID, "empty relation set");
    BCU(cudaSetDevice(I::device(ctx)));
    dim3g_relset* s = new dim3g_relset();
    s->ctx = ctx;
    s->tile_lg = tuning_of(ctx).tile_lg;
    int r = cudaMallocHost((void**)&s->h_need, 16) == cudaSuccess ? DIM3G_OK
                                                                   : I::fail(ctx, DIM3G_ERR_NOMEM, "pinned allocation failed");
    if (!r) r = set_batch_attributes(ctx);
    if (!r) r = relset_sketch(s, rels, n);
    if (!r) r = relset_plan(s, rels, n, 0);
    if (!r) r = relset_build_sync(s, rels);
    if (r) {
        delete s;
        return r;
    }
    *out = s;
    return DIM3G_OK;
}

void dim3g_relset_destroy(dim3g_relset* s) {
    if (!s) return;
    cudaStreamSynchronize(I::stream(s->ctx));
    delete s;
}

uint64_t dim3g_relset_bytes(const dim3g_relset* s) {
    return s ? (uint64_t)(s->mem_bytes + s->qs.qmem_bytes + s->qs.agg_bytes) : 0;
}

int dim3g_relset_join(dim3g_relset* s, dim3g_query* q, uint32_t n) {
    if (!s || (n && !q)) return DIM3G_ERR_INVALID;
    if (n == 0) return DIM3G_OK;
    dim3g_ctx* ctx = s->ctx;
    BCU(cudaSetDevice(I::device(ctx)));
    cudaStream_t st = I::stream(ctx);
    QueryPlan qp;
    int r = query_plan(s, s->qs, q, n, qp);
    if (!r && qp.has_count) r = ensure_agg_scratch(s, s->qs);
    if (!r) r = query_upload(s, qp);
    if (r) return r;
    uint64_t launches = 0;
    r = query_enqueue(s, s->qs, qp, st, launches);
    I::add_launches(ctx, launches);
    if (r) return r;
    BCU(cudaStreamSynchronize(st));
    return query_results(s, s->qs, qp, q);
}

int dim3g_batch_create(dim3g_ctx* ctx, const dim3g_relation* rels, const dim3g_query* q, uint32_t n, dim3g_batch** out) {
    if (!ctx || !out || (n && (!rels || !q))) return DIM3G_ERR_INVALID;
    *out = nullptr;
    if (n == 0) return I::fail(ctx, DIM3G_ERR_INVALID, "empty batch");
    BCU(cudaSetDevice(I::device(ctx)));
    dim3g_batch* b = new dim3g_batch();
    b->set.ctx = ctx;
    b->set.tile_lg = tuning_of(ctx).tile_lg;
    b->rels.assign(rels, rels + 2 * (size_t)n);
    b->queries.assign(q, q + n);
    for (uint32_t i = 0; i < n; i++) {
        b->queries[i].r = 2 * i;
        b->queries[i].s = 2 * i + 1;
    }
    int r = cudaMallocHost((void**)&b->set.h_need, 16) == cudaSuccess
                ? DIM3G_OK
                : I::fail(ctx, DIM3G_ERR_NOMEM, "pinned allocation failed");
    if (!r && (cudaEventCreate(&b->ev0) != cudaSuccess || cudaEventCreate(&b->ev1) != cudaSuccess))
        r = I::fail(ctx, DIM3G_ERR_CUDA, "event creation failed");
    if (!r) r = set_batch_attributes(ctx);
    if (!r) {
        // each relation of a batch has one role: the relation that drives its
        // join (the larger, as query_plan swaps) needs only its CSR by first
        // value, the other only its CSR by (y, z tile)
        b->set.h_roles.assign(2 * (size_t)n, 0);
        for (uint32_t i = 0; i < n; i++) {
            const bool sw = rels[2 * i].n < rels[2 * i + 1].n;
            b->set.h_roles[2 * i + (sw ? 1 : 0)] |= kRoleRows;
            b->set.h_roles[2 * i + (sw ? 0 : 1)] |= kRoleCols;
        }
    }
    if (!r) r = relset_sketch(&b->set, b->rels.data(), 2 * n);
    if (!r) r = relset_plan(&b->set, b->rels.data(), 2 * n, 0);
    if (!r) r = query_plan(&b->set, b->set.qs, b->queries.data(), n, b->qp);
    if (!r && b->qp.has_count) r = ensure_agg_scratch(&b->set, b->set.qs);
    if (!r) r = batch_capture(b);
    if (r) {
        delete b;
        return r;
    }
    *out = b;
    return DIM3G_OK;
}

int dim3g_batch_run(dim3g_batch* b, dim3g_query* q) {
    if (!b || !q) return DIM3G_ERR_INVALID;
    dim3g_ctx* ctx = b->set.ctx;
    BCU(cudaSetDevice(I::device(ctx)));
    cudaStream_t st = I::stream(ctx);
    for (int attempt = 0; attempt < 3; attempt++) {
        BCU(cudaEventRecord(b->ev0, st));
        BCU(cudaGraphLaunch(b->exec, st));
        BCU(cudaEventRecord(b->ev1, st));
        BCU(cudaStreamSynchronize(st));
        I::add_launches(ctx, b->launches_per_run);
        cudaEventElapsedTime(&b->ms_last, b->ev0, b->ev1);
        int r = DIM3G_OK;
        if (relset_unsize(&b->set, b->rels.data(), &r)) {
            // a sketch-sized table overflowed: tuple-sized tables from now on
            if (!r) r = query_plan(&b->set, b->set.qs, b->queries.data(), b->qp.nq, b->qp);
            if (!r) r = batch_capture(b);
            if (r) return r;
            continue;
        }
        const uint64_t need = b->set.h_need[0];
        if (need <= b->set.yt_cap) {
            const uint32_t err = (uint32_t)b->set.h_need[1];
            if (err) return I::fail(ctx, DIM3G_ERR_DEVICE, "batch index build: device bound violated (flags %u)", err);
            for (uint32_t i = 0; i < b->qp.nq; i++) {
                q[i].capacity = b->queries[i].capacity;
                q[i].op = b->queries[i].op;
            }
            return query_results(&b->set, b->set.qs, b->qp, q);
        }
        // the (y, f tile) key space outgrew its pool: re-plan and capture
        r = relset_plan(&b->set, b->rels.data(), (uint32_t)b->rels.size(), need);
        if (!r) r = query_plan(&b->set, b->set.qs, b->queries.data(), b->qp.nq, b->qp);
        if (!r) r = batch_capture(b);
        if (r) return r;
    }
    return I::fail(ctx, DIM3G_ERR_DEVICE, "batch: key space did not converge");
}

// The autotuner for a batch: the batch graph itself is timed under candidate
// knob settings (re-captured per trial), coordinate descent as in
// dim3g_autotune; the fastest settings stay applied and captured.
int dim3g_batch_autotune(dim3g_batch* b, uint32_t max_trials, dim3g_tuning* out) {
    if (!b || !out) return DIM3G_ERR_INVALID;
    dim3g_ctx* ctx = b->set.ctx;
    memset(out, 0, sizeof *out);
    struct K {
        const char* name;
        std::vector<int64_t> values;
    };
    const std::vector<K> knobs = {{"cta_walk", {3, 0, 1, 2}},
                                  {"block_slots_log2", {14, 13, 12}},
                                  {"warp_slots_log2", {11, 10, 9, 12}},
                                  {"block_threads", {512, 256, 1024}},
                                  {"tile_bits_log2", {19, 18, 17}}};
    std::vector<int64_t> best(knobs.size());
    for (size_t i = 0; i < knobs.size(); i++) {
        const int r = dim3g_get_param(ctx, knobs[i].name, &best[i]);
        if (r) return r;
    }
    std::vector<dim3g_query> q = b->queries;
    auto time_it = [&](float* ms) -> int {
        int r = batch_capture(b);
        float m = 1e30f;
        for (int k = 0; k < 2 && !r; k++) {
            r = dim3g_batch_run(b, q.data());
            if (b->ms_last < m) m = b->ms_last;
        }
        *ms = m;
        return r;
    };
    auto apply = [&](const std::vector<int64_t>& v) -> int {
        for (size_t i = 0; i < knobs.size(); i++) {
            const int r = dim3g_set_param(ctx, knobs[i].name, v[i]);
            if (r) return r;
        }
        return DIM3G_OK;
    };
    float best_ms = 0;
    int r = time_it(&best_ms);
    uint32_t trials = 1;
    const float ms_default = best_ms;
    for (size_t i = 0; i < knobs.size() && !r; i++) {
        for (int64_t v : knobs[i].values) {
            if (v == best[i]) continue;
            if (max_trials && trials >= max_trials) break;
            std::vector<int64_t> cand = best;
            cand[i] = v;
            if (apply(cand)) continue;
            float ms = 0;
            r = time_it(&ms);
            trials++;
            if (r) break;
            if (ms < best_ms) {
                best_ms = ms;
                best = cand;
            }
        }
    }
    const int r2 = apply(best);
    const int r3 = r2 ? r2 : batch_capture(b);
    if (r) return r;
    if (r3) return r3;
    {
        int64_t db = 0, dk = 0;
        dim3g_get_param(ctx, "dense_block", &db);
        dim3g_get_param(ctx, "dense_k_max", &dk);
        out->dense_block = (int32_t)db;  // not swept: batches run no dense block
        out->dense_k_max = (int32_t)dk;
    }
    out->cta_walk = (int32_t)best[0];
    out->block_slots_log2 = (int32_t)best[1];
    out->warp_slots_log2 = (int32_t)best[2];
    out->block_threads = (int32_t)best[3];
    out->tile_bits_log2 = (int32_t)best[4];
    out->ms = best_ms;
    out->ms_default = ms_default;
    out->trials = trials;
    return DIM3G_OK;
}

int dim3g_batch_info(const dim3g_batch* b, float* ms_last, uint64_t* launches_per_run, uint64_t* device_bytes) {
    if (!b) return DIM3G_ERR_INVALID;
    if (ms_last) *ms_last = b->ms_last;
    if (launches_per_run) *launches_per_run = b->launches_per_run;
    if (device_bytes) *device_bytes = (uint64_t)(b->set.mem_bytes + b->set.qs.qmem_bytes + b->set.qs.agg_bytes);
    return DIM3G_OK;
}

void dim3g_batch_destroy(dim3g_batch* b) {
    if (!b) return;
    cudaStreamSynchronize(I::stream(b->set.ctx));
    delete b;
}

}  // extern "C"

// ================================================================ serving
namespace {

struct SrvReq {
    uint32_t r = 0, s = 0, op = 0;
    uint64_t cap = 0;    // reserved pairs
    uint64_t bytes = 0;  // reserved output bytes
    uint64_t rows = 0;   // entries of the driving relation (lane scratch)
    void* d_out = nullptr;
    void* d_cnt = nullptr;
    double t_submit = 0, t_start = 0, t_done = 0;
    int32_t status = 0;
    uint32_t swapped = 0, pass_size = 0, lane = 0;
    uint64_t n_out = 0, out_j = 0;
    bool done = false;
};

struct Lane {
    cudaStream_t st = nullptr;
    QueryScratch qs;
    QueryPlan qp;
    QueryIn* h_qin = nullptr;  // pinned staging of the pass's descriptors
    uint64_t* h_qt = nullptr;
    uint64_t* h_qr = nullptr;
    std::thread th;
    ~Lane() {
        if (h_qin) cudaFreeHost(h_qin);
        if (h_qt) cudaFreeHost(h_qt);
        if (h_qr) cudaFreeHost(h_qr);
        if (st) cudaStreamDestroy(st);
    }
};

}  // namespace

struct dim3g_server {
    dim3g_relset* set = nullptr;
    dim3g_ctx* ctx = nullptr;
    uint32_t max_batch = 0;
    uint64_t entries_cap = 0;  // entries of driving relations one pass may hold
    uint64_t out_budget = 0, reserved = 0;
    std::vector<uint64_t> outj, nt;  // pair matrix; tuples per relation
    std::vector<uint64_t> nf;        // distinct first values per relation
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<SrvReq*> pending;
    std::unordered_map<uint64_t, std::unique_ptr<SrvReq>> reqs;
    uint64_t next_ticket = 1, completed = 0, passes = 0;
    bool stop = false;
    std::vector<std::unique_ptr<Lane>> lanes;
    cudaStream_t free_st = nullptr;
    cudaMemPool_t pool = nullptr;
    std::chrono::steady_clock::time_point t0;

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }
};

namespace {

// One lane: admit, run one pass, complete; until stopped with nothing queued.
void lane_main(dim3g_server* S, uint32_t li) {
    Lane& L = *S->lanes[li];
    dim3g_relset* set = S->set;
    cudaSetDevice(I::device(S->ctx));
    std::vector<SrvReq*> batch;
    std::vector<dim3g_query> qv;
    for (;;) {
        batch.clear();
        {
            std::unique_lock<std::mutex> lk(S->mu);
            S->cv_work.wait(lk, [&] {
                return (S->stop && S->pending.empty()) ||
                       (!S->pending.empty() && S->reserved + S->pending.front()->bytes <= S->out_budget);
            });
            if (S->pending.empty()) return;  // stopping
            uint64_t entries = 0;
            while (!S->pending.empty() && batch.size() < S->max_batch) {
                SrvReq* q = S->pending.front();
                if (S->reserved + q->bytes > S->out_budget) break;
                if (!batch.empty() && entries + q->rows > S->entries_cap) break;
                S->reserved += q->bytes;
                entries += q->rows;
                batch.push_back(q);
                S->pending.pop_front();
            }
        }
        const double ts = S->now();
        const uint32_t n = (uint32_t)batch.size();
        qv.assign(n, dim3g_query{});
        int rc = DIM3G_OK;
        for (uint32_t i = 0; i < n && !rc; i++) {
            SrvReq* q = batch[i];
            const size_t pb = (size_t)(q->cap ? q->cap : 1) * 8;
            if (cudaMallocFromPoolAsync(&q->d_out, pb, S->pool, L.st) != cudaSuccess ||
                (q->op == DIM3G_OP_COUNT && cudaMallocFromPoolAsync(&q->d_cnt, pb, S->pool, L.st) != cudaSuccess)) {
                cudaGetLastError();
                rc = DIM3G_ERR_NOMEM;
            }
            qv[i].r = q->r;
            qv[i].s = q->s;
            qv[i].op = q->op;
            qv[i].d_out = (uint32_t*)q->d_out;
            qv[i].d_cnt = (uint64_t*)q->d_cnt;
            qv[i].capacity = q->cap;
        }
        uint64_t launches = 0;
        if (!rc) rc = query_plan(set, L.qs, qv.data(), n, L.qp);
        if (!rc) {
            const QueryPlan& qp = L.qp;
            memcpy(L.h_qin, qp.h_qin.data(), n * sizeof(QueryIn));
            memcpy(L.h_qt, qp.h_qt_off.data(), (n + 1) * 8);
            memcpy(L.h_qr, qp.h_qrow_off.data(), (n + 1) * 8);
            if (cudaMemcpyAsync((void*)qp.Q.qin, L.h_qin, n * sizeof(QueryIn), cudaMemcpyHostToDevice, L.st) ||
                cudaMemcpyAsync((void*)qp.Q.qt_off, L.h_qt, (n + 1) * 8, cudaMemcpyHostToDevice, L.st) ||
                cudaMemcpyAsync((void*)qp.Q.qrow_off, L.h_qr, (n + 1) * 8, cudaMemcpyHostToDevice, L.st))
                rc = DIM3G_ERR_CUDA;
        }
        if (!rc) rc = query_enqueue(set, L.qs, L.qp, L.st, launches);
        if (!rc && cudaStreamSynchronize(L.st) != cudaSuccess) rc = DIM3G_ERR_CUDA;
        const double td = S->now();
        {
            std::lock_guard<std::mutex> lk(S->mu);
            for (uint32_t i = 0; i < n; i++) {
                SrvReq* q = batch[i];
                if (rc) {
                    q->status = rc;
                } else {
                    const QueryRes& r = L.qs.h_res[i];
                    q->n_out = r.n_out;
                    q->out_j = r.out_j;
                    q->swapped = L.qp.swapped[i];
                    q->status = r.err ? DIM3G_ERR_DEVICE : (r.n_out > q->cap ? DIM3G_ERR_CAPACITY : DIM3G_OK);
                }
                q->t_start = ts;
                q->t_done = td;
                q->pass_size = n;
                q->lane = li;
                q->done = true;
            }
            S->completed += n;
            S->passes++;
            I::add_launches(S->ctx, launches);
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
}

int pair_outj(dim3g_relset* s, uint64_t* outj) {
    dim3g_ctx* ctx = s->ctx;
    cudaStream_t st = I::stream(ctx);
    const size_t nb = (size_t)s->nrel * s->nrel * 8;
    unsigned long long* d = nullptr;
    BCU(cudaMalloc(&d, nb));
    cudaError_t e = cudaMemsetAsync(d, 0, nb, st);
    if (e == cudaSuccess) {
        k_pair_outj<<<elem_grid(s->ntot, I::sm_count(ctx)), 256, 0, st>>>(s->P, d);
        e = cudaGetLastError();
        I::add_launches(ctx, 1);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(outj, d, nb, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(d);
    if (e != cudaSuccess) return I::fail(ctx, DIM3G_ERR_CUDA, "pair matrix: %s", cudaGetErrorString(e));
    return DIM3G_OK;
}

}  // namespace

extern "C" {

int dim3g_relset_pair_outj(dim3g_relset* s, uint64_t* outj) {
    if (!s || !outj) return DIM3G_ERR_INVALID;
    dim3g_ctx* ctx = s->ctx;
    BCU(cudaSetDevice(I::device(ctx)));
    return pair_outj(s, outj);
}

int dim3g_server_create(dim3g_relset* set, uint32_t lanes, uint32_t max_batch, uint64_t budget_bytes,
                        dim3g_server** out) {
    if (!set || !out || lanes == 0 || lanes > 16 || max_batch == 0) return DIM3G_ERR_INVALID;
    *out = nullptr;
    dim3g_ctx* ctx = set->ctx;
    BCU(cudaSetDevice(I::device(ctx)));
    std::unique_ptr<dim3g_server> S(new dim3g_server());
    S->set = set;
    S->ctx = ctx;
    S->max_batch = max_batch;
    S->t0 = std::chrono::steady_clock::now();
    const uint32_t n = set->nrel;
    S->outj.assign((size_t)n * n, 0);
    int r = pair_outj(set, S->outj.data());
    if (r) return r;
    // distinct first values per relation (the layout the build computed)
    std::vector<RelDev> rel(n);
    BCU(cudaMemcpy(rel.data(), set->P.rel, n * sizeof(RelDev), cudaMemcpyDeviceToHost));
    S->nf.resize(n);
    S->nt.resize(n);
    uint64_t max_nt = 1;
    for (uint32_t i = 0; i < n; i++) {
        S->nf[i] = rel[i].nf;
        S->nt[i] = rel[i].nt;
        if (rel[i].nt > max_nt) max_nt = rel[i].nt;
    }
    S->entries_cap = 4 * max_nt > ((uint64_t)1 << 25) ? 4 * max_nt : ((uint64_t)1 << 25);
    // lanes: stream, scratch sized for the largest pass, pinned staging
    uint64_t fixed = dim3g_relset_bytes(set);
    for (uint32_t li = 0; li < lanes; li++) {
        std::unique_ptr<Lane> L(new Lane());
        BCU(cudaStreamCreateWithFlags(&L->st, cudaStreamNonBlocking));
        const QLayout o = query_layout(max_batch, S->entries_cap, S->entries_cap + max_batch);
        if (cudaMalloc(&L->qs.qmem, o.total) != cudaSuccess) {
            cudaGetLastError();
            return I::fail(ctx, DIM3G_ERR_NOMEM, "server lane scratch of %zu bytes", o.total);
        }
        L->qs.qmem_bytes = o.total;
        if (cudaMallocHost((void**)&L->qs.h_res, (size_t)max_batch * sizeof(QueryRes)) != cudaSuccess ||
            cudaMallocHost((void**)&L->h_qin, (size_t)max_batch * sizeof(QueryIn)) != cudaSuccess ||
            cudaMallocHost((void**)&L->h_qt, (size_t)(max_batch + 1) * 8) != cudaSuccess ||
            cudaMallocHost((void**)&L->h_qr, (size_t)(max_batch + 1) * 8) != cudaSuccess) {
            cudaGetLastError();
            return I::fail(ctx, DIM3G_ERR_NOMEM, "server lane pinned staging");
        }
        L->qs.h_res_n = max_batch;
        r = ensure_agg_scratch(set, L->qs);
        if (r) return r;
        fixed += L->qs.qmem_bytes + L->qs.agg_bytes;
        S->lanes.push_back(std::move(L));
    }
    if (fixed >= budget_bytes)
        return I::fail(ctx, DIM3G_ERR_NOMEM, "budget %llu bytes below the set and lane scratch (%llu bytes)",
                       (unsigned long long)budget_bytes, (unsigned long long)fixed);
    S->out_budget = budget_bytes - fixed;
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = I::device(ctx);
    BCU(cudaMemPoolCreate(&S->pool, &props));
    uint64_t keep = ~0ull;
    BCU(cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep));
    BCU(cudaStreamCreateWithFlags(&S->free_st, cudaStreamNonBlocking));
    dim3g_server* raw = S.release();
    for (uint32_t li = 0; li < lanes; li++) raw->lanes[li]->th = std::thread(lane_main, raw, li);
    *out = raw;
    return DIM3G_OK;
}

int dim3g_server_submit(dim3g_server* S, uint32_t r, uint32_t s, uint32_t op, uint64_t* ticket) {
    if (!S || !ticket) return DIM3G_ERR_INVALID;
    const uint32_t n = S->set->nrel;
    if (r >= n || s >= n || (op != DIM3G_OP_PROJECT && op != DIM3G_OP_COUNT)) return DIM3G_ERR_INVALID;
    std::unique_ptr<SrvReq> q(new SrvReq());
    q->r = r;
    q->s = s;
    q->op = op;
    const uint64_t oj = S->outj[(size_t)r * n + s];
    const double grid = (double)S->nf[r] * (double)S->nf[s];
    q->cap = (double)oj < grid ? oj : (uint64_t)grid;
    q->bytes = align256((size_t)(q->cap ? q->cap : 1) * 8) * (op == DIM3G_OP_COUNT ? 2 : 1);
    q->rows = S->nt[r] > S->nt[s] ? S->nt[r] : S->nt[s];
    if (q->bytes > S->out_budget || q->rows > S->entries_cap) return DIM3G_ERR_NOMEM;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->stop) return DIM3G_ERR_INVALID;
        q->t_submit = S->now();
        *ticket = S->next_ticket++;
        S->pending.push_back(q.get());
        S->reqs[*ticket] = std::move(q);
    }
    S->cv_work.notify_all();
    return DIM3G_OK;
}

int dim3g_server_wait(dim3g_server* S, uint64_t ticket, dim3g_result* out) {
    if (!S || !out) return DIM3G_ERR_INVALID;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->reqs.find(ticket);
    if (it == S->reqs.end()) return DIM3G_ERR_INVALID;
    SrvReq* q = it->second.get();
    S->cv_done.wait(lk, [&] { return q->done; });
    out->ticket = ticket;
    out->status = q->status;
    out->swapped = q->swapped;
    out->n_out = q->n_out;
    out->out_j = q->out_j;
    out->d_out = (const uint32_t*)q->d_out;
    out->d_cnt = (const uint64_t*)q->d_cnt;
    out->t_submit = q->t_submit;
    out->t_start = q->t_start;
    out->t_done = q->t_done;
    out->pass_size = q->pass_size;
    out->lane = q->lane;
    return DIM3G_OK;
}

int dim3g_server_release(dim3g_server* S, uint64_t ticket) {
    if (!S) return DIM3G_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        auto it = S->reqs.find(ticket);
        if (it == S->reqs.end() || !it->second->done) return DIM3G_ERR_INVALID;
        SrvReq* q = it->second.get();
        if (q->d_out) cudaFreeAsync(q->d_out, S->free_st);
        if (q->d_cnt) cudaFreeAsync(q->d_cnt, S->free_st);
        S->reserved -= q->bytes;
        S->reqs.erase(it);
    }
    S->cv_work.notify_all();
    return DIM3G_OK;
}

int dim3g_server_stats(const dim3g_server* S, uint64_t* completed, uint64_t* passes, uint64_t* reserved_bytes,
                       uint64_t* output_budget) {
    if (!S) return DIM3G_ERR_INVALID;
    std::lock_guard<std::mutex> lk(const_cast<dim3g_server*>(S)->mu);
    if (completed) *completed = S->completed;
    if (passes) *passes = S->passes;
    if (reserved_bytes) *reserved_bytes = S->reserved;
    if (output_budget) *output_budget = S->out_budget;
    return DIM3G_OK;
}

void dim3g_server_destroy(dim3g_server* S) {
    if (!S) return;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->stop = true;
        // completed, unreleased outputs go back to the budget so queued
        // requests can still be admitted and finished
        for (auto& kv : S->reqs) {
            SrvReq* q = kv.second.get();
            if (!q->done) continue;
            if (q->d_out) cudaFreeAsync(q->d_out, S->free_st);
            if (q->d_cnt) cudaFreeAsync(q->d_cnt, S->free_st);
            q->d_out = q->d_cnt = nullptr;
            S->reserved -= q->bytes;
            q->bytes = 0;
        }
    }
    S->cv_work.notify_all();
    for (auto& L : S->lanes)
        if (L->th.joinable()) L->th.join();
    for (auto& kv : S->reqs) {
        SrvReq* q = kv.second.get();
        if (q->d_out) cudaFreeAsync(q->d_out, S->free_st);
        if (q->d_cnt) cudaFreeAsync(q->d_cnt, S->free_st);
    }
    cudaStreamSynchronize(S->free_st);
    cudaStreamDestroy(S->free_st);
    if (S->pool) cudaMemPoolDestroy(S->pool);
    delete S;
}

}  // extern "C"

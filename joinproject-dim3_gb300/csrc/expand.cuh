// expand.cuh -- the sparse expansion with on-chip deduplication: the GPU
// form of Hybrid_solution's SPA loop (dim3.hpp:952-973).
//
// For an x row the candidates are every z of S row y for every y of R row x.
// Rows are binned by u = min(candidates, m), an upper bound on their distinct
// outputs:
//   class 1 (u <= cap_w):  one warp per row, a private shared-memory hash set
//   class 2 (u <= cap_b):  one CTA per row, a shared-memory hash set
//   class 3/4 (u > cap_b): one CTA per row, a shared-memory bitmap over one
//                          z tile at a time (S is bucketed by (y, z tile));
//                          class 4 (u > kHugeRow) rows are scheduled first.
// CTA classes take rows dynamically from an atomic counter.  Each kernel
// runs twice: a count pass writes cnt[x] = |distinct z|; after a prefix sum
// over cnt the write pass repeats the expansion and every first insertion of
// a z emits (x value, z value) at off[x] + a row-local slot, so each row's
// pairs are contiguous and the whole output is dense.
#pragma once
#include "common.cuh"

namespace dim3g {

constexpr uint32_t kEmpty32 = 0xFFFFFFFFu;
constexpr uint32_t kHugeRow = 1u << 16;
constexpr uint32_t kWarpWorkMax = 1u << 14;  // candidates a single warp takes alone
// Tiny rows (few distinct z, few candidates) run in the warp kernel with a
// 2^kTinyLg-slot table and a kTinyStage-pair stage: about 3 KB of shared
// memory per warp, so the latency-bound row walk runs at full occupancy.
constexpr uint32_t kTinyU = 128, kTinyW = 4096, kTinyLg = 8, kTinyStage = 256;

// A hash-class row dedups with a bitmap over the whole z domain instead of
// a hash set when that bitmap fits the kernel's table memory (2^slots_lg
// words) and clearing it costs no more than the row's candidates
// (m <= 32 u, u = min(candidates, m)): no probing, one atomicOr per
// candidate.  Small z domains with many duplicate candidates take this path.
__device__ __forceinline__ bool use_row_bitmap(uint32_t m, uint32_t u, uint32_t slots_lg) {
    return (uint64_t)m <= (32ull << slots_lg) && (uint64_t)m <= 32ull * u;
}
// Row class from its candidates w and u = min(w, m): 5 (one warp, small
// table; only where the caller runs that kernel) for tiny rows, 1 (one warp)
// for few distinct z and few candidates, 2 (one CTA, hash set or bitmap) up
// to cap_b distinct, 3 / 4 (one CTA, z-tile bitmaps; 4 = huge, scheduled
// first) beyond; 0 for an empty row.
__device__ __forceinline__ uint32_t row_class(unsigned long long w, uint32_t u, uint32_t cap_w, uint32_t cap_b,
                                              bool tiny) {
    if (u == 0) return 0;
    if (tiny && u <= kTinyU && w <= kTinyW) return 5;
    if (u <= cap_w && w <= kWarpWorkMax) return 1;
    if (u <= cap_b) return 2;
    return u <= kHugeRow ? 3 : 4;
}
// Words of a whole-domain bitmap, rounded to uint4 and at least 32 (idle
// lanes of TileBitmap touch words 0..31).
__device__ __forceinline__ uint32_t row_bitmap_words(uint32_t m) {
    const uint32_t w = (((m + 31) >> 5) + 3) & ~3u;
    return w < 32 ? 32 : w;
}

struct RowCtx {
    const uint32_t* JR_R;  // n+1 row pointers of R by x id
    const uint32_t* IC_R;  // y ids
    const uint32_t* JR_S;  // k*T+1 row pointers of S by (y id, z tile)
    const uint32_t* IC_S;  // z ids
    const uint32_t* VS;    // z values, parallel to IC_S (value paths when ISV is nullptr)
    const uint2* ISV;      // (z id, z value) pairs parallel to IC_S, or nullptr (value paths load one pair)
    uint32_t T;            // z tiles
    uint32_t tile_width;   // z ids per tile (bitmap width)
    uint32_t m;            // z domain size
    uint32_t cta_rr;       // CTA rows' walk: 0 flattened, 1 chunks round-robin, 2 chunks split, 3 balanced (cta_expand)
    uint32_t flat_avg;     // cross-segment gather below this many candidates a segment (0: kFlatAvgMax)
    const uint32_t* ucap;  // per row min(candidates, m)
    uint32_t* cnt;         // per row distinct count (count pass output)
    const unsigned long long* off;  // per row output offset (write pass input)
    const uint32_t* id2x;
    const uint32_t* id2z;
    uint2* out;
    uint32_t* err;
    uint32_t* next_row;    // dynamic row counters of the CTA classes
};

__device__ __forceinline__ uint32_t ceil_log2(uint32_t v) { return v <= 1 ? 0 : 32 - __clz(v - 1); }

// Insert z into an open-addressing set of 2^lg 32-bit slots in shared memory.
// Returns true for the first insertion of z.
__device__ __forceinline__ bool smem_set_insert(uint32_t* tab, uint32_t lg, uint32_t z, uint32_t* err) {
    const uint32_t mask = (1u << lg) - 1;
    uint32_t h = (z * 0x9E3779B1u) >> (32 - lg);
    volatile uint32_t* vt = tab;
    for (uint32_t p = 0; p <= mask; p++) {
        uint32_t cur = vt[h];
        if (cur == z) return false;
        if (cur == kEmpty32) {
            uint32_t prev = atomicCAS(&tab[h], kEmpty32, z);
            if (prev == kEmpty32) return true;
            if (prev == z) return false;
        }
        h = (h + 1) & mask;
    }
    raise_error(err, kErrTableFull);
    return false;
}

#ifndef DIM3G_UNROLL
#define DIM3G_UNROLL 4
#endif
#ifndef DIM3G_MIN_PIECE
#define DIM3G_MIN_PIECE 256
#endif
#ifndef DIM3G_FLAT_AVG
#define DIM3G_FLAT_AVG 96
#endif
constexpr uint32_t kUnroll = DIM3G_UNROLL;
constexpr uint32_t kMinPiece = DIM3G_MIN_PIECE;
// A chunk whose segments average fewer candidates than this is gathered
// across segment boundaries (see warp_expand); RowCtx::flat_avg overrides it
// per launch (the single pass sets it per row class).
constexpr uint32_t kFlatAvgMax = DIM3G_FLAT_AVG;

// Warp-level expansion of the candidates of R entries [e0, e1) over S tiles
// [t0, t1).  Entries are taken 32 at a time; a warp prefix sum over their S
// segment lengths flattens the chunk's candidates into [0, total), which is
// cut into a power-of-two number (<= nparts) of contiguous pieces of at least
// kMinPiece candidates; the calling warp takes piece `part`.  When the
// chunk's segments are short on average it gathers its piece across segment
// boundaries (each lane looks up its candidate's segment); otherwise it
// finds the segment holding its first candidate with one ballot over the
// lanes' inclusive prefixes, then walks the segments overlapping its piece,
// the lanes striding each segment kUnroll x 32 candidates at a time.
//   set.insert(z, active) -> bool   per lane (false when !active)
//   sink.take(b[], v[])             warp-collective once per group: b[u] is
//                                   the ballot of first insertions of step u;
//                                   v[u] is the lane's z value when the sink
//                                   asks for values (Sink::kValues), loaded
//                                   together with the z id to hide latency
// One 32-entry chunk of R entries: per lane its S segment over tiles
// [t0, t1) (start, length), the warp's inclusive / exclusive prefixes of the
// lengths and the chunk's candidate total.
struct Chunk {
    uint32_t s0, len, incl, excl, total;
};

__device__ __forceinline__ Chunk load_chunk(const RowCtx& c, uint32_t eb, uint32_t e1, uint32_t t0, uint32_t t1,
                                            uint64_t pol) {
    Chunk ch;
    const uint32_t e = eb + lane_id();
    ch.s0 = 0;
    ch.len = 0;
    if (e < e1) {
        const uint32_t y = ld_keep(&c.IC_R[e], pol);
        const uint64_t r = (uint64_t)y * c.T;
        ch.s0 = ld_keep(&c.JR_S[r + t0], pol);
        ch.len = ld_keep(&c.JR_S[r + t1], pol) - ch.s0;
    }
    ch.incl = warp_incl_scan(ch.len);
    if (__any_sync(0xffffffffu, ch.incl < ch.len)) raise_error(c.err, kErrCountRange);
    ch.total = __shfl_sync(0xffffffffu, ch.incl, 31);
    ch.excl = ch.incl - ch.len;
    return ch;
}

// Candidates [p0, p1) of a chunk through the set into the sink (the calling
// warp).  Many short segments: gather across segment boundaries -- each lane
// finds the segment of its candidate (the number of lanes with incl <= c;
// incl is nondecreasing over lanes) by a 5-step binary search over the
// lanes' prefixes, so one group of kUnroll x 32 loads covers many segments
// with a single memory latency.  Long segments: the lanes stride each
// segment overlapping the piece, kUnroll x 32 candidates at a time, all
// loads of a group issued first.
// One candidate's z id (and z value when the sink asks for values): a pair
// load from ISV, or the id and value arrays.
template <bool kPair, bool kValues>
__device__ __forceinline__ void load_cand(const RowCtx& c, uint32_t j, bool act, uint64_t pol, uint32_t& z,
                                          uint32_t& v) {
    if (kPair && kValues) {
        const uint2 p = act ? ld_keep2(&c.ISV[j], pol) : make_uint2(kEmpty32, 0u);
        z = p.x;
        v = p.y;
    } else {
        z = act ? ld_keep(&c.IC_S[j], pol) : kEmpty32;
        if (kValues) v = act ? ld_keep(&c.VS[j], pol) : 0u;
    }
}

template <bool kPair, class Set, class Sink>
__device__ __forceinline__ void expand_piece_impl(const RowCtx& c, const Chunk& ch, uint32_t p0, uint32_t p1,
                                                  Set& set, Sink& sink, uint64_t pol) {
    const uint32_t lane = lane_id();
    const uint32_t nseg = __popc(__ballot_sync(0xffffffffu, ch.len != 0));
    if (ch.total < (c.flat_avg ? c.flat_avg : kFlatAvgMax) * nseg) {
        for (uint32_t cb = p0; cb < p1; cb += 32 * kUnroll) {
            uint32_t z[kUnroll], v[kUnroll];
#pragma unroll
            for (uint32_t u = 0; u < kUnroll; u++) {
                const uint32_t cc = cb + u * 32 + lane;
                const bool act = cc < p1;
                const uint32_t ci = act ? cc : p0;  // idle lanes search a valid index
                uint32_t k = 0;
#pragma unroll
                for (uint32_t step = 16; step >= 1; step >>= 1)
                    if (__shfl_sync(0xffffffffu, ch.incl, k + step - 1) <= ci) k += step;
                const uint32_t j = __shfl_sync(0xffffffffu, ch.s0, k) + (ci - __shfl_sync(0xffffffffu, ch.excl, k));
                load_cand<kPair, Sink::kValues>(c, j, act, pol, z[u], v[u]);
            }
            uint32_t b[kUnroll];
#pragma unroll
            for (uint32_t u = 0; u < kUnroll; u++)
                b[u] = (cb + u * 32 < p1) ? __ballot_sync(0xffffffffu, set.insert(z[u], z[u] != kEmpty32)) : 0u;
            sink.take(b, v);
        }
        return;
    }
    // first segment holding candidate p0: lanes with incl <= p0 form a prefix
    for (uint32_t k = __popc(__ballot_sync(0xffffffffu, ch.incl <= p0)); k < 32; k++) {
        const uint32_t kex = __shfl_sync(0xffffffffu, ch.excl, k);
        if (kex >= p1) break;
        const uint32_t klen = __shfl_sync(0xffffffffu, ch.len, k);
        const uint32_t ks0 = __shfl_sync(0xffffffffu, ch.s0, k);
        const uint32_t lo = (p0 > kex ? p0 - kex : 0);
        const uint32_t hi = (kex + klen < p1 ? klen : p1 - kex);
        uint32_t jb = lo;
        // full groups: kUnroll x 32 candidates, all loads issued first
        for (; jb + 32 * kUnroll <= hi; jb += 32 * kUnroll) {
            uint32_t z[kUnroll], v[kUnroll];
#pragma unroll
            for (uint32_t u = 0; u < kUnroll; u++) load_cand<kPair, Sink::kValues>(c, ks0 + jb + u * 32 + lane, true, pol, z[u], v[u]);
            uint32_t b[kUnroll];
#pragma unroll
            for (uint32_t u = 0; u < kUnroll; u++) b[u] = __ballot_sync(0xffffffffu, set.insert(z[u], true));
            sink.take(b, v);
        }
        // tail (< kUnroll x 32 left): all its loads issued together, so one
        // load latency per segment tail; steps past the end are skipped
        // warp-uniformly
        if (jb < hi) {
            uint32_t z[kUnroll], v[kUnroll];
#pragma unroll
            for (uint32_t u = 0; u < kUnroll; u++) {
                const uint32_t j = jb + u * 32 + lane;
                load_cand<kPair, Sink::kValues>(c, ks0 + j, j < hi, pol, z[u], v[u]);
            }
            uint32_t b[kUnroll];
#pragma unroll
            for (uint32_t u = 0; u < kUnroll; u++)
                b[u] = (jb + u * 32 < hi) ? __ballot_sync(0xffffffffu, set.insert(z[u], z[u] != kEmpty32)) : 0u;
            sink.take(b, v);
        }
    }
}

// Candidates [p0, p1) of a chunk: paired loads where the (z id, z value)
// pairs exist and the sink takes values.
template <class Set, class Sink>
__device__ __forceinline__ void expand_piece(const RowCtx& c, const Chunk& ch, uint32_t p0, uint32_t p1, Set& set,
                                             Sink& sink, uint64_t pol) {
    if (Sink::kValues && c.ISV != nullptr)
        expand_piece_impl<true>(c, ch, p0, p1, set, sink, pol);
    else
        expand_piece_impl<false>(c, ch, p0, p1, set, sink, pol);
}

// Warp-level expansion of the candidates of R entries [e0, e1) over S tiles
// [t0, t1).  Entries are taken 32 at a time; a warp prefix sum over their S
// segment lengths flattens the chunk's candidates into [0, total), which is
// cut into a power-of-two number (<= 2^nparts_lg) of contiguous pieces of at
// least kMinPiece candidates; the calling warp takes piece `part`.
//   set.insert(z, active) -> bool   per lane (false when !active)
//   sink.take(b[], v[])             warp-collective once per group: b[u] is
//                                   the ballot of first insertions of step u;
//                                   v[u] is the lane's z value when the sink
//                                   asks for values (Sink::kValues), loaded
//                                   together with the z id to hide latency
template <class Set, class Sink>
__device__ __forceinline__ void warp_expand(const RowCtx& c, uint32_t e0, uint32_t e1, uint32_t part,
                                            uint32_t nparts_lg, uint32_t t0, uint32_t t1, Set& set, Sink& sink) {
    const uint64_t pol = l2_keep_policy();
    for (uint32_t eb = e0; eb < e1; eb += 32) {
        const Chunk ch = load_chunk(c, eb, e1, t0, t1, pol);
        const uint32_t want = ch.total / kMinPiece;
        uint32_t np_lg = want <= 1 ? 0 : 31 - __clz(want);
        np_lg = np_lg > nparts_lg ? nparts_lg : np_lg;
        if (part >= (1u << np_lg)) continue;
        const uint32_t piece = (ch.total >> np_lg) + ((ch.total & ((1u << np_lg) - 1)) ? 1u : 0u);
        const uint32_t p0 = min(part * piece, ch.total);
        const uint32_t p1 = min(p0 + piece, ch.total);
        if (p0 < p1) expand_piece(c, ch, p0, p1, set, sink, pol);
    }
}

// Chunks a CTA defers to its cooperative phase (round-robin walk), and the
// staged segment table of the row-flattened and balanced walks (see
// cta_expand).
constexpr uint32_t kBigChunk = 4096, kBigCap = 64;
constexpr uint32_t kRowBlk = 1024;  // R entries staged at a time by the flattened / balanced walks
struct CtaChunks {
    uint32_t n;              // deferred chunks (may exceed kBigCap: the rest ran at once)
    uint32_t eb[kBigCap];
    union {
        struct {
            uint32_t s0[kRowBlk];    // segment start of each staged entry
            uint32_t incl[kRowBlk];  // flattened walk: inclusive prefix of the lengths; balanced walk: the lengths
        } seg;
        uint32_t bnd[2 * kRowBlk];   // a row's entries' S row bounds over all z tiles (bitmap rows)
    } st;
    uint32_t ctot[kRowBlk / 32];  // balanced walk: candidates of each staged 32-entry chunk
};

// Row-flattened CTA walk over R entries [e0, e1) and S tiles [t0, t1): the
// CTA stages kRowBlk entries' segment bounds in shared memory at once (one
// load latency for the whole block instead of one per 32-entry chunk),
// scans their lengths CTA-wide and splits the block's candidates evenly
// over the warps; each lane finds its candidate's segment by binary search
// in the staged prefixes.  Contains barriers; called by the whole CTA.
template <class Set, class Sink>
__device__ __forceinline__ void cta_expand_flat(const RowCtx& c, uint32_t e0, uint32_t e1, uint32_t t0, uint32_t t1,
                                                Set& set, Sink& sink, CtaChunks* cc) {
    const uint32_t tid = threadIdx.x, lane = lane_id(), wib = tid >> 5, nw = blockDim.x >> 5;
    const uint32_t per = (kRowBlk + blockDim.x - 1) / blockDim.x;  // entries per thread (<= 4)
    const uint64_t pol = l2_keep_policy();
    __shared__ uint32_t sm_scan[1024 / 32 + 1];
    for (uint32_t eb = e0; eb < e1; eb += kRowBlk) {
        const uint32_t ne = min(kRowBlk, e1 - eb);
        // stage: thread tid owns entries [tid*per, tid*per + per)
        uint32_t s0[4], len[4], sum = 0;
#pragma unroll
        for (uint32_t k = 0; k < 4; k++) {
            s0[k] = 0;
            len[k] = 0;
            const uint32_t i = tid * per + k;
            if (k < per && i < ne) {
                const uint32_t y = ld_keep(&c.IC_R[eb + i], pol);
                const uint64_t r = (uint64_t)y * c.T;
                s0[k] = ld_keep(&c.JR_S[r + t0], pol);
                len[k] = ld_keep(&c.JR_S[r + t1], pol) - s0[k];
                sum += len[k];
            }
        }
        // CTA-wide exclusive scan of the threads' sums (blockDim <= 1024)
        const uint32_t inc = warp_incl_scan(sum);
        if (lane == 31) sm_scan[wib] = inc;
        __syncthreads();
        if (wib == 0) {
            const uint32_t v = lane < nw ? sm_scan[lane] : 0u;
            const uint32_t vi = warp_incl_scan(v);
            if (lane < nw) sm_scan[lane] = vi - v;
            if (lane == nw - 1) sm_scan[nw] = vi;
        }
        __syncthreads();
        uint32_t run = sm_scan[wib] + inc - sum;
        if (sm_scan[nw] < run) raise_error(c.err, kErrCountRange);  // 32-bit prefix wrapped
#pragma unroll
        for (uint32_t k = 0; k < 4; k++) {
            const uint32_t i = tid * per + k;
            if (k < per && i < ne) {
                run += len[k];
                cc->st.seg.s0[i] = s0[k];
                cc->st.seg.incl[i] = run;
            }
        }
        const uint32_t total = sm_scan[nw];
        __syncthreads();
        // the warps' even shares of the block's candidates
        const uint32_t piece = (total + nw - 1) / nw;
        const uint32_t p0 = min(wib * piece, total), p1 = min(p0 + piece, total);
        for (uint32_t cb = p0; cb < p1; cb += 32 * kUnroll) {
            uint32_t z[kUnroll], v[kUnroll];
#pragma unroll
            for (uint32_t u = 0; u < kUnroll; u++) {
                const uint32_t ci = cb + u * 32 + lane;
                const bool act = ci < p1;
                // first staged entry with incl > ci
                uint32_t lo = 0, hi = ne - 1;
                while (lo < hi) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (cc->st.seg.incl[mid] > ci) hi = mid;
                    else lo = mid + 1;
                }
                const uint32_t excl = lo ? cc->st.seg.incl[lo - 1] : 0u;
                const uint32_t j = cc->st.seg.s0[lo] + (ci - excl);
                if (Sink::kValues && c.ISV != nullptr)
                    load_cand<true, true>(c, j, act, pol, z[u], v[u]);
                else
                    load_cand<false, Sink::kValues>(c, j, act, pol, z[u], v[u]);
            }
            uint32_t b[kUnroll];
#pragma unroll
            for (uint32_t u = 0; u < kUnroll; u++)
                b[u] = (cb + u * 32 < p1) ? __ballot_sync(0xffffffffu, set.insert(z[u], z[u] != kEmpty32)) : 0u;
            sink.take(b, v);
        }
        __syncthreads();  // the staged table is rewritten by the next block
    }
}

// Balanced walk, staging half: the warps stage the segments of R entries
// [eb, eb + ne) (ne <= kRowBlk) over S tiles [t0, t1) in shared memory, each
// warp loading whole 32-entry chunks (every entry is loaded once), with each
// chunk's candidate total.  No barrier; the expanding half follows one.
// (wib, nw): this warp's index among the nw warps that share the work.
__device__ __forceinline__ void balanced_stage(const RowCtx& c, uint32_t eb, uint32_t ne, uint32_t t0, uint32_t t1,
                                               CtaChunks* cc, uint64_t pol, uint32_t wib, uint32_t nw) {
    const uint32_t lane = lane_id();
    const uint32_t nch = (ne + 31) >> 5;
    for (uint32_t k = wib; k < nch; k += nw) {
        const uint32_t i = k * 32 + lane, e = eb + i;
        uint32_t s0 = 0, len = 0;
        if (i < ne) {
            const uint32_t y = ld_keep(&c.IC_R[e], pol);
            const uint64_t r = (uint64_t)y * c.T;
            s0 = ld_keep(&c.JR_S[r + t0], pol);
            len = ld_keep(&c.JR_S[r + t1], pol) - s0;
        }
        cc->st.seg.s0[i] = s0;
        cc->st.seg.incl[i] = len;
        const uint32_t inc = warp_incl_scan(len);
        if (__any_sync(0xffffffffu, inc < len)) raise_error(c.err, kErrCountRange);  // 32-bit prefix wrapped
        if (lane == 31) cc->ctot[k] = inc;
    }
}

// Balanced walk, expanding half: every warp takes an equal share of the
// staged block's candidates -- the chunks overlapping its share, each through
// expand_piece with the chunk rebuilt from shared memory -- so no warp idles
// at the next barrier while another expands a long chunk alone.  No barrier.
// s0 / len / ctot: the staged segment starts and lengths and the chunk
// totals (a CtaChunks' arrays, or a prefetched row's).
// dyn (optional, zeroed before the barrier that precedes this): a shared
// counter from which the warps take pieces of dyn_piece candidates instead
// of equal static shares.
template <class Set, class Sink>
__device__ __forceinline__ void balanced_expand(const RowCtx& c, uint32_t ne, Set& set, Sink& sink,
                                                const uint32_t* s0a, const uint32_t* lena, const uint32_t* ctota,
                                                uint64_t pol, uint32_t wib, uint32_t nw, uint32_t* dyn = nullptr,
                                                uint32_t dyn_piece = 0) {
    const uint32_t lane = lane_id();
    const uint32_t nch = (ne + 31) >> 5;
    // prefix of the chunk totals (every warp computes it; nch <= 32)
    const uint32_t v = lane < nch ? ctota[lane] : 0u;
    const uint32_t inc = warp_incl_scan(v);
    if (__any_sync(0xffffffffu, inc < v)) raise_error(c.err, kErrCountRange);
    const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
    const uint32_t piece = dyn ? dyn_piece : total / nw + (total % nw ? 1u : 0u);
    for (uint32_t round = 0;; round++) {
    uint32_t p0;
    if (dyn) {
        p0 = 0;
        if (lane == 0) p0 = atomicAdd(dyn, piece);
        p0 = __shfl_sync(0xffffffffu, p0, 0);
        if (p0 >= total) break;
    } else {
        if (round) break;
        p0 = min(wib * piece, total);
    }
    const uint32_t p1 = min(p0 + piece, total);
    // first chunk holding candidate p0: chunks with incl <= p0 form a prefix
    for (uint32_t k = __popc(__ballot_sync(0xffffffffu, lane < nch && inc <= p0)); p0 < p1 && k < nch; k++) {
        const uint32_t cin = __shfl_sync(0xffffffffu, inc, k), ctot = __shfl_sync(0xffffffffu, v, k);
        const uint32_t cex = cin - ctot;
        if (cex >= p1) break;
        if (ctot == 0) continue;
        Chunk ch;
        ch.s0 = s0a[k * 32 + lane];
        ch.len = lena[k * 32 + lane];
        ch.incl = warp_incl_scan(ch.len);
        ch.excl = ch.incl - ch.len;
        ch.total = ctot;
        const uint32_t lo = p0 > cex ? p0 - cex : 0u, hi = p1 < cin ? p1 - cex : ctot;
        expand_piece(c, ch, lo, hi, set, sink, pol);
    }
    }
}

// Balanced CTA walk over R entries [e0, e1) and S tiles [t0, t1), kRowBlk
// entries at a time.  Contains barriers; called by the whole CTA.
template <class Set, class Sink>
__device__ __forceinline__ void cta_expand_balanced(const RowCtx& c, uint32_t e0, uint32_t e1, uint32_t t0,
                                                    uint32_t t1, Set& set, Sink& sink, CtaChunks* cc) {
    const uint64_t pol = l2_keep_policy();
    const uint32_t wib = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (uint32_t eb = e0; eb < e1; eb += kRowBlk) {
        const uint32_t ne = min(kRowBlk, e1 - eb);
        balanced_stage(c, eb, ne, t0, t1, cc, pol, wib, nw);
        __syncthreads();
        balanced_expand(c, ne, set, sink, cc->st.seg.s0, cc->st.seg.incl, cc->ctot, pol, wib, nw);
        __syncthreads();  // the staged table is rewritten by the next block
    }
}

// CTA-level expansion of R entries [e0, e1) over S tiles [t0, t1), called
// by all warps of the CTA (2^nw_lg of them) with the same arguments.
// c.cta_rr selects the walk: 3 the balanced walk (cta_expand_balanced),
// 0 the row-flattened walk (cta_expand_flat),
// 2 every chunk split across the warps (warp_expand), 1 with at least as
// many chunks as warps, each warp takes whole
// chunks round-robin -- a chunk's entries and segment bounds are loaded by
// one warp, not by every warp -- and chunks of more than kBigChunk
// candidates are deferred and then split across all warps.  Otherwise every
// chunk is split across the warps (warp_expand).  Which is faster depends on
// the workload (the autotuner times both).  cc->n must be 0
// on entry (it is 0 again on return); contains barriers.
template <class Set, class Sink>
__device__ __forceinline__ void cta_expand(const RowCtx& c, uint32_t e0, uint32_t e1, uint32_t wib, uint32_t nw_lg,
                                           uint32_t t0, uint32_t t1, Set& set, Sink& sink, CtaChunks* cc) {
    const uint32_t nchunks = (e1 - e0 + 31) >> 5;
    if (c.cta_rr == 3) {
        cta_expand_balanced(c, e0, e1, t0, t1, set, sink, cc);
        return;
    }
    if (c.cta_rr == 0) {
        cta_expand_flat(c, e0, e1, t0, t1, set, sink, cc);
        return;
    }
    if (c.cta_rr == 2 || nchunks < (1u << nw_lg)) {
        warp_expand(c, e0, e1, wib, nw_lg, t0, t1, set, sink);
        return;
    }
    const uint64_t pol = l2_keep_policy();
    for (uint32_t ci = wib; ci < nchunks; ci += 1u << nw_lg) {
        const uint32_t eb = e0 + 32 * ci;
        const Chunk ch = load_chunk(c, eb, e1, t0, t1, pol);
        if (ch.total > kBigChunk) {
            uint32_t slot = 0;
            if (lane_id() == 0) slot = atomicAdd(&cc->n, 1u);
            slot = __shfl_sync(0xffffffffu, slot, 0);
            if (slot < kBigCap) {
                if (lane_id() == 0) cc->eb[slot] = eb;
                continue;
            }
        }
        if (ch.total) expand_piece(c, ch, 0, ch.total, set, sink, pol);
    }
    __syncthreads();
    const uint32_t nbig = min(cc->n, kBigCap);
    for (uint32_t i = 0; i < nbig; i++) {
        const uint32_t eb = cc->eb[i];
        warp_expand(c, eb, min(eb + 32, e1), wib, nw_lg, t0, t1, set, sink);
    }
    __syncthreads();
    if (threadIdx.x == 0) cc->n = 0;
}

// ----------------------------------------------------------------- sets
struct HashSet {
    uint32_t* tab;
    uint32_t lg;
    uint32_t* err;
    __device__ __forceinline__ bool insert(uint32_t z, bool act) { return act ? smem_set_insert(tab, lg, z, err) : false; }
};

// Bitmap over one z tile; branch-free (idle lanes OR a zero into words
// 0..31, so the bitmap allocation is at least 32 words).
struct TileBitmap {
    uint32_t* bm;
    uint32_t lo;
    __device__ __forceinline__ bool insert(uint32_t z, bool act) {
        const uint32_t zl = z - lo;
        const uint32_t w = act ? (zl >> 5) : lane_id();
        const uint32_t bit = act ? (1u << (zl & 31)) : 0u;
        return (atomicOr(&bm[w], bit) & bit) == 0 && act;
    }
};

// ---------------------------------------------------------------- sinks
struct CountSink {
    static constexpr bool kValues = false;
    uint32_t count = 0;
    template <uint32_t N>
    __device__ __forceinline__ void take(const uint32_t (&b)[N], const uint32_t (&)[N]) {
#pragma unroll
        for (uint32_t u = 0; u < N; u++) count += __popc(b[u]);
    }
};

// Emits first insertions at base + a row-local slot.  shared_pos == nullptr:
// the warp owns the row and counts locally; otherwise one shared-memory claim
// per group reserves the slots.
struct WriteSink {
    static constexpr bool kValues = true;
    uint2* out;
    uint32_t* err;
    unsigned long long base;
    uint32_t lim, xv;
    uint32_t* shared_pos;
    uint32_t local = 0;
    template <uint32_t N>
    __device__ __forceinline__ void take(const uint32_t (&b)[N], const uint32_t (&v)[N]) {
        uint32_t n = 0;
#pragma unroll
        for (uint32_t u = 0; u < N; u++) n += __popc(b[u]);
        if (n == 0) return;
        uint32_t pb;
        if (shared_pos) {
            pb = 0;
            if (lane_id() == 0) pb = atomicAdd(shared_pos, n);
            pb = __shfl_sync(0xffffffffu, pb, 0);
        } else {
            pb = local;
            local += n;
        }
        const uint32_t lt = lanemask_lt();
#pragma unroll
        for (uint32_t u = 0; u < N; u++) {
            if (b[u] & (1u << lane_id())) {
                const uint32_t pos = pb + __popc(b[u] & lt);
                if (pos < lim) st_stream(&out[base + pos], make_uint2(xv, v[u]));
                else raise_error(err, kErrOutputBound);
            }
            pb += __popc(b[u]);
        }
    }
};

// Next row of a CTA class, taken dynamically (the whole CTA gets the index).
__device__ __forceinline__ uint32_t cta_next_row(uint32_t* counter, uint32_t* s_row) {
    __syncthreads();
    if (threadIdx.x == 0) *s_row = atomicAdd(counter, 1u);
    __syncthreads();
    return *s_row;
}

// Class 1: one warp per row, 2^warp_lg slots per warp.
template <bool WRITE>
static __global__ void __launch_bounds__(256) k_rows_warp(RowCtx c, const uint32_t* __restrict__ rows,
                                                   const unsigned long long* __restrict__ nrows_p, uint32_t warp_lg) {
    extern __shared__ uint32_t smem[];
    const uint32_t nw = blockDim.x >> 5, wib = threadIdx.x >> 5, lane = lane_id();
    uint32_t* tab = smem + ((size_t)wib << warp_lg);
    const uint32_t nrows = (uint32_t)*nrows_p;
    for (uint32_t ri = blockIdx.x * nw + wib; ri < nrows; ri += gridDim.x * nw) {
        const uint32_t x = rows[ri];
        const uint32_t u = c.ucap[x];
        const bool bm = use_row_bitmap(c.m, u, warp_lg);
        uint32_t lg = ceil_log2(2 * u);
        lg = lg < 5 ? 5 : (lg > warp_lg ? warp_lg : lg);
        const uint32_t nclr = bm ? row_bitmap_words(c.m) : (1u << lg);
        const uint32_t fill = bm ? 0u : kEmpty32;
        for (uint32_t s = lane; s < nclr; s += 32) tab[s] = fill;
        __syncwarp();
        WriteSink wsink{c.out, c.err, 0, 0, 0, nullptr};
        CountSink csink;
        if (WRITE) {
            wsink.base = c.off[x];
            wsink.lim = c.cnt[x];
            wsink.xv = c.id2x[x];
        }
        if (bm) {
            TileBitmap set{tab, 0};
            if (WRITE) warp_expand(c, c.JR_R[x], c.JR_R[x + 1], 0, 0, 0, c.T, set, wsink);
            else warp_expand(c, c.JR_R[x], c.JR_R[x + 1], 0, 0, 0, c.T, set, csink);
        } else {
            HashSet set{tab, lg, c.err};
            if (WRITE) warp_expand(c, c.JR_R[x], c.JR_R[x + 1], 0, 0, 0, c.T, set, wsink);
            else warp_expand(c, c.JR_R[x], c.JR_R[x + 1], 0, 0, 0, c.T, set, csink);
        }
        if (!WRITE && lane == 0) c.cnt[x] = csink.count;
        __syncwarp();
    }
}

// Class 2: one CTA per row, 2^block_lg slots.
template <bool WRITE>
static __global__ void __launch_bounds__(1024) k_rows_block(RowCtx c, const uint32_t* __restrict__ rows,
                                                    const unsigned long long* __restrict__ nrows_p, uint32_t block_lg) {
    extern __shared__ uint32_t smem[];
    __shared__ uint32_t s_count, s_row;
    const uint32_t wib = threadIdx.x >> 5, lane = lane_id();
    const uint32_t nw_lg = 31 - __clz(blockDim.x >> 5);
    const uint32_t nrows = (uint32_t)*nrows_p;
    for (uint32_t ri = cta_next_row(&c.next_row[2], &s_row); ri < nrows; ri = cta_next_row(&c.next_row[2], &s_row)) {
        const uint32_t x = rows[ri];
        const uint32_t u = c.ucap[x];
        const bool bm = use_row_bitmap(c.m, u, block_lg);
        uint32_t lg = ceil_log2(2 * u);
        lg = lg < 5 ? 5 : (lg > block_lg ? block_lg : lg);
        const uint32_t fill = bm ? 0u : kEmpty32;
        const uint32_t n4 = (bm ? row_bitmap_words(c.m) : (1u << lg)) / 4;
        uint4* t4 = reinterpret_cast<uint4*>(smem);
        for (uint32_t s = threadIdx.x; s < n4; s += blockDim.x) t4[s] = make_uint4(fill, fill, fill, fill);
        if (threadIdx.x == 0) s_count = 0;
        __syncthreads();
        WriteSink wsink{c.out, c.err, 0, 0, 0, &s_count};
        CountSink csink;
        if (WRITE) {
            wsink.base = c.off[x];
            wsink.lim = c.cnt[x];
            wsink.xv = c.id2x[x];
        }
        if (bm) {
            TileBitmap set{smem, 0};
            if (WRITE) warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, 0, c.T, set, wsink);
            else warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, 0, c.T, set, csink);
        } else {
            HashSet set{smem, lg, c.err};
            if (WRITE) warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, 0, c.T, set, wsink);
            else warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, 0, c.T, set, csink);
        }
        if (!WRITE && lane == 0 && csink.count) atomicAdd(&s_count, csink.count);
        __syncthreads();
        if (!WRITE && threadIdx.x == 0) c.cnt[x] = s_count;
    }
}

// Classes 3 and 4: one CTA per row, a bitmap over one z tile at a time.  The
// row list holds the class-4 rows first; nrows = *n4 + *n3.
template <bool WRITE>
static __global__ void __launch_bounds__(1024) k_rows_bitmap(RowCtx c, const uint32_t* __restrict__ rows,
                                                      const unsigned long long* __restrict__ n3,
                                                      const unsigned long long* __restrict__ n4) {
    extern __shared__ uint32_t bm[];
    __shared__ uint32_t s_count, s_row;
    const uint32_t wib = threadIdx.x >> 5, lane = lane_id();
    const uint32_t nw_lg = 31 - __clz(blockDim.x >> 5);
    const uint32_t nrows = (uint32_t)(*n3 + *n4);
    for (uint32_t ri = cta_next_row(&c.next_row[3], &s_row); ri < nrows; ri = cta_next_row(&c.next_row[3], &s_row)) {
        const uint32_t x = rows[ri];
        if (threadIdx.x == 0) s_count = 0;
        WriteSink wsink{c.out, c.err, 0, 0, 0, &s_count};
        if (WRITE) {
            wsink.base = c.off[x];
            wsink.lim = c.cnt[x];
            wsink.xv = c.id2x[x];
        }
        CountSink csink;
        for (uint32_t t = 0; t < c.T; t++) {
            const uint32_t lo = t * c.tile_width;
            const uint32_t width = min(c.tile_width, c.m - lo);
            const uint32_t words4 = (((width + 31) >> 5) + 3) >> 2;
            uint4* b4 = reinterpret_cast<uint4*>(bm);
            for (uint32_t w = threadIdx.x; w < words4; w += blockDim.x) b4[w] = make_uint4(0, 0, 0, 0);
            __syncthreads();
            TileBitmap set{bm, lo};
            if (WRITE) warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, t, t + 1, set, wsink);
            else warp_expand(c, c.JR_R[x], c.JR_R[x + 1], wib, nw_lg, t, t + 1, set, csink);
            __syncthreads();
        }
        if (!WRITE) {
            if (lane == 0 && csink.count) atomicAdd(&s_count, csink.count);
            __syncthreads();
            if (threadIdx.x == 0) c.cnt[x] = s_count;
        }
    }
}

// Per-row candidate count w = sum over y in R_x of |S_y|, u = min(w, m) and
// the row class (0: empty, or outside sel's A-tiles).  One warp per row.  With check_range set
// (join-aggregate, 32-bit per-group counters) a row of 2^32 or more
// candidates raises kErrCountRange.
static __global__ void k_row_work(RowCtx c, uint32_t n, uint32_t cap_w, uint32_t cap_b, bool check_range, bool tiny, SumAcc sel,
                           uint32_t* __restrict__ ucap, uint8_t* __restrict__ cls, unsigned long long* outj,
                           unsigned long long* outj_cls) {
    const uint32_t lane = lane_id();
    const uint64_t gw = ((uint64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t nwarps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    unsigned long long acc = 0, acc_cls[6] = {0, 0, 0, 0, 0, 0};
    for (uint64_t x = gw; x < n; x += nwarps) {
        if (sel.tiles && !sel.selected(c.id2x[x])) {  // summaries over a slice of A-tiles
            if (lane == 0) {
                ucap[x] = 0;
                cls[x] = 0;
            }
            continue;
        }
        uint32_t e0 = c.JR_R[x], e1 = c.JR_R[x + 1];
        unsigned long long w = 0;
        for (uint32_t e = e0 + lane; e < e1; e += 32) {
            uint64_t r = (uint64_t)c.IC_R[e] * c.T;
            w += c.JR_S[r + c.T] - c.JR_S[r];
        }
        w = warp_sum(w);
        if (lane == 0) {
            uint32_t u = (uint32_t)(w < c.m ? w : c.m);
            ucap[x] = u;
            const uint32_t k = row_class(w, u, cap_w, cap_b, tiny);
            cls[x] = (uint8_t)k;
            if (check_range && w >= 0xFFFFFFFFull) raise_error(c.err, kErrCountRange);
            acc += w;
#pragma unroll
            for (uint32_t j = 1; j < 6; j++) acc_cls[j] += (j == k) ? w : 0ull;
        }
    }
    if (lane == 0 && acc) {
        atomicAdd(outj, acc);
#pragma unroll
        for (uint32_t j = 1; j < 6; j++)
            if (acc_cls[j]) atomicAdd(&outj_cls[j], acc_cls[j]);
    }
}

struct ClassSrc {
    const uint8_t* cls;
    uint8_t want;
    __device__ uint64_t operator()(uint64_t i) const { return cls[i] == want ? 1u : 0u; }
};
// Block-class (class 2) rows whose distinct bound u is in (lo, hi].
struct BlockSizeSrc {
    const uint8_t* cls;
    const uint32_t* ucap;
    uint32_t lo, hi;
    __device__ uint64_t operator()(uint64_t i) const {
        return cls[i] == 2 && ucap[i] > lo && ucap[i] <= hi ? 1u : 0u;
    }
};
// list[*base + *base2 + rank] = row (bases: counts of rows placed before
// this class; either may be null).
struct ListDst {
    uint32_t* list;
    const unsigned long long* base;
    const unsigned long long* base2 = nullptr;
    __device__ void operator()(uint64_t i, uint64_t e, uint64_t v) const {
        if (v) list[(base ? *base : 0) + (base2 ? *base2 : 0) + e] = (uint32_t)i;
    }
};
struct OffDst {
    unsigned long long* off;
    __device__ void operator()(uint64_t i, uint64_t e, uint64_t) const { off[i] = e; }
};

}  // namespace dim3g

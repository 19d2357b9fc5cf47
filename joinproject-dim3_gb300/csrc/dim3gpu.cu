// dim3gpu.cu -- host orchestration and C ABI of the GB300 join-project path.
//
// One call runs, on the context's stream:
//   mapping   hash build on P (first column, y), semi-join probe of Q with z
//             insertion, dense ids by prefix sums over occupied slots
//             (replaces mapping_step + LS_mapper, dim3.hpp:394-883)
//   CSR       R by x id, S by (y id, z tile) (divide_R / divide_S,
//             dim3.hpp:1058-1259), per-row work and row binning
//   count     per-row distinct counts, prefix sum to output offsets
//   write     the same expansion emitting (x value, z value) pairs
// (Hybrid_solution, dim3.hpp:889-974).  Two host synchronisations: one for
// the id domain sizes, one for the output size.
#include <cuda_runtime.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/dim3gpu.h"
#include "aggregate.cuh"
#include "internal.h"
#include "common.cuh"
#include "dense.cuh"
#include "expand.cuh"
#include "mapper.cuh"
#include "mapping.cuh"
#include "scan.cuh"
#include "single.cuh"
#include "stream.cuh"
#include "prefetch.cuh"

using namespace dim3g;

namespace {

// ------------------------------------------------------------ workspace
// Grow-only list of device blocks with a bump pointer each; reset at the
// start of every call, so repeated calls of the same shape reuse the same
// addresses and never allocate.
struct Arena {
    struct Block {
        char* p;
        size_t size, used;
    };
    std::vector<Block> blocks;
    void reset() {
        for (auto& b : blocks) b.used = 0;
    }
    void* alloc(size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        if (bytes == 0) bytes = 256;
        for (auto& b : blocks)
            if (b.size - b.used >= bytes) {
                void* r = b.p + b.used;
                b.used += bytes;
                return r;
            }
        size_t sz = bytes < ((size_t)256 << 20) ? ((size_t)256 << 20) : bytes;
        char* p = nullptr;
        if (cudaMalloc(&p, sz) != cudaSuccess) {
            cudaGetLastError();
            return nullptr;
        }
        blocks.push_back({p, sz, bytes});
        return p;
    }
    void release() {
        for (auto& b : blocks) cudaFree(b.p);
        blocks.clear();
    }
};

// Rates of the dense block's cost model (run_dense).
struct CostModel {
    double tile_s = 0.8e-6;              // fixed time of one product tile (TMA fill, epilogue)
    double sm_flops = 3.8e15 / 152;      // product rate of one SM
    double dense_bw = 6.0e12;            // bitmap and light-pass streaming, bytes/s
    double sparse_bw = 5.0e12;           // sparse expansion, 4 algorithmic bytes a candidate
    bool calibrated = false;             // product rates and bandwidth measured on this device
};

struct Params {
    uint32_t warp_lg = 11;    // 2048 slots per warp set  -> class 1 up to 1024
    uint32_t block_lg = 14;   // 16384 slots per CTA set  -> class 2 up to 8192
    uint32_t block_threads = 512;  // CTA width of the class-2 kernels
    uint32_t tile_lg = 19;    // 2^19-bit z tiles (64 KB bitmap)
    bool ordered = false;     // two-pass, rows in x-id order
    bool host_direct = true;  // pinned host outputs are written by the kernels directly
    uint32_t cta_rr = 3;      // CTA rows' walk: 0 flattened, 1 chunks round-robin, 2 chunks split, 3 balanced
    uint32_t dense = 1;       // dense block on the tensor cores: 0 off, 1 by cost model, 2 whenever it fits
    uint32_t dense_k_max = 2048;  // most join values in the dense product
    uint64_t dense_mem = (uint64_t)16 << 30;  // bitmap bytes of the dense block
    bool keep_roles = false;  // R drives the join whatever the sizes (no swap)
    bool sized_tables = true;  // mapping tables sized by a distinct-key sketch (mapping.cuh)
    uint32_t table_slack_pct = 150;  // sketch-sized table slots per estimated distinct key, percent
    uint32_t stream_rows = 0;  // single pass: bitmap-class rows streamed by TMA (stream.cuh)
    uint32_t prefetch_rows = 0;  // single pass, balanced walk: block-class rows fetched ahead (prefetch.cuh)
    uint32_t block_split = 1;    // single pass: block-class rows in three launches by hash-set size
};

constexpr size_t kMaxSmemOptin = 227 * 1024;  // dynamic shared memory a CTA may opt into
constexpr uint32_t kFlatAvgBitmap = 160, kFlatAvgBlock = 560, kFlatAvgWarp = 160;  // single pass, per row class
constexpr uint32_t kAggTileLg = 15;  // join-aggregate class-3 tile: 32K counters (128 KB)

struct Scalars {
    unsigned long long nx, ny, nz, nkept, total, outj;
    unsigned long long cursor;     // single-pass output cursor
    unsigned long long nrows[6];   // rows per class (index = class)
    unsigned long long outj_cls[6];  // candidates per class (index = class)
    unsigned long long cursor_at[3]; // single-pass cursor after the bitmap / block / warp kernel
    unsigned long long dense_base;   // single-pass start of the dense block's pairs (~0: past the capacity)
    unsigned int err;
    unsigned long long nrows_b[3];  // block-class rows by hash-set size (single pass, block_split)
    unsigned int next_row[8];      // dynamic row counters of the CTA classes (4..6: block_split launches)
    unsigned int pad;
};

}  // namespace

struct dim3g_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;
    Arena ws;
    Params prm;
    CostModel cm;
    dim3g_stats stats{};
    // host-API staging (device) buffers, grow-only
    void* d_in = nullptr;
    size_t d_in_bytes = 0;
    void* d_out = nullptr;
    size_t d_out_bytes = 0;
    void* d_sum = nullptr;  // per-A-tile summary accumulators
    size_t d_sum_bytes = 0;
    Scalars* h_sc = nullptr;  // pinned
    cudaStream_t aux = nullptr;  // side stream: R's CSR build alongside S's (fork/join by events)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    cudaEvent_t ev[6] = {};
    cudaEvent_t evc[8] = {};  // per row-class kernel timing
    cudaEvent_t evd[4] = {};  // dense block: selection, operands, product, light pass
    uint64_t launches = 0;  // kernels launched on this context since creation
};

struct dim3g_mapper {
    dim3g_ctx* ctx;
    unsigned long long* slots = nullptr;
    uint64_t cap = 0;
    int64_t cnt = 0;
    int64_t nkeys = 0;
};

namespace {

int fail(dim3g_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}

#define CU(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) return fail(c, DIM3G_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define CHECK_LAUNCH()         \
    do {                       \
        CU(cudaGetLastError());\
        c->launches++;         \
    } while (0)

// device_scan plus launch accounting (three kernels when n > 0).
template <class Src, class Dst>
int run_scan(dim3g_ctx* c, Src src, Dst dst, uint64_t n, uint64_t* bsum, unsigned long long* total,
             cudaStream_t on = nullptr) {
    device_scan(src, dst, n, bsum, total, on ? on : c->stream);
    CU(cudaGetLastError());
    c->launches += scan_launches(n);
    return DIM3G_OK;
}
#define SCAN(...)                                \
    do {                                         \
        int r_ = run_scan(c, __VA_ARGS__);       \
        if (r_) return r_;                       \
    } while (0)


unsigned grid_for(uint64_t n, int sm, int per_sm = 8, int block = 256) {
    uint64_t b = (n + block - 1) / block;
    uint64_t cap = (uint64_t)sm * per_sm;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    return (unsigned)b;
}

template <class T>
T* ws_get(dim3g_ctx* c, uint64_t count) {
    return (T*)c->ws.alloc(count * sizeof(T));
}

// Where the write pass puts its result: called once the count pass knows the
// number of output pairs; returns the device buffers or an error status.
// peek() gives the current buffer and its capacity without growing it (the
// single pass writes into whatever is there and reports the size needed).
struct OutPrep {
    int (*fn)(dim3g_ctx* c, void* user, uint64_t total, uint2** out, unsigned long long** cnt);
    void (*peek)(dim3g_ctx* c, void* user, uint2** out, uint64_t* capacity);
    void* user;
};

// Device state of one join call.
struct JoinPlan {
    const uint2* P;
    uint64_t nP;
    const uint2* Q;
    uint64_t nQ;
    bool swapped;
    bool aggregate;   // COUNT(*) per group instead of distinct pairs
    bool count_only;  // stop after the count pass
    bool single_pass; // one expansion, rows reserve their output range
    OutPrep prep;
    SumAcc sum{nullptr, 0, 0, 0};  // tiles set: per-A-tile summaries, no output
};

bool set_aggregate_attributes();
struct RowLists {
    const uint32_t *w, *b, *m;                          // class 1, class 2, classes 4 then 3
    const unsigned long long *nw, *nb, *n3, *n4;        // their sizes (device)
};
int run_aggregate_write(dim3g_ctx* c, const RowCtx& rc, AggOut ao, const RowLists& L);

// Warps per CTA of a warp-per-row kernel whose warps each own per_warp
// bytes of shared memory: up to 8, within about half an SM's shared memory
// so two CTAs fit per SM.
constexpr size_t kWarpCtaSmem = 112 * 1024;
inline uint32_t warps_per_cta(size_t per_warp) {
    size_t w = kWarpCtaSmem / per_warp;
    return (uint32_t)(w < 1 ? 1 : (w > 8 ? 8 : w));
}

// Grid of a persistent / grid-stride kernel: resident CTAs per SM x SMs.
template <class K>
unsigned resident_grid(K kernel, int block, size_t smem, int sm) {
    int per = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, block, smem) != cudaSuccess || per < 1) {
        cudaGetLastError();
        per = 1;
    }
    return (unsigned)(per * sm);
}

// ------------------------------------------------------------ dense block
// The heavy rows' (bitmap classes') join through their heaviest join values
// as one boolean product on the tensor cores (dense.cuh).  Cost model, in
// seconds, against the bitmap-class expansion it replaces (4 algorithmic
// bytes per candidate):
//   product   tiles per SM x max(CostModel::tile_s, MMA time of a tile at
//             CostModel::sm_flops); the fixed part is a tile's TMA fill and
//             epilogue, which the MMAs hide from about Kp = 384 on
//   bitmap    written by the product, read by the light pass and emission
//   light     the candidates through the other join values, kLightBytes each
// The CostModel defaults were measured once on a GB300 (zipf_1m: 0.8 us a
// tile at Kp <= 256, about 3.8 PFLOP/s for Kp = 384 .. 1024; the light pass
// 3-6 ps a candidate); dim3g_calibrate replaces the product's rates and the
// bandwidth with ones measured on the context's device, and the autotuner's
// sparse trial the sparse rate.
// summary epilogue, measured on the 16M x 16M Zipf-1.2 COUNT: ~32K group
// hashes a tile (11.1 us) + 0.34 us per light candidate in the tile's bucket
constexpr double kDenseTileSumS = 11.1e-6;
constexpr double kDenseBucketS = 0.34e-6;
constexpr double kLightBytes = 40.0;
constexpr uint64_t kDenseMinCand = (uint64_t)1 << 26;  // smaller heavy work stays sparse (cost model mode)

struct DensePlan {
    bool on = false;
    uint32_t nd = 0;      // rows of the block: list_m[0 .. nd) (the bitmap classes' rows, huge ones first)
    uint32_t Wd = 0;      // bitmap words per row (allocated)
    uint32_t Wm = 0;      // bitmap words per row holding z < m
    uint32_t cpr = 0;     // 32-word chunks per row
    const uint32_t* D = nullptr;
    const unsigned long long* coff = nullptr;  // nd * cpr + 1 chunk offsets (exclusive prefix of popcounts)
};

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
    static EncodeTiledFn fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess) {
            cudaGetLastError();
            return (EncodeTiledFn) nullptr;
        }
        return (EncodeTiledFn)p;
    }();
    return fn;
}

// 2-D byte tensor of `rows` rows of Kp bytes; boxes of 128 bytes x box_rows,
// 128-byte swizzle (the layout the product's descriptors expect).
int dense_map(dim3g_ctx* c, CUtensorMap* map, void* base, uint64_t rows, uint32_t Kp, uint32_t box_rows) {
    EncodeTiledFn fn = encode_tiled();
    if (!fn) return fail(c, DIM3G_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
    const cuuint64_t dims[2] = {Kp, rows};
    const cuuint64_t strides[1] = {Kp};
    const cuuint32_t box[2] = {kDenseBK, box_rows};
    const cuuint32_t es[2] = {1, 1};
    const CUresult r = fn(map, CU_TENSOR_MAP_DATA_TYPE_UINT8, 2, base, dims, strides, box, es,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(c, DIM3G_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    return DIM3G_OK;
}

uint64_t round_up(uint64_t v, uint64_t a) { return (v + a - 1) / a * a; }

// Decides on and runs the dense block for a prefix of list_m (as many of
// the bitmap classes' rows as the bitmap budget holds); on success with
// dp->on the bitmap holds those rows' distinct z, and the device counts of
// classes 3 and 4 add up to the rows left (list_m + nd onwards), which the
// bitmap-class kernels then take.
int run_dense(dim3g_ctx* c, const JoinPlan& jp, const RowCtx& rc, Scalars* sc, const uint32_t* list_m, uint32_t k,
              uint32_t m, DensePlan* dp) {
    *dp = DensePlan{};
    const uint32_t mode = c->prm.dense;
    // materialised COUNT output stays on the sparse kernels
    uint32_t& skip = c->stats.dense_skip;
    skip = 1;  // off, or materialised COUNT
    if (mode == 0 || (jp.aggregate && !jp.sum.tiles)) return DIM3G_OK;
    const int kind = !jp.sum.tiles ? kDenseBits : (jp.aggregate ? kDenseSumCount : kDenseSumProject);
    const bool bits = kind == kDenseBits;
    cudaStream_t st = c->stream;
    const int sm = c->sm_count;
    CU(cudaMemcpyAsync(c->h_sc, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (c->h_sc->err) return fail(c, DIM3G_ERR_DEVICE, "device bound violated in row binning (flags %u)", c->h_sc->err);
    const uint64_t n_heavy = c->h_sc->nrows[3] + c->h_sc->nrows[4];
    const uint64_t cd_all = c->h_sc->outj_cls[3] + c->h_sc->outj_cls[4];
    skip = 2;  // no heavy rows, or too little heavy work
    if (n_heavy == 0 || cd_all == 0) return DIM3G_OK;
    if (mode == 1 && cd_all < kDenseMinCand) return DIM3G_OK;
    skip = 3;  // the budget holds no row or no K
    const uint64_t Np = round_up(m, kDenseBN), Wd = Np / 32;
    // bitmap: the rows its budget holds, whole 128-row tiles; summaries keep
    // no bitmap and take every heavy row (their operand counts are bounded
    // by the same budget through K below)
    const uint64_t fit = bits ? c->prm.dense_mem / (Wd * 4) / kDenseBM * kDenseBM : n_heavy;
    const uint64_t nd = n_heavy < fit ? n_heavy : fit;
    if (nd == 0) return DIM3G_OK;
    const uint64_t Mp = round_up(nd, kDenseBM), dbytes = bits ? Mp * Wd * 4 : 0;
    uint64_t kmax = c->prm.dense_k_max;
    if (!bits) {
        // the product's tiles are indexed in 32 bits; their light-bucket
        // bounds take 12 B each out of the budget
        const uint64_t tiles = (Mp / kDenseBM) * (Np / kDenseBN);
        if (tiles >= (1ull << 31) || tiles * 12 >= c->prm.dense_mem) return DIM3G_OK;
        const uint64_t kfit = (c->prm.dense_mem - tiles * 12) / ((Mp + Np) * 4) / kDenseBK * kDenseBK;  // 32-bit counts
        if (kfit < kmax) kmax = kfit;
        if (kmax == 0) return DIM3G_OK;
    }
    const double t_bitmap = 3.0 * (double)dbytes / c->cm.dense_bw;
    const double ntile_all = (double)(Mp / kDenseBM) * (double)(Np / kDenseBN);
    const double tiles_per_sm = ceil(ntile_all / sm);
    const double tile_fixed = bits ? c->cm.tile_s : kDenseTileSumS;
    auto t_product = [&](uint64_t Kp, double light) {
        const double t_mma = 2.0 * kDenseBM * kDenseBN * (double)Kp / c->cm.sm_flops;
        // summaries also count the operands in 32 bits first, and every
        // epilogue thread scans its tile's light bucket
        const double t_ops = bits ? 0.0 : (double)(Mp + Np) * Kp * 9.0 / c->cm.dense_bw;
        const double t_epi = tile_fixed + (bits ? 0.0 : kDenseBucketS * light / ntile_all);
        return tiles_per_sm * (t_mma > t_epi ? t_mma : t_epi) + t_ops;
    };
    // light candidates: OR-ed into the bitmap, or counted and bucketed by tile
    const double light_bytes = bits ? kLightBytes : 2.0 * kLightBytes;
    const double t_min = t_product(kDenseBK, 0.0) + t_bitmap;
    // the sparse cost of all heavy rows bounds that of any prefix of them
    skip = 4;  // the cost model keeps the sparse path
    if (mode == 1 && t_min >= (double)cd_all * 4.0 / c->cm.sparse_bw) return DIM3G_OK;

    CU(cudaEventRecord(c->evd[0], st));
    uint32_t* degd = ws_get<uint32_t>(c, k);
    int32_t* hid = ws_get<int32_t>(c, k);
    uint32_t* hy = ws_get<uint32_t>(c, kmax);
    // bin_n[kDenseBins]: heavy-column counter, [+1]: multiplicity flag, [+2]: largest light bucket
    unsigned int* bin_n = ws_get<unsigned int>(c, kDenseBins + 3);
    unsigned long long* bin_mass = ws_get<unsigned long long>(c, kDenseBins + 1);  // [kDenseBins]: light total
    if (!degd || !hid || !hy || !bin_n || !bin_mass) return fail(c, DIM3G_ERR_NOMEM, "workspace allocation failed (dense)");
    CU(cudaMemsetAsync(degd, 0, (size_t)k * 4, st));
    CU(cudaMemsetAsync(bin_n, 0, (kDenseBins + 3) * 4, st));
    CU(cudaMemsetAsync(bin_mass, 0, (kDenseBins + 1) * 8, st));
    // a sample of about 8192 heavy rows estimates the join values' mass
    const uint32_t step = nd > 8192 ? (uint32_t)(nd / 8192) : 1u;
    k_dense_deg<<<grid_for((nd / step + 1) * 32, sm), 256, 0, st>>>(rc.JR_R, rc.IC_R, list_m, (uint32_t)nd, step, degd);
    CHECK_LAUNCH();
    k_dense_bins<<<grid_for(k, sm), 256, 0, st>>>(degd, rc.JR_S, rc.T, k, bin_n, bin_mass);
    CHECK_LAUNCH();
    std::vector<unsigned int> hn(kDenseBins);
    std::vector<unsigned long long> hm(kDenseBins);
    CU(cudaMemcpyAsync(hn.data(), bin_n, kDenseBins * 4, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(hm.data(), bin_mass, kDenseBins * 8, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    // the block's candidates: exact for all heavy rows, else the sample's;
    // the light candidates of a cut are the sample's mass below it
    double sampled = 0;
    for (uint32_t b = 0; b < kDenseBins; b++) sampled += (double)hm[b] * step;
    const double cd = nd < n_heavy ? sampled : (double)cd_all;
    const double t_sparse = cd * 4.0 / c->cm.sparse_bw;
    // the heavy join values: whole bins from the top, at most kmax of them;
    // the cut with the lowest modelled cost (mode 2: the most)
    uint64_t kc = 0, best_k = 0;
    double heavy = 0;
    uint32_t best_cut = kDenseBins;
    double best_t = 0, best_light = 0;
    for (int b = (int)kDenseBins - 1; b >= 0; b--) {
        if (!hn[b]) continue;
        if (kc + hn[b] > kmax) break;
        kc += hn[b];
        heavy += (double)hm[b] * step;
        const uint64_t Kp = round_up(kc, kDenseBK);
        const double light = sampled > heavy ? sampled - heavy : 0.0;
        const double t = t_product(Kp, light) + t_bitmap + light * light_bytes / c->cm.dense_bw;
        // summaries: each epilogue thread scans its tile's light bucket, so
        // only cuts with a small average bucket qualify
        if (!bits && light > (double)ntile_all * kDenseBucketMax / 4 && b > 0) continue;
        if (mode == 2 || best_k == 0 || t < best_t) {
            best_t = t;
            best_k = kc;
            best_cut = (uint32_t)b;
            best_light = light;
        }
    }
    if (best_k == 0) return DIM3G_OK;
    if (mode == 1 && best_t >= t_sparse) return DIM3G_OK;
    const uint32_t Kp = (uint32_t)round_up(best_k, kDenseBK);
    const uint32_t mt = (uint32_t)(Mp / kDenseBM), nt = (uint32_t)(Np / kDenseBN);
    const uint64_t ntile = (uint64_t)mt * nt;
    uint8_t* A = ws_get<uint8_t>(c, Mp * Kp);
    uint8_t* B = ws_get<uint8_t>(c, Np * Kp);
    uint32_t* D = bits ? ws_get<uint32_t>(c, Mp * Wd) : nullptr;
    if (!A || !B || (bits && !D)) return fail(c, DIM3G_ERR_NOMEM, "workspace allocation failed (dense operands)");
    k_dense_hid<<<grid_for(k, sm), 256, 0, st>>>(degd, rc.JR_S, rc.T, k, best_cut, hid, hy, bin_n + kDenseBins);
    CHECK_LAUNCH();
    DenseSum ds{};
    if (bits) {
        CU(cudaMemsetAsync(A, 0, Mp * Kp, st));
        CU(cudaMemsetAsync(B, 0, Np * Kp, st));
        k_dense_fill_a<<<grid_for(nd * 32, sm), 256, 0, st>>>(rc.JR_R, rc.IC_R, list_m, (uint32_t)nd, hid, A, Kp);
        CHECK_LAUNCH();
        k_dense_fill_b<<<dim3(16, (unsigned)best_k), 256, 0, st>>>(rc.JR_S, rc.IC_S, rc.T, hy, B, Kp);
        CHECK_LAUNCH();
    } else {
        // multiplicities, then e4m3 codes (a multiplicity above 16 keeps the
        // sparse path); the light candidates bucketed by product tile
        uint32_t* A32 = ws_get<uint32_t>(c, Mp * Kp);
        uint32_t* B32 = ws_get<uint32_t>(c, Np * Kp);
        uint32_t* tcnt = ws_get<uint32_t>(c, ntile + 1);
        uint32_t* toff = ws_get<uint32_t>(c, ntile + 1);
        uint32_t* tcur = ws_get<uint32_t>(c, ntile + 1);
        uint64_t* bsum = ws_get<uint64_t>(c, scan_storage(ntile + 1));
        if (!A32 || !B32 || !tcnt || !toff || !tcur || !bsum)
            return fail(c, DIM3G_ERR_NOMEM, "workspace allocation failed (dense counts)");
        unsigned int* flag = bin_n + kDenseBins + 1;
        unsigned long long* ltotal = bin_mass + kDenseBins;
        CU(cudaMemsetAsync(A32, 0, Mp * Kp * 4, st));
        CU(cudaMemsetAsync(B32, 0, Np * Kp * 4, st));
        CU(cudaMemsetAsync(tcnt, 0, (ntile + 1) * 4, st));
        k_dense_cnt_a<<<grid_for(nd * 32, sm), 256, 0, st>>>(rc.JR_R, rc.IC_R, list_m, (uint32_t)nd, hid, A32, Kp);
        CHECK_LAUNCH();
        k_dense_cnt_b<<<dim3(16, (unsigned)best_k), 256, 0, st>>>(rc.JR_S, rc.IC_S, rc.T, hy, B32, Kp);
        CHECK_LAUNCH();
        k_dense_to_fp8<<<grid_for(Mp * Kp, sm), 256, 0, st>>>(A32, A, Mp * Kp, flag);
        CHECK_LAUNCH();
        k_dense_to_fp8<<<grid_for(Np * Kp, sm), 256, 0, st>>>(B32, B, Np * Kp, flag);
        CHECK_LAUNCH();
        k_dense_light<<<grid_for(nd * 32, sm), 256, 0, st>>>(rc.JR_R, rc.IC_R, rc.JR_S, rc.IC_S, rc.T, list_m,
                                                             (uint32_t)nd, hid, LightCount{tcnt, nt});
        CHECK_LAUNCH();
        k_dense_maxcnt<<<grid_for(ntile, sm), 256, 0, st>>>(tcnt, ntile, flag + 1);
        CHECK_LAUNCH();
        SCAN(U32Src{tcnt}, RowPtrDst{toff, tcur}, ntile + 1, bsum, ltotal);
        unsigned int hflag[2] = {0, 0};
        unsigned long long hl = 0;
        CU(cudaMemcpyAsync(hflag, flag, 8, cudaMemcpyDeviceToHost, st));
        CU(cudaMemcpyAsync(&hl, ltotal, 8, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        // not exact in e4m3, or light buckets too large for the epilogue
        c->stats.dense_bucket_max = hflag[1];
        skip = hflag[0] ? 5 : 6;
        if (hflag[0] || hflag[1] > kDenseBucketMax || hl >= 0xFFFFFFFFull) return DIM3G_OK;
        uint16_t* lb = ws_get<uint16_t>(c, hl + 1);
        if (!lb) return fail(c, DIM3G_ERR_NOMEM, "workspace allocation failed (dense light buckets)");
        k_dense_light<<<grid_for(nd * 32, sm), 256, 0, st>>>(rc.JR_R, rc.IC_R, rc.JR_S, rc.IC_S, rc.T, list_m,
                                                             (uint32_t)nd, hid, LightScatter{tcur, lb, nt});
        CHECK_LAUNCH();
        ds = DenseSum{list_m, (uint32_t)nd, rc.id2x, rc.id2z, toff, lb, jp.sum};
        best_light = (double)hl;
    }
    CUtensorMap mA, mB;
    int r = dense_map(c, &mA, A, Mp, Kp, kDenseBM);
    if (!r) r = dense_map(c, &mB, B, Np, Kp, kDenseBN);
    if (r) return r;
    const unsigned grid = (unsigned)(ntile < (uint64_t)sm ? ntile : (uint64_t)sm);
    CU(cudaEventRecord(c->evd[1], st));
    if (kind == kDenseBits)
        k_dense_mma<kDenseBits><<<grid, kDenseThreads, kDenseSmem, st>>>(mA, mB, D, (uint32_t)Wd, mt, nt, Kp / kDenseBK,
                                                                          &sc->err, ds);
    else if (kind == kDenseSumProject)
        k_dense_mma<kDenseSumProject><<<grid, kDenseSumThreads, kDenseSmem, st>>>(mA, mB, nullptr, 0, mt, nt,
                                                                                   Kp / kDenseBK, &sc->err, ds);
    else
        k_dense_mma<kDenseSumCount><<<grid, kDenseSumThreads, kDenseSmem, st>>>(mA, mB, nullptr, 0, mt, nt,
                                                                                 Kp / kDenseBK, &sc->err, ds);
    CHECK_LAUNCH();
    CU(cudaEventRecord(c->evd[2], st));
    uint32_t cpr = 0;
    unsigned long long* coff = nullptr;
    if (bits) {
        k_dense_light<<<grid_for(nd * 32, sm), 256, 0, st>>>(rc.JR_R, rc.IC_R, rc.JR_S, rc.IC_S, rc.T, list_m,
                                                             (uint32_t)nd, hid, LightOr{D, (uint32_t)Wd});
        CHECK_LAUNCH();
        // chunk popcounts and their offsets
        cpr = (uint32_t)((Wd + 31) / 32);
        const uint64_t nc = nd * cpr;
        uint32_t* cc = ws_get<uint32_t>(c, nc + 1);
        coff = ws_get<unsigned long long>(c, nc + 1);
        uint64_t* bsum = ws_get<uint64_t>(c, scan_storage(nc + 1));
        if (!cc || !coff || !bsum) return fail(c, DIM3G_ERR_NOMEM, "workspace allocation failed (dense chunks)");
        k_dense_chunks<<<grid_for(nc * 8, sm), 256, 0, st>>>((uint32_t)nd, D, (uint32_t)Wd, cpr, cc);
        CHECK_LAUNCH();
        SCAN(U32Src{cc}, OffDst{coff}, nc + 1, bsum, nullptr);
    }
    CU(cudaEventRecord(c->evd[3], st));
    {
        // the row-class kernels take the heavy rows after the block's
        const unsigned long long rest[2] = {n_heavy - nd, 0};
        CU(cudaMemcpyAsync(&sc->nrows[3], rest, sizeof rest, cudaMemcpyHostToDevice, st));
        CU(cudaStreamSynchronize(st));  // `rest` is on this frame
    }
    skip = 0;
    c->stats.rows_dense = (uint32_t)nd;
    c->stats.heavy_y = (uint32_t)best_k;
    c->stats.dense_kp = Kp;
    c->stats.dense_light = (uint64_t)best_light;
    dp->on = true;
    dp->nd = (uint32_t)nd;
    dp->Wd = (uint32_t)Wd;
    dp->Wm = (m + 31) / 32;
    dp->cpr = cpr;
    dp->D = D;
    dp->coff = coff;
    return DIM3G_OK;
}

// Device ms of the dense block's phases into the stats (after a sync).
void dense_times(dim3g_ctx* c, const DensePlan& dp) {
    if (!dp.on) return;
    for (int i = 0; i < 3; i++) cudaEventElapsedTime(&c->stats.ms_dense[i], c->evd[i], c->evd[i + 1]);
}

int run_join(dim3g_ctx* c, const JoinPlan& jp, uint64_t* n_out) {
    cudaStream_t st = c->stream;
    c->ws.reset();
    dim3g_stats& S = c->stats;
    memset(&S, 0, sizeof S);
    S.n_big = jp.nP;
    S.n_small = jp.nQ;
    S.swapped = jp.swapped;
    *n_out = 0;
    if (jp.nP >= 0xFFFFFFFFull || jp.nQ >= 0xFFFFFFFFull)
        return fail(c, DIM3G_ERR_UNSUPPORTED, "relations of 2^32-1 or more tuples are not supported");
    if (jp.nP == 0 || jp.nQ == 0) return DIM3G_OK;
    const int sm = c->sm_count;
    CU(cudaEventRecord(c->ev[0], st));

    Scalars* sc = ws_get<Scalars>(c, 1);
    const uint64_t fullP = next_pow2(jp.nP * 2 < 1024 ? 1024 : jp.nP * 2);
    const uint64_t fullQ = next_pow2(jp.nQ * 2 < 1024 ? 1024 : jp.nQ * 2);
    uint2* Qk = ws_get<uint2>(c, jp.nQ);
    uint2* Pm = ws_get<uint2>(c, jp.nP);
    uint32_t* id2x = ws_get<uint32_t>(c, jp.nP);
    uint32_t* id2z = ws_get<uint32_t>(c, round_up(jp.nQ, 1024) + 1024);  // whole 1024-id chunks (dense emission)
    uint32_t* regs = ws_get<uint32_t>(c, 3 * kSketchRegs);
    if (!sc || !Qk || !Pm || !id2x || !id2z || !regs) return fail(c, DIM3G_ERR_NOMEM, "workspace allocation failed (mapping)");

    // table capacities from the distinct-key sketch (see mapping.cuh)
    uint64_t capX = fullP, capY = fullP, capZ = fullQ;
    if (c->prm.sized_tables) {
        CU(cudaMemsetAsync(regs, 0, 3 * kSketchRegs * 4, st));
        k_sketch<<<grid_for(jp.nP > jp.nQ ? jp.nP : jp.nQ, sm, 2), 256, 0, st>>>(jp.P, jp.nP, jp.Q, jp.nQ, regs);
        CHECK_LAUNCH();
        std::vector<uint32_t> hr(3 * kSketchRegs);
        CU(cudaMemcpyAsync(hr.data(), regs, 3 * kSketchRegs * 4, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        auto sized = [&](const uint32_t* r, uint64_t full) {
            double sum = 0;
            uint32_t zeros = 0;
            for (uint32_t k = 0; k < kSketchRegs; k++) {
                sum += ldexp(1.0, -(int)r[k]);
                zeros += r[k] == 0;
            }
            return sketch_capacity(sketch_estimate(sum, zeros), full, c->prm.table_slack_pct);
        };
        capX = sized(hr.data(), fullP);
        capY = sized(hr.data() + kSketchRegs, fullP);
        capZ = sized(hr.data() + 2 * kSketchRegs, fullQ);
    }
    DevTable tx{}, ty{}, tz{};
    for (int attempt = 0;; attempt++) {
        const bool sized = capX < fullP || capY < fullP || capZ < fullQ;
        const uint64_t lim = sized ? kSizedProbeLimit : 0;
        tx = DevTable{ws_get<unsigned long long>(c, capX), capX - 1, lim};
        ty = DevTable{ws_get<unsigned long long>(c, capY), capY - 1, lim};
        tz = DevTable{ws_get<unsigned long long>(c, capZ), capZ - 1, lim};
        const uint64_t capM = capX > capY ? (capX > capZ ? capX : capZ) : (capY > capZ ? capY : capZ);
        uint64_t* bsum = ws_get<uint64_t>(c, scan_storage(capM));
        if (!tx.slots || !ty.slots || !tz.slots || !bsum) return fail(c, DIM3G_ERR_NOMEM, "workspace allocation failed (mapping)");
        CU(cudaMemsetAsync(sc, 0, sizeof(Scalars), st));
        CU(cudaMemsetAsync(tx.slots, 0xff, capX * 8, st));
        CU(cudaMemsetAsync(ty.slots, 0xff, capY * 8, st));
        CU(cudaMemsetAsync(tz.slots, 0xff, capZ * 8, st));

        k_insert_p<<<grid_for(jp.nP, sm), 256, 0, st>>>(jp.P, jp.nP, tx, ty, &sc->err);
        CHECK_LAUNCH();
        SCAN(OccupiedSrc{ty.slots}, AssignIdDst{ty.slots, nullptr}, capY, bsum, &sc->ny);
        SCAN(OccupiedSrc{tx.slots}, AssignIdDst{tx.slots, id2x}, capX, bsum, &sc->nx);
        k_probe_q<<<grid_for(jp.nQ, sm), 256, 0, st>>>(jp.Q, jp.nQ, ty, tz, Qk, &sc->nkept, &sc->err);
        CHECK_LAUNCH();
        SCAN(OccupiedSrc{tz.slots}, AssignIdDst{tz.slots, id2z}, capZ, bsum, &sc->nz);
        CU(cudaMemcpyAsync(c->h_sc, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        if (sized && attempt == 0 && c->h_sc->err == kErrProbeLimit) {
            // a table fuller than the sketch said: build again at full size
            capX = capY = fullP;
            capZ = fullQ;
            S.table_rebuilds++;
            continue;
        }
        break;
    }
    if (c->h_sc->err) return fail(c, DIM3G_ERR_DEVICE, "device bound violated in mapping (flags %u)", c->h_sc->err);
    S.table_slots = capX + capY + capZ;
    const uint32_t n = (uint32_t)c->h_sc->nx, k = (uint32_t)c->h_sc->ny, m = (uint32_t)c->h_sc->nz;
    const uint64_t nq = c->h_sc->nkept;
    S.nx = n;
    S.ny = k;
    S.nz = m;
    S.n_small_kept = nq;
    CU(cudaEventRecord(c->ev[1], st));
    if (nq == 0) {
        S.ms_total = 0;
        return DIM3G_OK;
    }
    if (m >= 0x80000000u || n >= 0x80000000u)
        return fail(c, DIM3G_ERR_UNSUPPORTED, "key domains of 2^31 or more distinct values are not supported");

    // z tiles for the bitmap class
    uint32_t tile_lg = jp.aggregate ? kAggTileLg : c->prm.tile_lg;
    uint32_t T = 1, tile_shift = 31, tile_width = m;
    if (m > (1u << tile_lg)) {
        tile_shift = tile_lg;
        tile_width = 1u << tile_lg;
        T = (m + tile_width - 1) >> tile_lg;
    }
    if ((uint64_t)k * T >= 0xFFFFFFFFull)
        return fail(c, DIM3G_ERR_UNSUPPORTED, "join domain x z tiles too large");
    S.z_tiles = T;
    const uint64_t nyt = (uint64_t)k * T;

    uint32_t* degx = ws_get<uint32_t>(c, (uint64_t)n + 1);
    uint32_t* curx = ws_get<uint32_t>(c, (uint64_t)n + 1);
    uint32_t* JR_R = ws_get<uint32_t>(c, (uint64_t)n + 1);
    uint32_t* IC_R = ws_get<uint32_t>(c, jp.nP);
    uint32_t* cnt_yt = ws_get<uint32_t>(c, nyt + 1);
    uint32_t* cur_yt = ws_get<uint32_t>(c, nyt + 1);
    uint32_t* JR_S = ws_get<uint32_t>(c, nyt + 1);
    uint32_t* IC_S = ws_get<uint32_t>(c, nq);
    uint32_t* VS = nullptr;  // the value paths read the pairs in ISV
    // +2: the streamed bitmap rows copy 16-byte-aligned supersets of S
    // segments, up to one pair past the last one
    uint2* ISV = ws_get<uint2>(c, nq + 2);
    uint32_t* Zq = ws_get<uint32_t>(c, nq);
    uint32_t* ucap = ws_get<uint32_t>(c, n);
    uint8_t* cls = ws_get<uint8_t>(c, n);
    uint32_t* lists = ws_get<uint32_t>(c, (uint64_t)4 * n);
    uint32_t* cnt = ws_get<uint32_t>(c, (uint64_t)n + 1);  // cnt[n] = 0 closes the offsets scan
    unsigned long long* off = ws_get<unsigned long long>(c, (uint64_t)n + 1);
    uint64_t* bsum2 = ws_get<uint64_t>(c, scan_storage((nyt > n ? nyt : n) + 1));
    uint64_t* bsum_r = ws_get<uint64_t>(c, scan_storage((uint64_t)n + 1));
    if (!degx || !curx || !JR_R || !IC_R || !cnt_yt || !cur_yt || !JR_S || !IC_S || !ISV || !Zq || !ucap || !cls || !lists ||
        !cnt || !off || !bsum2 || !bsum_r)
        return fail(c, DIM3G_ERR_NOMEM, "workspace allocation failed (CSR)");

    // The two CSRs are independent: R's (by x) on the side stream while S's
    // (by (y, z tile)) runs here; both are latency-bound scatters, so they
    // overlap.  Joined before the row classification.
    const cudaStream_t ax = c->aux;
    CU(cudaEventRecord(c->ev_fork, st));
    CU(cudaStreamWaitEvent(ax, c->ev_fork, 0));
    CU(cudaMemsetAsync(degx, 0, ((uint64_t)n + 1) * 4, ax));
    k_map_p<<<grid_for(jp.nP, sm), 256, 0, ax>>>(jp.P, jp.nP, tx, ty, Pm, degx);
    CHECK_LAUNCH();
    {
        int r = run_scan(c, U32Src{degx}, RowPtrDst{JR_R, curx}, (uint64_t)n + 1, bsum_r, nullptr, ax);
        if (r) return r;
    }
    k_scatter_r<<<grid_for(jp.nP, sm), 256, 0, ax>>>(Pm, jp.nP, curx, IC_R);
    CHECK_LAUNCH();
    CU(cudaEventRecord(c->ev_join, ax));
    CU(cudaMemsetAsync(cnt_yt, 0, (nyt + 1) * 4, st));
    k_map_q<<<grid_for(nq, sm), 256, 0, st>>>(Qk, nq, tz, T, tile_shift, Zq, cnt_yt);
    CHECK_LAUNCH();
    SCAN(U32Src{cnt_yt}, RowPtrDst{JR_S, cur_yt}, nyt + 1, bsum2, nullptr);
    k_scatter_s<<<grid_for(nq, sm), 256, 0, st>>>(Qk, Zq, nq, T, tile_shift, cur_yt, IC_S, VS, ISV);
    CHECK_LAUNCH();
    CU(cudaStreamWaitEvent(st, c->ev_join, 0));

    RowCtx rc{};
    rc.JR_R = JR_R;
    rc.IC_R = IC_R;
    rc.JR_S = JR_S;
    rc.IC_S = IC_S;
    rc.VS = VS;
    rc.ISV = ISV;
    rc.T = T;
    rc.tile_width = tile_width;
    rc.m = m;
    rc.cta_rr = c->prm.cta_rr;
    rc.ucap = ucap;
    rc.cnt = cnt;
    rc.off = off;
    rc.id2x = id2x;
    rc.id2z = id2z;
    rc.out = nullptr;
    rc.err = &sc->err;
    const uint32_t cap_w = 1u << (c->prm.warp_lg - 1);
    const uint32_t cap_b = 1u << (c->prm.block_lg - 1);
    // tiny rows get their own warp launch in the single pass only
    const bool tiny = jp.single_pass && !jp.aggregate && !jp.count_only;
    k_row_work<<<grid_for((uint64_t)n * 32, sm), 256, 0, st>>>(rc, n, cap_w, cap_b, jp.aggregate, tiny, jp.sum, ucap, cls,
                                                                &sc->outj, sc->outj_cls);
    CHECK_LAUNCH();
    uint32_t* list_w = lists;
    uint32_t* list_b = lists + n;
    uint32_t* list_m = lists + 2 * (uint64_t)n;
    uint32_t* list_t = lists + 3 * (uint64_t)n;
    SCAN(ClassSrc{cls, 1}, ListDst{list_w, nullptr}, n, bsum2, &sc->nrows[1]);
    SCAN(ClassSrc{cls, 2}, ListDst{list_b, nullptr}, n, bsum2, &sc->nrows[2]);
    const bool block_split = jp.single_pass && !jp.aggregate && !jp.count_only && !jp.sum.tiles &&
                             c->prm.block_split && !(c->prm.prefetch_rows && c->prm.cta_rr == 3);
    if (block_split) {
        // the same rows again, ordered by hash-set size: u <= 2^(b-3), then
        // u <= 2^(b-2), then the rest (b = block_lg; 2^lg slots for 2u keys)
        const uint32_t b = c->prm.block_lg;
        SCAN(BlockSizeSrc{cls, ucap, 0u, 1u << (b - 3)}, ListDst{list_b, nullptr}, n, bsum2, &sc->nrows_b[0]);
        SCAN(BlockSizeSrc{cls, ucap, 1u << (b - 3), 1u << (b - 2)}, ListDst{list_b, &sc->nrows_b[0]}, n, bsum2,
             &sc->nrows_b[1]);
        SCAN(BlockSizeSrc{cls, ucap, 1u << (b - 2), 0xFFFFFFFFu}, ListDst{list_b, &sc->nrows_b[0], &sc->nrows_b[1]}, n,
             bsum2, &sc->nrows_b[2]);
    }
    // bitmap rows: class 4 (huge) first, then class 3
    SCAN(ClassSrc{cls, 4}, ListDst{list_m, nullptr}, n, bsum2, &sc->nrows[4]);
    SCAN(ClassSrc{cls, 3}, ListDst{list_m, &sc->nrows[4]}, n, bsum2, &sc->nrows[3]);
    if (tiny) SCAN(ClassSrc{cls, 5}, ListDst{list_t, nullptr}, n, bsum2, &sc->nrows[5]);
    CU(cudaMemsetAsync(cnt, 0, ((uint64_t)n + 1) * 4, st));
    CU(cudaEventRecord(c->ev[2], st));
    DensePlan dp;
    {
        int r = run_dense(c, jp, rc, sc, list_m, k, m, &dp);
        if (r) return r;
    }

    // Row counts are read on the device; grids are resident CTAs x SMs.
    const RowLists L{list_w, list_b, list_m + dp.nd, &sc->nrows[1], &sc->nrows[2], &sc->nrows[3], &sc->nrows[4]};
    rc.next_row = sc->next_row;
    const uint32_t wpc = warps_per_cta((size_t)4 << c->prm.warp_lg);  // warp-class CTA width
    const size_t smem_w = (size_t)wpc << c->prm.warp_lg << 2;
    const size_t smem_b = (size_t)1 << c->prm.block_lg << 2;
    size_t smem_m = (size_t)((((tile_width + 31) / 32) + 3) / 4) * 16;  // whole uint4 words (cleared as uint4)
    if (smem_m < 128) smem_m = 128;  // idle lanes touch words 0..31
    const int blk_m = tile_width > (1u << 19) ? 1024 : DIM3G_BM_THREADS;
    const unsigned g_w = resident_grid(k_rows_warp<true>, 32 * wpc, smem_w, sm);
    const int blk_b = (int)c->prm.block_threads;
    const unsigned g_b = resident_grid(k_rows_block<true>, blk_b, smem_b, sm);
    const unsigned g_m = resident_grid(k_rows_bitmap<true>, blk_m, smem_m, sm);

    if (jp.sum.tiles) {
        // summaries: the expansion kernels hash instead of writing; COUNT
        // needs no count pass (nothing is placed)
        CU(cudaEventRecord(c->evc[4], st));
        if (jp.aggregate) {
            int r = run_aggregate_write(c, rc, AggOut{nullptr, jp.sum}, L);
            if (r) return r;
        } else {
            k_sum_bitmap<<<resident_grid(k_sum_bitmap, blk_m, smem_m, sm), blk_m, smem_m, st>>>(rc, jp.sum, L.m,
                                                                                            L.n3, L.n4);
            CHECK_LAUNCH();
            k_sum_block<<<resident_grid(k_sum_block, blk_b, smem_b, sm), blk_b, smem_b, st>>>(rc, jp.sum, L.b, L.nb,
                                                                                          c->prm.block_lg);
            CHECK_LAUNCH();
            const size_t sw = (size_t)wpc << c->prm.warp_lg << 2;
            k_sum_warp<<<resident_grid(k_sum_warp, 32 * wpc, sw, sm), 32 * wpc, sw, st>>>(rc, jp.sum, L.w, L.nw,
                                                                                      c->prm.warp_lg);
            CHECK_LAUNCH();
        }
        CU(cudaMemcpyAsync(c->h_sc, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
        CU(cudaEventRecord(c->ev[3], st));
        CU(cudaStreamSynchronize(st));
        if (c->h_sc->err) return fail(c, DIM3G_ERR_DEVICE, "device bound violated in summary (flags %u)", c->h_sc->err);
        dense_times(c, dp);
        S.out_j = c->h_sc->outj;
        S.rows_warp = (uint32_t)c->h_sc->nrows[1];
        S.rows_block = (uint32_t)c->h_sc->nrows[2];
        S.rows_bitmap = (uint32_t)(c->h_sc->nrows[3] + c->h_sc->nrows[4]);
        float a, b, e;
        cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
        cudaEventElapsedTime(&e, c->ev[2], c->ev[3]);
        S.ms_map = a;
        S.ms_csr = b;
        S.ms_write = e;
        S.ms_total = a + b + e;
        return DIM3G_OK;
    }
    if (jp.single_pass && !jp.aggregate && !jp.count_only) {
        uint2* out = nullptr;
        uint64_t cap = 0;
        jp.prep.peek(c, jp.prep.user, &out, &cap);
        if (!out) cap = 0;
        rc.out = out;
        const Reserve rs{&sc->cursor, cap};
        CU(cudaEventRecord(c->evc[4], st));
        // single-pass kernels add one kStage-entry staging buffer per warp
        const uint32_t bm_words = (uint32_t)(smem_m / 4);
        const size_t ss_m = smem_m + (size_t)(blk_m / 32) * kStage * 4;
        const size_t ss_b = smem_b + (size_t)(blk_b / 32) * kStage * 4;
        const uint32_t wps = warps_per_cta(warp_row_words(c->prm.warp_lg, kStage) * 4);
        const size_t ss_w = (size_t)wps * warp_row_words(c->prm.warp_lg, kStage) * 4;
        const uint32_t wpt = warps_per_cta(warp_row_words(kTinyLg, kTinyStage) * 4);
        const size_t ss_t = (size_t)wpt * warp_row_words(kTinyLg, kTinyStage) * 4;
        if (dp.on) {
            k_dense_reserve<<<1, 1, 0, st>>>(dp.coff + (uint64_t)dp.nd * dp.cpr, &sc->cursor, cap, &sc->dense_base);
            CHECK_LAUNCH();
            k_dense_emit<<<resident_grid(k_dense_emit, 256, kDenseEmitSmem, sm), 256, kDenseEmitSmem, st>>>(
                list_m, dp.nd, dp.D, dp.Wd, dp.Wm, dp.cpr, dp.coff, id2x, id2z, out, nullptr, &sc->dense_base);
            CHECK_LAUNCH();
        }
        // the cross-segment gather's threshold per row class, measured on
        // the 2-hop (bitmap rows 45.5 -> 44.7 ms at 160, block rows 26.3 ->
        // 25.7 at 560, warp rows 2.62 -> 2.58 at 160; every setting exact)
        rc.flat_avg = kFlatAvgBitmap;
        if (c->prm.stream_rows && stream_smem_bytes(bm_words) <= kMaxSmemOptin) {
            const size_t ss_s = stream_smem_bytes(bm_words);
            k_stream_bitmap<<<resident_grid(k_stream_bitmap, kStreamThreads, ss_s, sm), kStreamThreads, ss_s, st>>>(
                rc, rs, L.m, L.n3, L.n4, bm_words);
        } else {
            k_single_bitmap<<<resident_grid(k_single_bitmap, blk_m, ss_m, sm), blk_m, ss_m, st>>>(rc, rs, L.m, L.n3,
                                                                                             L.n4, bm_words);
        }
        CHECK_LAUNCH();
        CU(cudaEventRecord(c->evc[5], st));
        CU(cudaMemcpyAsync(&sc->cursor_at[0], &sc->cursor, 8, cudaMemcpyDeviceToDevice, st));
        rc.flat_avg = kFlatAvgBlock;
        if (c->prm.prefetch_rows && c->prm.cta_rr == 3) {
            const size_t ss_p = (((size_t)1 << c->prm.block_lg) + (size_t)kPfWorkers * kStage) * 4;
            k_single_block_pf<<<resident_grid(k_single_block_pf, kPfThreads, ss_p, sm), kPfThreads, ss_p, st>>>(
                rc, rs, L.b, L.nb, c->prm.block_lg);
        } else if (block_split) {
            // three launches over list_b's three parts, smallest sets first
            const uint32_t b = c->prm.block_lg;
            const unsigned long long* skip[3][2] = {{nullptr, nullptr}, {&sc->nrows_b[0], nullptr},
                                                    {&sc->nrows_b[0], &sc->nrows_b[1]}};
            for (uint32_t k = 0; k < 3; k++) {
                const int thr = k < 2 ? (int)kBlockSplitThreads : blk_b;
                const uint32_t lg = b - 2 + k;
                const size_t ss = ((size_t)1 << lg << 2) + (size_t)(thr / 32) * kStage * 4;
                k_single_block<<<resident_grid(k_single_block, thr, ss, sm), thr, ss, st>>>(
                    rc, rs, L.b, &sc->nrows_b[k], lg, skip[k][0], skip[k][1], 4 + k);
                CHECK_LAUNCH();
            }
        } else {
            k_single_block<<<resident_grid(k_single_block, blk_b, ss_b, sm), blk_b, ss_b, st>>>(
                rc, rs, L.b, L.nb, c->prm.block_lg, nullptr, nullptr, 2);
        }
        CHECK_LAUNCH();
        CU(cudaEventRecord(c->evc[6], st));
        CU(cudaMemcpyAsync(&sc->cursor_at[1], &sc->cursor, 8, cudaMemcpyDeviceToDevice, st));
        rc.flat_avg = kFlatAvgWarp;
        k_single_warp<<<resident_grid(k_single_warp, 32 * wps, ss_w, sm), 32 * wps, ss_w, st>>>(rc, rs, L.w, L.nw,
                                                                                           c->prm.warp_lg, kStage);
        CHECK_LAUNCH();
        k_single_warp<<<resident_grid(k_single_warp, 32 * wpt, ss_t, sm), 32 * wpt, ss_t, st>>>(rc, rs, list_t,
                                                                                           &sc->nrows[5], kTinyLg,
                                                                                           kTinyStage);
        CHECK_LAUNCH();
        CU(cudaEventRecord(c->evc[7], st));
        CU(cudaMemcpyAsync(c->h_sc, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
        CU(cudaEventRecord(c->ev[3], st));
        CU(cudaStreamSynchronize(st));
        if (c->h_sc->err) return fail(c, DIM3G_ERR_DEVICE, "device bound violated in single pass (flags %u)", c->h_sc->err);
        dense_times(c, dp);
        const uint64_t total = c->h_sc->cursor;
        S.out_j = c->h_sc->outj;
        S.n_out_cls[0] = c->h_sc->cursor_at[0];
        S.n_out_cls[1] = c->h_sc->cursor_at[1] - c->h_sc->cursor_at[0];
        S.n_out_cls[2] = total - c->h_sc->cursor_at[1];
        S.n_out = total;
        S.rows_warp = (uint32_t)(c->h_sc->nrows[1] + c->h_sc->nrows[5]);
        S.rows_block = (uint32_t)c->h_sc->nrows[2];
        S.rows_bitmap = (uint32_t)(c->h_sc->nrows[3] + c->h_sc->nrows[4]);
        S.out_j_cls[0] = c->h_sc->outj_cls[3] + c->h_sc->outj_cls[4];
        S.out_j_cls[1] = c->h_sc->outj_cls[2];
        S.out_j_cls[2] = c->h_sc->outj_cls[1] + c->h_sc->outj_cls[5];
        *n_out = total;
        float a, b, e;
        cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
        cudaEventElapsedTime(&e, c->ev[2], c->ev[3]);
        for (int i = 0; i < 3; i++) cudaEventElapsedTime(&S.ms_write_cls[i], c->evc[4 + i], c->evc[5 + i]);
        S.ms_map = a;
        S.ms_csr = b;
        S.ms_write = e;
        S.ms_total = a + b + e;
        if (total > cap)
            return fail(c, DIM3G_ERR_CAPACITY, "output needs %llu pairs, capacity is %llu", (unsigned long long)total,
                        (unsigned long long)cap);
        return DIM3G_OK;
    }

    // count pass (the bitmap rows, the largest, start first)
    CU(cudaEventRecord(c->evc[0], st));
    if (dp.on) {
        k_dense_rowcnt<<<grid_for(dp.nd, sm), 256, 0, st>>>(list_m, dp.nd, dp.cpr, dp.coff, cnt);
        CHECK_LAUNCH();
    }
    k_rows_bitmap<false><<<g_m, blk_m, smem_m, st>>>(rc, L.m, L.n3, L.n4);
    CHECK_LAUNCH();
    CU(cudaEventRecord(c->evc[1], st));
    k_rows_block<false><<<g_b, blk_b, smem_b, st>>>(rc, L.b, L.nb, c->prm.block_lg);
    CHECK_LAUNCH();
    CU(cudaEventRecord(c->evc[2], st));
    k_rows_warp<false><<<g_w, 32 * wpc, smem_w, st>>>(rc, L.w, L.nw, c->prm.warp_lg);
    CHECK_LAUNCH();
    CU(cudaEventRecord(c->evc[3], st));
    SCAN(U32Src{cnt}, OffDst{off}, (uint64_t)n + 1, bsum2, &sc->total);
    CU(cudaMemcpyAsync(c->h_sc, sc, sizeof(Scalars), cudaMemcpyDeviceToHost, st));
    CU(cudaEventRecord(c->ev[3], st));
    CU(cudaStreamSynchronize(st));
    if (c->h_sc->err) return fail(c, DIM3G_ERR_DEVICE, "device bound violated in count pass (flags %u)", c->h_sc->err);
    dense_times(c, dp);
    const uint64_t total = c->h_sc->total;
    for (int i = 0; i < 3; i++) cudaEventElapsedTime(&S.ms_count_cls[i], c->evc[i], c->evc[i + 1]);
    S.out_j = c->h_sc->outj;
    S.n_out = total;
    S.rows_warp = (uint32_t)c->h_sc->nrows[1];
    S.rows_block = (uint32_t)c->h_sc->nrows[2];
    S.rows_bitmap = (uint32_t)(c->h_sc->nrows[3] + c->h_sc->nrows[4]);
    S.out_j_cls[0] = c->h_sc->outj_cls[3] + c->h_sc->outj_cls[4];
    S.out_j_cls[1] = c->h_sc->outj_cls[2];
    S.out_j_cls[2] = c->h_sc->outj_cls[1];
    *n_out = total;
    if (jp.count_only) {
        float a, b, d;
        cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
        cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
        cudaEventElapsedTime(&d, c->ev[2], c->ev[3]);
        S.ms_map = a;
        S.ms_csr = b;
        S.ms_count = d;
        S.ms_total = a + b + d;
        return DIM3G_OK;
    }
    uint2* out = nullptr;
    unsigned long long* out_cnt = nullptr;
    int pr = jp.prep.fn(c, jp.prep.user, total, &out, &out_cnt);
    if (pr) return pr;
    rc.out = out;
    CU(cudaMemsetAsync(sc->next_row, 0, sizeof(sc->next_row), st));
    if (total > 0) {
        if (jp.aggregate) {
            int r = run_aggregate_write(c, rc, AggOut{out_cnt}, L);
            if (r) return r;
        } else {
            CU(cudaEventRecord(c->evc[4], st));
            if (dp.on) {
                k_dense_emit<<<resident_grid(k_dense_emit, 256, kDenseEmitSmem, sm), 256, kDenseEmitSmem, st>>>(
                    list_m, dp.nd, dp.D, dp.Wd, dp.Wm, dp.cpr, dp.coff, id2x, id2z, out, off, nullptr);
                CHECK_LAUNCH();
            }
            k_rows_bitmap<true><<<g_m, blk_m, smem_m, st>>>(rc, L.m, L.n3, L.n4);
            CHECK_LAUNCH();
            CU(cudaEventRecord(c->evc[5], st));
            k_rows_block<true><<<g_b, blk_b, smem_b, st>>>(rc, L.b, L.nb, c->prm.block_lg);
            CHECK_LAUNCH();
            CU(cudaEventRecord(c->evc[6], st));
            k_rows_warp<true><<<g_w, 32 * wpc, smem_w, st>>>(rc, L.w, L.nw, c->prm.warp_lg);
            CHECK_LAUNCH();
            CU(cudaEventRecord(c->evc[7], st));
        }
    }
    CU(cudaMemcpyAsync(&c->h_sc->err, &sc->err, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    CU(cudaEventRecord(c->ev[4], st));
    CU(cudaStreamSynchronize(st));
    if (c->h_sc->err) return fail(c, DIM3G_ERR_DEVICE, "device bound violated in write pass (flags %u)", c->h_sc->err);
    float a, b, d, e;
    cudaEventElapsedTime(&a, c->ev[0], c->ev[1]);
    cudaEventElapsedTime(&b, c->ev[1], c->ev[2]);
    cudaEventElapsedTime(&d, c->ev[2], c->ev[3]);
    cudaEventElapsedTime(&e, c->ev[3], c->ev[4]);
    S.ms_map = a;
    S.ms_csr = b;
    S.ms_count = d;
    S.ms_write = e;
    S.ms_total = a + b + d + e;
    if (total > 0 && !jp.aggregate)
        for (int i = 0; i < 3; i++) cudaEventElapsedTime(&S.ms_write_cls[i], c->evc[4 + i], c->evc[5 + i]);
    return DIM3G_OK;
}

int run_aggregate_write(dim3g_ctx* c, const RowCtx& rc, AggOut ao, const RowLists& L) {
    cudaStream_t st = c->stream;
    const int sm = c->sm_count;
    const uint32_t wpa = warps_per_cta((size_t)8 << c->prm.warp_lg);
    const size_t smem_w = (size_t)wpa << (c->prm.warp_lg + 1) << 2;
    const size_t smem_b = (size_t)2 << c->prm.block_lg << 2;
    const size_t smem_m = (size_t)rc.tile_width * 4;
    k_agg_tile<<<resident_grid(k_agg_tile, 1024, smem_m, sm), 1024, smem_m, st>>>(rc, ao, L.m, L.n3, L.n4);
    CHECK_LAUNCH();
    k_agg_block<<<resident_grid(k_agg_block, 256, smem_b, sm), 256, smem_b, st>>>(rc, ao, L.b, L.nb, c->prm.block_lg);
    CHECK_LAUNCH();
    k_agg_warp<<<resident_grid(k_agg_warp, 32 * wpa, smem_w, sm), 32 * wpa, smem_w, st>>>(rc, ao, L.w, L.nw,
                                                                                         c->prm.warp_lg);
    CHECK_LAUNCH();
    return DIM3G_OK;
}

bool set_aggregate_attributes() {
    return cudaFuncSetAttribute(k_agg_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess &&
           cudaFuncSetAttribute(k_sum_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) == cudaSuccess &&
           cudaFuncSetAttribute(k_sum_block, cudaFuncAttributeMaxDynamicSharedMemorySize, 1 << 14 << 2) == cudaSuccess &&
           cudaFuncSetAttribute(k_sum_bitmap, cudaFuncAttributeMaxDynamicSharedMemorySize, (1 << 20) / 8) == cudaSuccess &&
           cudaFuncSetAttribute(k_agg_block, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 << 14 << 2) == cudaSuccess &&
           cudaFuncSetAttribute(k_agg_tile, cudaFuncAttributeMaxDynamicSharedMemorySize, (1 << kAggTileLg) * 4) == cudaSuccess;
}

int ensure_dev(dim3g_ctx* c, void** p, size_t* have, size_t need) {
    if (*have >= need && *p) return DIM3G_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *have = 0;
    size_t sz = need < 4096 ? 4096 : need;
    if (cudaMalloc(p, sz) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return fail(c, DIM3G_ERR_NOMEM, "device allocation of %zu bytes failed", sz);
    }
    *have = sz;
    return DIM3G_OK;
}

bool aligned8(const void* p) { return ((uintptr_t)p & 7u) == 0; }

// Output preparation for device-resident callers: their buffer and capacity.
struct DeviceOut {
    uint2* out;
    unsigned long long* cnt;
    uint64_t capacity;
};
int prep_device(dim3g_ctx* c, void* user, uint64_t total, uint2** out, unsigned long long** cnt) {
    DeviceOut* d = (DeviceOut*)user;
    if (total > d->capacity)
        return fail(c, DIM3G_ERR_CAPACITY, "output needs %llu pairs, capacity is %llu", (unsigned long long)total,
                    (unsigned long long)d->capacity);
    *out = d->out;
    *cnt = d->cnt;
    return DIM3G_OK;
}
void peek_device(dim3g_ctx*, void* user, uint2** out, uint64_t* capacity) {
    DeviceOut* d = (DeviceOut*)user;
    *out = d->out;
    *capacity = d->capacity;
}

// Output preparation for host callers: the context's grow-only device staging.
struct StagingOut {
    bool aggregate;
};
int prep_staging(dim3g_ctx* c, void* user, uint64_t total, uint2** out, unsigned long long** cnt) {
    bool agg = ((StagingOut*)user)->aggregate;
    int r = ensure_dev(c, &c->d_out, &c->d_out_bytes, total * (agg ? 16 : 8));
    if (r) return r;
    *out = (uint2*)c->d_out;
    *cnt = agg ? (unsigned long long*)((char*)c->d_out + total * 8) : nullptr;
    return DIM3G_OK;
}
void peek_staging(dim3g_ctx* c, void*, uint2** out, uint64_t* capacity) {
    *out = (uint2*)c->d_out;
    *capacity = c->d_out ? c->d_out_bytes / 8 : 0;
}

// Host-input join: stage R and S on the device, run, copy the result back
// into the caller's buffer (out_into) or a malloc'd one (out_alloc).
int host_join(dim3g_ctx* c, const uint32_t* R, uint64_t nR, const uint32_t* S, uint64_t nS, bool aggregate,
              uint32_t** out_alloc, uint64_t** cnt_alloc, uint32_t* out_into, uint64_t capacity, uint64_t* n_out) {
    if (!c) return DIM3G_ERR_INVALID;
    if (!n_out || (nR && !R) || (nS && !S)) return fail(c, DIM3G_ERR_INVALID, "null argument");
    *n_out = 0;
    if (out_alloc) *out_alloc = nullptr;
    if (cnt_alloc) *cnt_alloc = nullptr;
    CU(cudaSetDevice(c->device));
    const bool swap = !c->prm.keep_roles && nR < nS;
    const uint32_t* P = swap ? S : R;
    const uint32_t* Q = swap ? R : S;
    const uint64_t nP = swap ? nS : nR, nQ = swap ? nR : nS;
    int r = ensure_dev(c, &c->d_in, &c->d_in_bytes, (nP + nQ) * 8 + 256);
    if (r) return r;
    uint2* dP = (uint2*)c->d_in;
    uint2* dQ = dP + nP;
    cudaStream_t st = c->stream;
    if (nP) CU(cudaMemcpyAsync(dP, P, nP * 8, cudaMemcpyHostToDevice, st));
    if (nQ) CU(cudaMemcpyAsync(dQ, Q, nQ * 8, cudaMemcpyHostToDevice, st));
    // A pinned host output buffer is mapped into the device's address space:
    // the single pass stores pairs straight into it (over NVLink-C2C on
    // GB300), overlapping the transfer with the expansion instead of a copy
    // after it.
    if (out_into && !aggregate && !c->prm.ordered && c->prm.host_direct) {
        cudaPointerAttributes pa;
        if (cudaPointerGetAttributes(&pa, out_into) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
            pa.devicePointer && aligned8(pa.devicePointer)) {
            DeviceOut d{(uint2*)pa.devicePointer, nullptr, capacity};
            JoinPlan jd{dP, nP, dQ, nQ, swap, false, false, true, OutPrep{prep_device, peek_device, &d}};
            return run_join(c, jd, n_out);
        }
        cudaGetLastError();
    }
    StagingOut so{aggregate};
    // single pass once the staging buffer exists; a result larger than it
    // grows the buffer and runs again
    const bool single = !aggregate && !c->prm.ordered && c->d_out != nullptr;
    JoinPlan jp{dP, nP, dQ, nQ, swap, aggregate, false, single, OutPrep{prep_staging, peek_staging, &so}};
    uint64_t n = 0;
    r = run_join(c, jp, &n);
    if (r == DIM3G_ERR_CAPACITY && single) {
        r = ensure_dev(c, &c->d_out, &c->d_out_bytes, n * 8);
        if (r) return r;
        r = run_join(c, jp, &n);
    }
    if (r) return r;
    *n_out = n;
    const uint2* dout = (const uint2*)c->d_out;
    const unsigned long long* dcnt = aggregate ? (const unsigned long long*)((const char*)c->d_out + n * 8) : nullptr;
    if (out_into) {
        if (n > capacity)
            return fail(c, DIM3G_ERR_CAPACITY, "output needs %llu pairs, capacity is %llu", (unsigned long long)n,
                        (unsigned long long)capacity);
        if (n) CU(cudaMemcpyAsync(out_into, dout, n * 8, cudaMemcpyDeviceToHost, st));
        CU(cudaStreamSynchronize(st));
        return DIM3G_OK;
    }
    uint32_t* h = (uint32_t*)malloc(n ? n * 8 : 8);
    uint64_t* hc = nullptr;
    if (!h) return fail(c, DIM3G_ERR_NOMEM, "host allocation of %llu pairs failed", (unsigned long long)n);
    if (aggregate) {
        hc = (uint64_t*)malloc(n ? n * 8 : 8);
        if (!hc) {
            free(h);
            return fail(c, DIM3G_ERR_NOMEM, "host allocation of %llu counts failed", (unsigned long long)n);
        }
    }
    if (n) {
        cudaError_t e1 = cudaMemcpyAsync(h, dout, n * 8, cudaMemcpyDeviceToHost, st);
        cudaError_t e2 = aggregate ? cudaMemcpyAsync(hc, dcnt, n * 8, cudaMemcpyDeviceToHost, st) : cudaSuccess;
        cudaError_t e3 = cudaStreamSynchronize(st);
        if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
            free(h);
            free(hc);
            return fail(c, DIM3G_ERR_CUDA, "result copy failed: %s",
                        cudaGetErrorString(e1 != cudaSuccess ? e1 : (e2 != cudaSuccess ? e2 : e3)));
        }
    }
    *out_alloc = h;
    if (cnt_alloc) *cnt_alloc = hc;
    return DIM3G_OK;
}

}  // namespace

namespace dim3g_internal {
cudaStream_t stream(const dim3g_ctx* c) { return c->stream; }
int device(const dim3g_ctx* c) { return c->device; }
int sm_count(const dim3g_ctx* c) { return c->sm_count; }
void add_launches(dim3g_ctx* c, uint64_t n) { c->launches += n; }
void set_sparse_rate(dim3g_ctx* c, double bytes_per_s) {
    if (bytes_per_s > 0) c->cm.sparse_bw = bytes_per_s;
}
int fail(dim3g_ctx* c, int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (c) c->err = buf;
    return code;
}
}  // namespace dim3g_internal

// ====================================================================== C ABI
extern "C" {

int dim3g_create(int device, dim3g_ctx** out) {
    if (!out) return DIM3G_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return DIM3G_ERR_CUDA;
    }
    dim3g_ctx* c = new dim3g_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->aux, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
        cudaMallocHost((void**)&c->h_sc, sizeof(Scalars)) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return DIM3G_ERR_CUDA;
    }
    for (auto& e : c->ev) cudaEventCreate(&e);
    for (auto& e : c->evc) cudaEventCreate(&e);
    for (auto& e : c->evd) cudaEventCreate(&e);
    c->stream = c->own_stream;
    // Shared-memory carve-outs for the expansion kernels (largest settings).
    const int smem_b = 1 << 14 << 2, smem_m = (1 << 20) / 8;
    const int smem_wmax = 200 * 1024;
    bool ok = cudaFuncSetAttribute(k_rows_warp<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_wmax) == cudaSuccess &&
              cudaFuncSetAttribute(k_rows_warp<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_wmax) == cudaSuccess &&
              cudaFuncSetAttribute(k_rows_block<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_b) == cudaSuccess &&
              cudaFuncSetAttribute(k_rows_block<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_b) == cudaSuccess &&
              cudaFuncSetAttribute(k_rows_bitmap<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_m) == cudaSuccess &&
              cudaFuncSetAttribute(k_rows_bitmap<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_m) == cudaSuccess &&
              cudaFuncSetAttribute(k_single_warp, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_wmax) == cudaSuccess &&
              cudaFuncSetAttribute(k_single_block, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   ((1 << 14) + 32 * (int)kStage) * 4) == cudaSuccess &&
              cudaFuncSetAttribute(k_single_bitmap, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   smem_m + 32 * (int)kStage * 4) == cudaSuccess &&
              cudaFuncSetAttribute(k_single_block_pf, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   ((1 << 14) + (int)(kPfWorkers * kStage)) * 4) == cudaSuccess &&
              cudaFuncSetAttribute(k_stream_bitmap, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(stream_smem_bytes(smem_m / 4) < kMaxSmemOptin ? stream_smem_bytes(smem_m / 4)
                                                                                      : kMaxSmemOptin)) == cudaSuccess &&
              cudaFuncSetAttribute(k_dense_mma<kDenseBits>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kDenseSmem) == cudaSuccess &&
              cudaFuncSetAttribute(k_dense_mma<kDenseSumProject>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kDenseSmem) == cudaSuccess &&
              cudaFuncSetAttribute(k_dense_mma<kDenseSumCount>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)kDenseSmem) == cudaSuccess &&
              cudaFuncSetAttribute(k_dense_emit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kDenseEmitSmem) ==
                  cudaSuccess &&
              set_aggregate_attributes();
    if (!ok) {
        cudaGetLastError();
        dim3g_destroy(c);
        return DIM3G_ERR_CUDA;
    }
    *out = c;
    return DIM3G_OK;
}

void dim3g_destroy(dim3g_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    c->ws.release();
    if (c->d_in) cudaFree(c->d_in);
    if (c->d_out) cudaFree(c->d_out);
    if (c->d_sum) cudaFree(c->d_sum);
    if (c->h_sc) cudaFreeHost(c->h_sc);
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->evc)
        if (e) cudaEventDestroy(e);
    for (auto& e : c->evd)
        if (e) cudaEventDestroy(e);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->aux) cudaStreamDestroy(c->aux);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
}

int dim3g_set_stream(dim3g_ctx* c, void* s) {
    if (!c) return DIM3G_ERR_INVALID;
    c->stream = s ? (cudaStream_t)s : c->own_stream;
    return DIM3G_OK;
}

const char* dim3g_last_error(const dim3g_ctx* c) { return c ? c->err.c_str() : "null context"; }

int dim3g_get_stats(const dim3g_ctx* c, dim3g_stats* out) {
    if (!c || !out) return DIM3G_ERR_INVALID;
    *out = c->stats;
    out->launches = c->launches;
    return DIM3G_OK;
}

int dim3g_set_param(dim3g_ctx* c, const char* name, int64_t v) {
    if (!c || !name) return DIM3G_ERR_INVALID;
    if (!strcmp(name, "warp_slots_log2")) {
        if (v < 5 || v > 14) return fail(c, DIM3G_ERR_INVALID, "warp_slots_log2 must be in 5..14");
        if ((uint32_t)v > c->prm.block_lg) c->prm.block_lg = (uint32_t)v;
        c->prm.warp_lg = (uint32_t)v;
    } else if (!strcmp(name, "block_slots_log2")) {
        if (v < 8 || v > 14) return fail(c, DIM3G_ERR_INVALID, "block_slots_log2 must be in 8..14");
        if ((uint32_t)v < c->prm.warp_lg) return fail(c, DIM3G_ERR_INVALID, "block_slots_log2 below warp_slots_log2");
        c->prm.block_lg = (uint32_t)v;
    } else if (!strcmp(name, "tile_bits_log2")) {
        if (v < 10 || v > 20) return fail(c, DIM3G_ERR_INVALID, "tile_bits_log2 must be in 10..20");
        c->prm.tile_lg = (uint32_t)v;
    } else if (!strcmp(name, "cta_walk")) {
        if (v < 0 || v > 3) return fail(c, DIM3G_ERR_INVALID, "cta_walk must be 0, 1, 2 or 3");
        c->prm.cta_rr = (uint32_t)v;
    } else if (!strcmp(name, "host_direct_output")) {
        if (v != 0 && v != 1) return fail(c, DIM3G_ERR_INVALID, "host_direct_output must be 0 or 1");
        c->prm.host_direct = v != 0;
    } else if (!strcmp(name, "block_threads")) {
        if (v != 256 && v != 512 && v != 1024) return fail(c, DIM3G_ERR_INVALID, "block_threads must be 256, 512 or 1024");
        c->prm.block_threads = (uint32_t)v;
    } else if (!strcmp(name, "ordered_output")) {
        if (v != 0 && v != 1) return fail(c, DIM3G_ERR_INVALID, "ordered_output must be 0 or 1");
        c->prm.ordered = v == 1;
    } else if (!strcmp(name, "dense_block")) {
        if (v < 0 || v > 2) return fail(c, DIM3G_ERR_INVALID, "dense_block must be 0, 1 or 2");
        c->prm.dense = (uint32_t)v;
    } else if (!strcmp(name, "dense_k_max")) {
        if (v < 32 || v > 4096) return fail(c, DIM3G_ERR_INVALID, "dense_k_max must be in 32..4096");
        c->prm.dense_k_max = (uint32_t)v;
    } else if (!strcmp(name, "dense_mem_mb")) {
        if (v < 1 || v > (1 << 20)) return fail(c, DIM3G_ERR_INVALID, "dense_mem_mb must be in 1..2^20");
        c->prm.dense_mem = (uint64_t)v << 20;
    } else if (!strcmp(name, "sized_tables")) {
        if (v != 0 && v != 1) return fail(c, DIM3G_ERR_INVALID, "sized_tables must be 0 or 1");
        c->prm.sized_tables = v == 1;
    } else if (!strcmp(name, "table_slack_pct")) {
        if (v < 5 || v > 1000) return fail(c, DIM3G_ERR_INVALID, "table_slack_pct must be in 5..1000");
        c->prm.table_slack_pct = (uint32_t)v;
    } else if (!strcmp(name, "block_split")) {
        if (v != 0 && v != 1) return fail(c, DIM3G_ERR_INVALID, "block_split must be 0 or 1");
        c->prm.block_split = (uint32_t)v;
    } else if (!strcmp(name, "prefetch_rows")) {
        if (v != 0 && v != 1) return fail(c, DIM3G_ERR_INVALID, "prefetch_rows must be 0 or 1");
        c->prm.prefetch_rows = (uint32_t)v;
    } else if (!strcmp(name, "stream_rows")) {
        if (v != 0 && v != 1) return fail(c, DIM3G_ERR_INVALID, "stream_rows must be 0 or 1");
        c->prm.stream_rows = (uint32_t)v;
    } else if (!strcmp(name, "keep_roles")) {
        if (v != 0 && v != 1) return fail(c, DIM3G_ERR_INVALID, "keep_roles must be 0 or 1");
        c->prm.keep_roles = v == 1;
    } else {
        return fail(c, DIM3G_ERR_INVALID, "unknown parameter %s", name);
    }
    return DIM3G_OK;
}

int dim3g_get_param(const dim3g_ctx* c, const char* name, int64_t* v) {
    if (!c || !name || !v) return DIM3G_ERR_INVALID;
    if (!strcmp(name, "warp_slots_log2")) *v = c->prm.warp_lg;
    else if (!strcmp(name, "block_slots_log2")) *v = c->prm.block_lg;
    else if (!strcmp(name, "tile_bits_log2")) *v = c->prm.tile_lg;
    else if (!strcmp(name, "ordered_output")) *v = c->prm.ordered ? 1 : 0;
    else if (!strcmp(name, "block_threads")) *v = c->prm.block_threads;
    else if (!strcmp(name, "host_direct_output")) *v = c->prm.host_direct ? 1 : 0;
    else if (!strcmp(name, "cta_walk")) *v = c->prm.cta_rr;
    else if (!strcmp(name, "dense_block")) *v = c->prm.dense;
    else if (!strcmp(name, "dense_k_max")) *v = c->prm.dense_k_max;
    else if (!strcmp(name, "dense_mem_mb")) *v = (int64_t)(c->prm.dense_mem >> 20);
    else if (!strcmp(name, "keep_roles")) *v = c->prm.keep_roles ? 1 : 0;
    else if (!strcmp(name, "stream_rows")) *v = c->prm.stream_rows;
    else if (!strcmp(name, "prefetch_rows")) *v = c->prm.prefetch_rows;
    else if (!strcmp(name, "block_split")) *v = c->prm.block_split;
    else if (!strcmp(name, "sized_tables")) *v = c->prm.sized_tables ? 1 : 0;
    else if (!strcmp(name, "table_slack_pct")) *v = c->prm.table_slack_pct;
    else return DIM3G_ERR_INVALID;
    return DIM3G_OK;
}

int dim3g_trim(dim3g_ctx* c) {
    if (!c) return DIM3G_ERR_INVALID;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    c->ws.release();
    if (c->d_in) cudaFree(c->d_in);
    if (c->d_out) cudaFree(c->d_out);
    if (c->d_sum) cudaFree(c->d_sum);
    c->d_in = c->d_out = c->d_sum = nullptr;
    c->d_in_bytes = c->d_out_bytes = c->d_sum_bytes = 0;
    return DIM3G_OK;
}

int dim3g_join_project(dim3g_ctx* c, const uint32_t* R, uint64_t nR, const uint32_t* S, uint64_t nS,
                       uint32_t** out_xz, uint64_t* n_out) {
    if (!out_xz) return fail(c, DIM3G_ERR_INVALID, "null output pointer");
    return host_join(c, R, nR, S, nS, false, out_xz, nullptr, nullptr, 0, n_out);
}

int dim3g_join_project_into(dim3g_ctx* c, const uint32_t* R, uint64_t nR, const uint32_t* S, uint64_t nS,
                            uint32_t* out_xz, uint64_t capacity, uint64_t* n_out) {
    if (!out_xz) return fail(c, DIM3G_ERR_INVALID, "null output buffer");
    return host_join(c, R, nR, S, nS, false, nullptr, nullptr, out_xz, capacity, n_out);
}

int dim3g_join_project_device(dim3g_ctx* c, const uint32_t* dR, uint64_t nR, const uint32_t* dS, uint64_t nS,
                              uint32_t* d_out, uint64_t capacity, uint64_t* n_out) {
    if (!c || !n_out || (nR && !dR) || (nS && !dS) || (capacity && !d_out))
        return fail(c, DIM3G_ERR_INVALID, "null argument");
    if (!aligned8(dR) || !aligned8(dS) || !aligned8(d_out)) return fail(c, DIM3G_ERR_INVALID, "device pointers must be 8-byte aligned");
    CU(cudaSetDevice(c->device));
    const bool swap = !c->prm.keep_roles && nR < nS;
    DeviceOut d{(uint2*)d_out, nullptr, capacity};
    JoinPlan jp{(const uint2*)(swap ? dS : dR), swap ? nS : nR, (const uint2*)(swap ? dR : dS), swap ? nR : nS,
                swap, false, false, !c->prm.ordered, OutPrep{prep_device, peek_device, &d}};
    return run_join(c, jp, n_out);
}

int dim3g_join_project_count_device(dim3g_ctx* c, const uint32_t* dR, uint64_t nR, const uint32_t* dS, uint64_t nS,
                                    uint64_t* n_out) {
    if (!c || !n_out || (nR && !dR) || (nS && !dS)) return fail(c, DIM3G_ERR_INVALID, "null argument");
    if (!aligned8(dR) || !aligned8(dS)) return fail(c, DIM3G_ERR_INVALID, "device pointers must be 8-byte aligned");
    CU(cudaSetDevice(c->device));
    const bool swap = !c->prm.keep_roles && nR < nS;
    DeviceOut d{nullptr, nullptr, 0};
    JoinPlan jp{(const uint2*)(swap ? dS : dR), swap ? nS : nR, (const uint2*)(swap ? dR : dS), swap ? nR : nS,
                swap, false, true, false, OutPrep{prep_device, peek_device, &d}};
    return run_join(c, jp, n_out);
}

int dim3g_join_count(dim3g_ctx* c, const uint32_t* R, uint64_t nR, const uint32_t* S, uint64_t nS,
                     uint32_t** out_xz, uint64_t** out_cnt, uint64_t* n_out) {
    if (!out_xz || !out_cnt) return fail(c, DIM3G_ERR_INVALID, "null output pointer");
    return host_join(c, R, nR, S, nS, true, out_xz, out_cnt, nullptr, 0, n_out);
}

int dim3g_join_count_device(dim3g_ctx* c, const uint32_t* dR, uint64_t nR, const uint32_t* dS, uint64_t nS,
                            uint32_t* d_out_xz, uint64_t* d_out_cnt, uint64_t capacity, uint64_t* n_out) {
    if (!c || !n_out || (nR && !dR) || (nS && !dS) || (capacity && (!d_out_xz || !d_out_cnt)))
        return fail(c, DIM3G_ERR_INVALID, "null argument");
    if (!aligned8(dR) || !aligned8(dS) || !aligned8(d_out_xz) || !aligned8(d_out_cnt))
        return fail(c, DIM3G_ERR_INVALID, "device pointers must be 8-byte aligned");
    CU(cudaSetDevice(c->device));
    const bool swap = !c->prm.keep_roles && nR < nS;
    DeviceOut d{(uint2*)d_out_xz, (unsigned long long*)d_out_cnt, capacity};
    JoinPlan jp{(const uint2*)(swap ? dS : dR), swap ? nS : nR, (const uint2*)(swap ? dR : dS), swap ? nR : nS,
                swap, true, false, false, OutPrep{prep_device, peek_device, &d}};
    return run_join(c, jp, n_out);
}

}  // extern "C"

namespace {

int run_summary(dim3g_ctx* c, const uint32_t* dR, uint64_t nR, const uint32_t* dS, uint64_t nS, bool aggregate,
                uint32_t tiles, uint32_t lo, uint32_t hi, dim3g_tile_summary* out) {
    if (!c || !out || (nR && !dR) || (nS && !dS)) return fail(c, DIM3G_ERR_INVALID, "null argument");
    if (tiles == 0 || tiles > (1u << 20) || (tiles & (tiles - 1)) || lo >= hi || hi > tiles)
        return fail(c, DIM3G_ERR_INVALID, "tiles must be a power of two <= 2^20 and lo < hi <= tiles");
    if (!aligned8(dR) || !aligned8(dS)) return fail(c, DIM3G_ERR_INVALID, "device pointers must be 8-byte aligned");
    CU(cudaSetDevice(c->device));
    memset(out, 0, (size_t)tiles * sizeof(dim3g_tile_summary));
    // the accumulators live outside the per-call workspace (reset by run_join)
    int r = ensure_dev(c, &c->d_sum, &c->d_sum_bytes, (size_t)tiles * 24);
    if (r) return r;
    CU(cudaMemsetAsync(c->d_sum, 0, (size_t)tiles * 24, c->stream));
    const bool swap = !c->prm.keep_roles && nR < nS;
    JoinPlan jp{(const uint2*)(swap ? dS : dR), swap ? nS : nR, (const uint2*)(swap ? dR : dS), swap ? nR : nS,
                swap, aggregate, false, false, OutPrep{nullptr, nullptr, nullptr}};
    jp.sum = SumAcc{(unsigned long long*)c->d_sum, tiles - 1, lo, hi};
    uint64_t n = 0;
    r = run_join(c, jp, &n);
    if (r) return r;
    CU(cudaMemcpyAsync(out, c->d_sum, (size_t)tiles * 24, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    uint64_t groups = 0;
    for (uint32_t t = 0; t < tiles; t++) groups += out[t].groups;
    c->stats.n_out = groups;
    return DIM3G_OK;
}

}  // namespace

extern "C" {

int dim3g_join_project_summary(dim3g_ctx* c, const uint32_t* dR, uint64_t nR, const uint32_t* dS, uint64_t nS,
                               uint32_t tiles, uint32_t tile_lo, uint32_t tile_hi, dim3g_tile_summary* out) {
    return run_summary(c, dR, nR, dS, nS, false, tiles, tile_lo, tile_hi, out);
}

int dim3g_join_count_summary(dim3g_ctx* c, const uint32_t* dR, uint64_t nR, const uint32_t* dS, uint64_t nS,
                             uint32_t tiles, uint32_t tile_lo, uint32_t tile_hi, dim3g_tile_summary* out) {
    return run_summary(c, dR, nR, dS, nS, true, tiles, tile_lo, tile_hi, out);
}

// The product kernel of the dense block on all-ones operands, timed with
// events on the context's stream (best of 5 launches after one warm-up): at
// K = 4096 over 8 tiles of 128 x 256 per SM (the MMA rate), and at K = 128
// over 8 and over 16 tiles per SM (a tile's fixed time: the difference
// divided by 8, so the launch's own fixed costs cancel); then a
// device-to-device copy of 512 MB.
int dim3g_calibrate(dim3g_ctx* c, dim3g_calibration* out) {
    if (!c || !out) return DIM3G_ERR_INVALID;
    memset(out, 0, sizeof *out);
    CU(cudaSetDevice(c->device));
    c->ws.reset();
    cudaStream_t st = c->stream;
    const int sm = c->sm_count;
    const uint32_t nt = 16, mt = (uint32_t)(8 * sm + nt - 1) / nt;  // >= 8 tiles per SM
    const uint64_t Mp = (uint64_t)mt * kDenseBM, Np = (uint64_t)nt * kDenseBN;
    const uint32_t kmax = 4096;
    uint8_t* A = ws_get<uint8_t>(c, Mp * kmax);
    uint8_t* B = ws_get<uint8_t>(c, Np * kmax);  // also 2 Np rows of 128 bytes
    uint32_t* D = ws_get<uint32_t>(c, Mp * (2 * Np / 32));
    unsigned int* err = ws_get<unsigned int>(c, 1);
    const size_t copy_bytes = (size_t)512 << 20;
    char* src = ws_get<char>(c, copy_bytes);
    char* dst = ws_get<char>(c, copy_bytes);
    if (!A || !B || !D || !err || !src || !dst) return fail(c, DIM3G_ERR_NOMEM, "workspace allocation failed (calibrate)");
    CU(cudaMemsetAsync(A, kFp8One, Mp * kmax, st));
    CU(cudaMemsetAsync(B, kFp8One, Np * kmax, st));
    CU(cudaMemsetAsync(err, 0, 4, st));
    CU(cudaMemsetAsync(src, 1, copy_bytes, st));
    // runs: {K, column tiles}
    const uint32_t kps[3] = {kmax, kDenseBK, kDenseBK}, nts[3] = {nt, nt, 2 * nt};
    float best[3] = {1e30f, 1e30f, 1e30f};
    for (int which = 0; which < 3; which++) {
        const uint32_t Kp = kps[which], ntw = nts[which];
        const uint64_t Npw = (uint64_t)ntw * kDenseBN, Wd = Npw / 32;
        const unsigned grid = (unsigned)((uint64_t)mt * ntw < (uint64_t)sm ? (uint64_t)mt * ntw : (uint64_t)sm);
        CUtensorMap mA, mB;
        int r = dense_map(c, &mA, A, Mp, Kp, kDenseBM);
        if (!r) r = dense_map(c, &mB, B, Npw, Kp, kDenseBN);
        if (r) return r;
        for (int rep = 0; rep < 6; rep++) {  // the first launch warms up
            CU(cudaEventRecord(c->evd[0], st));
            k_dense_mma<kDenseBits><<<grid, kDenseThreads, kDenseSmem, st>>>(mA, mB, D, (uint32_t)Wd, mt, ntw,
                                                                              Kp / kDenseBK, err, DenseSum{});
            CHECK_LAUNCH();
            CU(cudaEventRecord(c->evd[1], st));
            CU(cudaEventSynchronize(c->evd[1]));
            float ms = 0;
            CU(cudaEventElapsedTime(&ms, c->evd[0], c->evd[1]));
            if (rep && ms < best[which]) best[which] = ms;
        }
    }
    float copy_ms = 1e30f;
    for (int rep = 0; rep < 4; rep++) {
        CU(cudaEventRecord(c->evd[0], st));
        CU(cudaMemcpyAsync(dst, src, copy_bytes, cudaMemcpyDeviceToDevice, st));
        CU(cudaEventRecord(c->evd[1], st));
        CU(cudaEventSynchronize(c->evd[1]));
        float ms = 0;
        CU(cudaEventElapsedTime(&ms, c->evd[0], c->evd[1]));
        if (rep && ms < copy_ms) copy_ms = ms;
    }
    unsigned int h_err = 0;
    CU(cudaMemcpy(&h_err, err, 4, cudaMemcpyDeviceToHost));
    if (h_err) return fail(c, DIM3G_ERR_DEVICE, "calibration product reported flags %u", h_err);
    const unsigned grid0 = (unsigned)((uint64_t)mt * nt < (uint64_t)sm ? (uint64_t)mt * nt : (uint64_t)sm);
    const double tiles_per_sm = ceil((double)mt * nt / grid0);
    const double flops = 2.0 * (double)Mp * (double)Np * kmax;
    const double tile_s = (best[2] > best[1] ? best[2] - best[1] : best[1]) * 1e-3 / tiles_per_sm;
    out->fp8_tflops = (float)(flops / (best[0] * 1e-3) / 1e12);
    out->tile_us = (float)(tile_s * 1e6);
    out->hbm_gbs = (float)(2.0 * copy_bytes / (copy_ms * 1e-3) / 1e9);
    c->cm.sm_flops = flops / (best[0] * 1e-3) / grid0;
    c->cm.tile_s = tile_s;
    c->cm.dense_bw = 2.0 * copy_bytes / (copy_ms * 1e-3);
    c->cm.calibrated = true;
    out->sparse_gbs = (float)(c->cm.sparse_bw / 1e9);
    return DIM3G_OK;
}

}  // extern "C"

// ========================================================= L+S mapper ABI
namespace {

int mapper_stage(dim3g_mapper* m, const uint32_t* keys, uint64_t n, uint32_t** dkeys, int32_t** dids) {
    dim3g_ctx* c = m->ctx;
    c->ws.reset();
    *dkeys = ws_get<uint32_t>(c, n);
    *dids = ws_get<int32_t>(c, n);
    if (!*dkeys || !*dids) return fail(c, DIM3G_ERR_NOMEM, "mapper staging allocation failed");
    CU(cudaMemcpyAsync(*dkeys, keys, n * 4, cudaMemcpyHostToDevice, c->stream));
    return DIM3G_OK;
}

int mapper_reserve(dim3g_mapper* m, uint64_t want_keys) {
    dim3g_ctx* c = m->ctx;
    uint64_t need = next_pow2(want_keys * 2 < 1024 ? 1024 : want_keys * 2);
    if (need <= m->cap) return DIM3G_OK;
    unsigned long long* ns = nullptr;
    if (cudaMalloc(&ns, need * 8) != cudaSuccess) {
        cudaGetLastError();
        return fail(c, DIM3G_ERR_NOMEM, "mapper table allocation failed");
    }
    CU(cudaMemsetAsync(ns, 0xff, need * 8, c->stream));
    if (m->slots) {
        uint32_t* err = ws_get<uint32_t>(c, 1);
        if (!err) return fail(c, DIM3G_ERR_NOMEM, "mapper scratch allocation failed");
        CU(cudaMemsetAsync(err, 0, 4, c->stream));
        k_mapper_rehash<<<grid_for(m->cap, c->sm_count), 256, 0, c->stream>>>(DevTable{m->slots, m->cap - 1},
                                                                             DevTable{ns, need - 1}, err);
        CHECK_LAUNCH();
        CU(cudaStreamSynchronize(c->stream));
        cudaFree(m->slots);
    }
    m->slots = ns;
    m->cap = need;
    return DIM3G_OK;
}

}  // namespace

extern "C" {

int dim3g_mapper_create(dim3g_ctx* c, uint64_t hint, dim3g_mapper** out) {
    if (!c || !out) return DIM3G_ERR_INVALID;
    *out = nullptr;
    CU(cudaSetDevice(c->device));
    dim3g_mapper* m = new dim3g_mapper();
    m->ctx = c;
    int r = mapper_reserve(m, hint);
    if (r) {
        delete m;
        return r;
    }
    CU(cudaStreamSynchronize(c->stream));
    *out = m;
    return DIM3G_OK;
}

void dim3g_mapper_destroy(dim3g_mapper* m) {
    if (!m) return;
    cudaSetDevice(m->ctx->device);
    cudaStreamSynchronize(m->ctx->stream);
    if (m->slots) cudaFree(m->slots);
    delete m;
}

int dim3g_mapper_insert(dim3g_mapper* m, const uint32_t* keys, uint64_t n, int32_t* ids) {
    if (!m) return DIM3G_ERR_INVALID;
    dim3g_ctx* c = m->ctx;
    if ((n && (!keys || !ids)) || n >= 0x7FFFFFFFull) return fail(c, DIM3G_ERR_INVALID, "bad mapper batch");
    if (n == 0) return DIM3G_OK;
    if (m->cnt + (int64_t)n >= 0x7FFFFFFFll) return fail(c, DIM3G_ERR_UNSUPPORTED, "mapper id space exhausted");
    CU(cudaSetDevice(c->device));
    int r = mapper_reserve(m, (uint64_t)m->nkeys + n);
    if (r) return r;
    uint32_t* dk;
    int32_t* di;
    if ((r = mapper_stage(m, keys, n, &dk, &di))) return r;
    uint64_t* bsum = ws_get<uint64_t>(c, scan_storage(n));
    unsigned long long* total = ws_get<unsigned long long>(c, 1);
    uint32_t* err = ws_get<uint32_t>(c, 1);
    if (!bsum || !total || !err) return fail(c, DIM3G_ERR_NOMEM, "mapper scratch allocation failed");
    cudaStream_t st = c->stream;
    DevTable t{m->slots, m->cap - 1};
    CU(cudaMemsetAsync(err, 0, 4, st));
    k_mapper_claim<<<grid_for(n, c->sm_count), 256, 0, st>>>(t, dk, n, err);
    CHECK_LAUNCH();
    SCAN(FirstOccSrc{t, dk}, AssignNewIdDst{t, dk, (long long)m->cnt}, n, bsum, total);
    k_mapper_gather<<<grid_for(n, c->sm_count), 256, 0, st>>>(t, dk, n, di);
    CHECK_LAUNCH();
    unsigned long long h_total = 0;
    uint32_t h_err = 0;
    CU(cudaMemcpyAsync(ids, di, n * 4, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&h_total, total, 8, cudaMemcpyDeviceToHost, st));
    CU(cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, st));
    CU(cudaStreamSynchronize(st));
    if (h_err) return fail(c, DIM3G_ERR_DEVICE, "mapper probe bound violated");
    m->cnt += (int64_t)h_total;
    m->nkeys += (int64_t)h_total;
    return DIM3G_OK;
}

int dim3g_mapper_find(dim3g_mapper* m, const uint32_t* keys, uint64_t n, int32_t* ids) {
    if (!m) return DIM3G_ERR_INVALID;
    dim3g_ctx* c = m->ctx;
    if (n && (!keys || !ids)) return fail(c, DIM3G_ERR_INVALID, "bad mapper batch");
    if (n == 0) return DIM3G_OK;
    CU(cudaSetDevice(c->device));
    uint32_t* dk;
    int32_t* di;
    int r = mapper_stage(m, keys, n, &dk, &di);
    if (r) return r;
    k_mapper_find<<<grid_for(n, c->sm_count), 256, 0, c->stream>>>(DevTable{m->slots, m->cap - 1}, dk, n, di);
    CHECK_LAUNCH();
    CU(cudaMemcpyAsync(ids, di, n * 4, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    return DIM3G_OK;
}

int64_t dim3g_mapper_size(const dim3g_mapper* m) { return m ? m->cnt : -1; }

int dim3g_mapper_clear(dim3g_mapper* m) {
    if (!m) return DIM3G_ERR_INVALID;
    dim3g_ctx* c = m->ctx;
    CU(cudaSetDevice(c->device));
    CU(cudaMemsetAsync(m->slots, 0xff, m->cap * 8, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    m->nkeys = 0;
    return DIM3G_OK;
}

int dim3g_mapper_set_cnt(dim3g_mapper* m, int64_t cnt) {
    if (!m || cnt < 0 || cnt >= 0x7FFFFFFFll) return DIM3G_ERR_INVALID;
    m->cnt = cnt;
    return DIM3G_OK;
}

}  // extern "C"

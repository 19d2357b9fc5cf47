/*
 * dim3gpu.h -- C ABI of the GB300 (sm_103a) join-project / join-aggregate
 * path.  Plain pointers and sizes only.  Every entry point returns a status
 * code (DIM3G_OK == 0); dim3g_last_error() gives a one-line reason.
 *
 * The operation replaces the reference's DIM3 hybrid join-project
 * (schencoding/JoinProject-DIM3).  Inputs are arrays of interleaved uint32
 * pairs, the memory layout of the reference's myvector<pair<int,int>>:
 *   R = (x, y) pairs, S = (z, y) pairs.
 * The result is the distinct set {(P.first, Q.first) | P.y == Q.y} where P is
 * the larger input -- R when |R| >= |S|, otherwise S, exactly the reference's
 * swap (dim3.hpp:993-994), so a smaller R yields (z, x) pairs.  The order of
 * the pairs is unspecified (the reference's order is an artifact of its id
 * assignment too); with the "ordered_output" knob set, pairs come grouped by
 * their first value, groups in a fixed order.
 *
 * Limits: |R|, |S| < 2^32 - 1 tuples; the distinct key domains below 2^31;
 * output counts are 64-bit (no wrap at 2^31, unlike myvector's uint32 count).
 *
 * Threading: a context owns one CUDA stream and a workspace; calls on one
 * context are serialised by the caller, calls on different contexts may run
 * concurrently.
 */
#ifndef DIM3GPU_H
#define DIM3GPU_H
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

#define DIM3G_OK 0
#define DIM3G_ERR_INVALID 1     /* bad argument */
#define DIM3G_ERR_CUDA 2        /* a CUDA runtime call failed */
#define DIM3G_ERR_NOMEM 3       /* device or host allocation failed */
#define DIM3G_ERR_CAPACITY 4    /* output buffer too small; *n_out = pairs needed */
#define DIM3G_ERR_DEVICE 5      /* a kernel reported a violated bound */
#define DIM3G_ERR_UNSUPPORTED 6 /* input beyond the supported limits */

typedef struct dim3g_ctx dim3g_ctx;

/* Per-call figures of the last call on a context. */
typedef struct {
    uint64_t n_big, n_small;   /* tuples of the larger / smaller input */
    uint64_t n_small_kept;     /* smaller-input tuples surviving the semi-join */
    uint64_t out_j;            /* exact join size sum_b degP(b) * degQ(b) */
    uint64_t n_out;            /* distinct output pairs (groups) */
    uint32_t swapped;          /* 1 when |R| < |S| */
    uint32_t nx, ny, nz;       /* distinct first / join / second values */
    uint32_t rows_warp, rows_block, rows_bitmap, rows_dense; /* x rows per kernel class */
    uint32_t z_tiles;          /* z tiles of the bitmap class */
    uint32_t heavy_y;          /* join values whose S rows went to the dense block */
    float ms_map;              /* device ms: hash build, probe, id assignment */
    float ms_csr;              /* device ms: CSR builds, row binning */
    float ms_count;            /* device ms: count pass + offsets */
    float ms_write;            /* device ms: write pass */
    float ms_total;            /* device ms: whole call (inputs resident) */
    uint64_t launches;         /* kernels launched on this context since creation */
    float ms_count_cls[3];     /* count pass device ms per row kernel: bitmap, block, warp */
    float ms_write_cls[3];     /* write pass device ms per row kernel: bitmap, block, warp */
    uint64_t out_j_cls[3];     /* candidates (join tuples) per row kernel: bitmap, block, warp */
    uint64_t n_out_cls[3];     /* distinct pairs per row kernel (single pass): bitmap, block, warp */
    float ms_dense[3];         /* dense block device ms: selection + operands, tensor-core product, light pass */
    uint32_t dense_kp;         /* K of the dense product (heavy_y padded to 128) */
    uint64_t dense_light;      /* candidates of the dense block's rows through light join values (estimate) */
    uint32_t dense_skip;       /* why the dense block did not run: 0 it ran, 1 off or materialised COUNT, 2 no or
                                  too little heavy work, 3 no budget, 4 cost model, 5 a multiplicity above 16
                                  (summaries), 6 light buckets too large (summaries) */
    uint32_t dense_bucket_max; /* largest per-tile light bucket (summaries) */
    uint64_t table_slots;      /* slots of the three mapping hash tables (sized by a distinct-key sketch) */
    uint32_t table_rebuilds;   /* 1 when the sketch-sized tables overfilled and the mapping ran again at full size */
    uint32_t pad0;
} dim3g_stats;

/* ---- context ------------------------------------------------------- */
int dim3g_create(int device, dim3g_ctx** ctx);
void dim3g_destroy(dim3g_ctx* ctx);
/* Use the caller's cudaStream_t for all work of this context (NULL restores
 * the context's own stream). */
int dim3g_set_stream(dim3g_ctx* ctx, void* cuda_stream);
const char* dim3g_last_error(const dim3g_ctx* ctx);
int dim3g_get_stats(const dim3g_ctx* ctx, dim3g_stats* out);
/* Tuning knobs, validated on set: "warp_slots_log2" (5..14, warp-class hash
 * set size), "block_slots_log2" (8..14, block-class hash set size),
 * "tile_bits_log2" (10..20, bitmap-class z tile width), "ordered_output" (0: one expansion per row, rows in unspecified order;
 * 1: count pass + write pass, pairs grouped by first value),
 * "block_threads" (256, 512 or 1024: CTA width of the block class),
 * "host_direct_output" (1: pinned host outputs written directly),
 * "cta_walk" (how CTA rows share candidates among warps: 0 = the row's
 * segment table staged in shared memory and its candidates split evenly,
 * 1 = warps take whole 32-entry chunks in turn, 2 = every chunk split
 * across the warps, 3 = every warp an equal share of the row's candidates
 * over the chunks staged in shared memory), "dense_block" (the heavy rows' join through their
 * heaviest join values as one boolean product on the tensor cores: 0 off,
 * 1 when the cost model prefers it, 2 whenever its bitmap fits),
 * "dense_k_max" (32..4096: most join values in that product),
 * "dense_mem_mb" (bitmap budget of that product, default 16384: it takes as
 * many heavy rows as their x z bitmap fits, the largest first),
 * "sized_tables" (1: the mapping's hash tables are sized by a distinct-key
 * sketch to fit the L2 where keys repeat; 0: by the tuple counts),
 * "table_slack_pct" (5..1000, default 150: slots of a sketch-sized table per
 * estimated distinct key, in percent; a table that overfills is rebuilt at
 * full size),
 * "stream_rows" (1: bitmap-class rows of the single pass streamed into shared
 * memory by bulk copies -- exact, measured slower on the 2-hop),
 * "prefetch_rows" (1: block-class rows of the single pass fetched ahead by a
 * producer warp -- exact, measured slower on the 2-hop),
 * "block_split" (1, default: the single pass runs block-class rows in three
 * launches by hash-set size -- 2^(b-2), 2^(b-1) and 2^b slots for
 * block_slots_log2 = b -- the two smaller with 256-thread CTAs, so more rows
 * are in flight per SM; 0: one launch of 2^b-slot CTAs),
 * "keep_roles" (0: the larger relation drives the join, the reference's
 * swap at dim3.hpp:993-994, so a smaller R yields (S.first, R.first) pairs;
 * 1: R always drives and pairs are always (R.first, S.first) -- for joining
 * an A-slice of R with all of S, which keeps the whole join's row shape). */
int dim3g_set_param(dim3g_ctx* ctx, const char* name, int64_t value);
int dim3g_get_param(const dim3g_ctx* ctx, const char* name, int64_t* value);
/* Release device memory cached by the context (workspace, staging). */
int dim3g_trim(dim3g_ctx* ctx);

/* ---- join-project --------------------------------------------------
 * Replaces DIM3<int,int,int,...>::doJoinProject (dim3.hpp:982-1055) and
 * DIM3_parallel<...>::doJoinProject_parallel (dim3_parallel.hpp:137-210):
 * the same R, S and result, with the result as interleaved pairs. */

/* Host input, result in a malloc'd host array (free with free()); this is the
 * ownership of the reference's myvector result (malloc/realloc'd data). */
int dim3g_join_project(dim3g_ctx* ctx, const uint32_t* R_xy, uint64_t nR, const uint32_t* S_zy,
                       uint64_t nS, uint32_t** out_xz, uint64_t* n_out);
/* Host input, result into the caller's host buffer of `capacity` pairs.  A
 * pinned (page-locked, mapped) buffer is written by the kernels directly,
 * overlapping the transfer with the join ("host_direct_output" = 0 turns
 * this off); a pageable one is filled by a copy after the join.  On
 * DIM3G_ERR_CAPACITY *n_out holds the pairs needed and the buffer's contents
 * are unspecified. */
int dim3g_join_project_into(dim3g_ctx* ctx, const uint32_t* R_xy, uint64_t nR, const uint32_t* S_zy,
                            uint64_t nS, uint32_t* out_xz, uint64_t capacity, uint64_t* n_out);
/* Device-resident input and output: d_R, d_S, d_out are device pointers
 * (8-byte aligned).  On DIM3G_ERR_CAPACITY *n_out holds the pairs needed and
 * the buffer's contents are unspecified. */
int dim3g_join_project_device(dim3g_ctx* ctx, const uint32_t* d_R, uint64_t nR, const uint32_t* d_S,
                              uint64_t nS, uint32_t* d_out, uint64_t capacity, uint64_t* n_out);
/* Count only: the number of distinct pairs, no pairs written. */
int dim3g_join_project_count_device(dim3g_ctx* ctx, const uint32_t* d_R, uint64_t nR, const uint32_t* d_S,
                                    uint64_t nS, uint64_t* n_out);

/* ---- join-aggregate COUNT(*) GROUP BY (x, z) -------------------------
 * Replaces DIM3JoinAggregate<...>::doJoinAggregate (dim3.hpp:1313-1373) with
 * a COUNT aggregate: for every distinct (P.first, Q.first) the number of
 * joining tuple pairs, exact in 64 bits. */
int dim3g_join_count(dim3g_ctx* ctx, const uint32_t* R_xy, uint64_t nR, const uint32_t* S_zy, uint64_t nS,
                     uint32_t** out_xz, uint64_t** out_cnt, uint64_t* n_out);
int dim3g_join_count_device(dim3g_ctx* ctx, const uint32_t* d_R, uint64_t nR, const uint32_t* d_S, uint64_t nS,
                            uint32_t* d_out_xz, uint64_t* d_out_cnt, uint64_t capacity, uint64_t* n_out);

/* ---- summaries: results too large to materialise ----------------------
 * No counterpart in the reference.  Nothing is written to an output; the
 * pairs (or groups) are summarised per A-tile, t(a) = murmur3 fmix32(a) &
 * (tiles - 1) of the pair's first value a:
 *   groups     distinct pairs of the tile
 *   count_sum  sum of the groups' counts (COUNT; the tile's OUT_J), or
 *              groups (join-project)
 *   hash       sum mod 2^64 of pair_hash(a, c) (join-project) or of
 *              mix64(pair_hash(a, c) + count) (COUNT), pair_hash = mix64 =
 *              the splitmix64 finaliser of a << 32 | c
 * Only tiles in [tile_lo, tile_hi) are computed (rows of other tiles are
 * skipped), so a join too large for one call is covered in slices, and a
 * slice can be checked on the CPU from its rows of R alone.  tiles: a power
 * of two <= 2^20; out: host array of `tiles` entries (others zero).  Device
 * inputs as for dim3g_join_project_device. */
typedef struct {
    uint64_t groups, count_sum, hash;
} dim3g_tile_summary;
int dim3g_join_project_summary(dim3g_ctx* ctx, const uint32_t* d_R, uint64_t nR, const uint32_t* d_S, uint64_t nS,
                               uint32_t tiles, uint32_t tile_lo, uint32_t tile_hi, dim3g_tile_summary* out);
int dim3g_join_count_summary(dim3g_ctx* ctx, const uint32_t* d_R, uint64_t nR, const uint32_t* d_S, uint64_t nS,
                             uint32_t tiles, uint32_t tile_lo, uint32_t tile_hi, dim3g_tile_summary* out);

/* ---- allocation-free join-project ------------------------------------
 * No counterpart in the reference.  For callers that must not allocate
 * device memory where they need the join: code under a custom or
 * fixed-budget allocator, hosts that preallocate everything at start-up,
 * and pipelines that cannot afford the synchronisation an allocation may
 * bring.  Device inputs, the caller's output buffer, and all scratch in one
 * fixed array inside the library (about 19 MB, held on every GPU that loads
 * the library until the process exits); it calls no allocating routine.
 * Limits: the larger relation holds at most DIM3G_NOALLOC_MAX_TUPLES tuples
 * and the result at most DIM3G_NOALLOC_MAX_PAIRS distinct pairs; beyond
 * either it returns DIM3G_ERR_UNSUPPORTED.  The first call on a device looks
 * up the array's device address (once per device, with that device
 * current); make that first call before any stream capture.  All calls share
 * the array: calls that overlap on the GPU race, so serialise them.  The
 * result set, *n_out and DIM3G_ERR_CAPACITY are as for
 * dim3g_join_project_device.  d_R, d_S and d_out must be 8-byte aligned
 * (DIM3G_ERR_INVALID otherwise, before anything runs on the GPU).  An error
 * already pending on the calling thread's CUDA state is reported as
 * DIM3G_ERR_CUDA and left in place.  cuda_stream is a cudaStream_t (NULL:
 * the default stream), synchronised before the call returns. */
#define DIM3G_NOALLOC_MAX_TUPLES (1u << 18)
#define DIM3G_NOALLOC_MAX_PAIRS (1u << 20)
int dim3g_join_project_noalloc(const uint32_t* d_R, uint64_t nR, const uint32_t* d_S, uint64_t nS,
                               uint32_t* d_out, uint64_t capacity, uint64_t* n_out, void* cuda_stream);

/* ---- resident relation sets and many-query passes ---------------------
 * No counterpart in the reference, whose entry points take one join at a
 * time.  A relation set builds on the GPU, for all its relations in one
 * pass, each relation's value -> id maps and both CSR forms (the relation
 * as R, grouped by its first column; as S, grouped by its y column) and
 * keeps them in device memory.  A join of two relations of a set then skips
 * hashing and CSR construction: it costs a y-id translation and the
 * expansion.  dim3g_relset_join runs many such joins in one pass, the rows
 * of all queries sharing the row kernels.
 * Per query the result set is that of dim3g_join_project_device (R =
 * relation r, S = relation s; the larger relation drives the rows, so a
 * smaller R yields (z, x) pairs and `swapped` = 1) or, for DIM3G_OP_COUNT,
 * that of dim3g_join_count_device; pairs and groups come in unspecified
 * order. */
typedef struct dim3g_relset dim3g_relset;
typedef struct {
    const uint32_t* d_pairs; /* device (first, y) pairs, 8-byte aligned */
    uint64_t n;              /* tuples */
} dim3g_relation;
#define DIM3G_OP_PROJECT 0
#define DIM3G_OP_COUNT 1
typedef struct {
    uint32_t r, s;     /* relation indices: R(x, y), S(z, y) */
    uint32_t op;       /* DIM3G_OP_PROJECT or DIM3G_OP_COUNT */
    uint32_t swapped;  /* out: 1 when the pairs are (z, x) */
    uint32_t* d_out;   /* device pairs, `capacity` of them */
    uint64_t* d_cnt;   /* device counts, `capacity` of them (DIM3G_OP_COUNT) */
    uint64_t capacity;
    uint64_t n_out;    /* out: distinct pairs; on DIM3G_ERR_CAPACITY the pairs needed */
    uint64_t out_j;    /* out: joining tuple pairs (candidates) */
    int32_t status;    /* out: DIM3G_OK, DIM3G_ERR_CAPACITY or DIM3G_ERR_DEVICE */
    uint32_t pad;
} dim3g_query;
/* Builds the indexes of n relations; synchronous.  The pair arrays must stay
 * valid and unchanged while the set lives.  Limit: fewer than 2^32-1 tuples
 * in the whole set. */
int dim3g_relset_create(dim3g_ctx* ctx, const dim3g_relation* rels, uint32_t n, dim3g_relset** set);
void dim3g_relset_destroy(dim3g_relset* set);
/* Device bytes the set holds (indexes and query scratch). */
uint64_t dim3g_relset_bytes(const dim3g_relset* set);
/* Runs n queries over the set in one pass on the context's stream;
 * synchronous.  Each query gets its own status; the call returns DIM3G_OK
 * when all are DIM3G_OK, else the first failing status. */
int dim3g_relset_join(dim3g_relset* set, dim3g_query* q, uint32_t n);

/* Exact join size OUT_J of every ordered pair of the set's relations:
 * outj[r * n + s] = sum over y of deg_R(y) * deg_S(y) (R = relation r,
 * S = relation s; n = relations in the set).  One GPU pass; synchronous. */
int dim3g_relset_pair_outj(dim3g_relset* set, uint64_t* outj);

/* ---- serving: continuous batching over a resident relation set ---------
 * A server runs requests (a relation pair of the set and an op) on `lanes`
 * CUDA streams, each lane with its own query scratch.  Requests queue on
 * submit.  A lane that is free admits queued requests in arrival order
 * while their output reservations fit the budget, runs them as one query
 * pass and completes them; while one lane's pass runs on the GPU another
 * lane admits and launches the requests that arrived meanwhile, so passes
 * overlap on the device.  A request's reservation is
 * min(OUT_J, distinct R.first x distinct S.first) pairs (8 bytes each, plus
 * 8 for a COUNT), OUT_J exact from the set's pair matrix, so no request can
 * overflow its output.  Outputs are device memory held by the server until
 * the request is released.  budget_bytes bounds the device memory of the
 * whole serving system: the set, the lanes' scratch and every admitted
 * request's output.  Results are the same as from dim3g_relset_join. */
typedef struct dim3g_server dim3g_server;
typedef struct {
    uint64_t ticket;
    int32_t status;         /* DIM3G_OK or the request's error status */
    uint32_t swapped;       /* 1 when the pairs are (z, x) */
    uint64_t n_out, out_j;
    const uint32_t* d_out;  /* device pairs, valid until released */
    const uint64_t* d_cnt;  /* device counts (DIM3G_OP_COUNT) */
    double t_submit, t_start, t_done; /* seconds since the server started */
    uint32_t pass_size;     /* requests in the pass that ran it */
    uint32_t lane;
} dim3g_result;
int dim3g_server_create(dim3g_relset* set, uint32_t lanes, uint32_t max_batch, uint64_t budget_bytes,
                        dim3g_server** srv);
/* Queues a request; DIM3G_ERR_NOMEM if its reservation exceeds the output
 * budget (it could never be admitted). */
int dim3g_server_submit(dim3g_server* srv, uint32_t r, uint32_t s, uint32_t op, uint64_t* ticket);
/* Blocks until the request has completed and fills *out. */
int dim3g_server_wait(dim3g_server* srv, uint64_t ticket, dim3g_result* out);
/* Frees the request's output and returns its reservation to the budget. */
int dim3g_server_release(dim3g_server* srv, uint64_t ticket);
/* Completed requests, query passes run, output bytes reserved now, and the
 * output budget (budget_bytes less the set and the lanes' scratch). */
int dim3g_server_stats(const dim3g_server* srv, uint64_t* completed, uint64_t* passes, uint64_t* reserved_bytes,
                       uint64_t* output_budget);
/* Finishes queued requests, then stops the lanes and frees all outputs. */
void dim3g_server_destroy(dim3g_server* srv);

/* ---- batches of independent joins, one CUDA graph --------------------
 * n joins, each with its own device R (rels[2i]) and S (rels[2i+1]),
 * planned once: the index build of all 2n relations and the query pass are
 * captured into one CUDA graph, and every dim3g_batch_run is one graph
 * launch (no host synchronisation inside).  q[i].r / q[i].s are ignored;
 * outputs, capacities and ops are fixed at creation.  The inputs may change
 * between runs (not their sizes).  Results land in q[i] on every run. */
typedef struct dim3g_batch dim3g_batch;
int dim3g_batch_create(dim3g_ctx* ctx, const dim3g_relation* rels, const dim3g_query* q, uint32_t n,
                       dim3g_batch** b);
int dim3g_batch_run(dim3g_batch* b, dim3g_query* q);
/* Device ms of the last run (graph launch to completion), kernel launches
 * per run, device bytes held. */
int dim3g_batch_info(const dim3g_batch* b, float* ms_last, uint64_t* launches_per_run, uint64_t* device_bytes);
void dim3g_batch_destroy(dim3g_batch* b);

/* ---- autotuner ----------------------------------------------------------
 * Replaces server_parameter_estimator.cpp:77-269 and the cost models that
 * consume its constants (dim3.hpp:42-186): instead of machine constants fed
 * to a model, the join is timed on the caller's device-resident input under
 * candidate settings of the knobs that set the dense/sparse split
 * (dense_block: the heavy rows through the tensor-core product or the sparse
 * kernels; dense_k_max: how many of the heaviest join values the product
 * takes -- the threshold on a join value's candidate mass), the row classes'
 * thresholds and tile shapes (tile_bits_log2, block_threads,
 * block_slots_log2, warp_slots_log2) and the CTA rows' walk (cta_walk), by
 * coordinate descent from the context's current settings (always a trial),
 * and the fastest are applied to the context.  The trial that runs the
 * heavy rows on the sparse kernels also sets the context's measured sparse
 * rate, which the dense block's cost model uses from then on (see
 * dim3g_calibrate for the product's rates).  max_trials bounds the joins run
 * (0: no bound). */
typedef struct {
    int32_t tile_bits_log2, block_threads, block_slots_log2, warp_slots_log2, cta_walk;
    int32_t dense_block, dense_k_max;
    float ms;          /* best measured device ms of one join */
    float ms_default;  /* the starting settings' ms */
    uint32_t trials;   /* settings timed */
} dim3g_tuning;
int dim3g_autotune(dim3g_ctx* ctx, const uint32_t* d_R, uint64_t nR, const uint32_t* d_S, uint64_t nS,
                   uint32_t max_trials, dim3g_tuning* out);
int dim3g_tuning_apply(dim3g_ctx* ctx, const dim3g_tuning* t);
/* The same for a batch: the batch's CUDA graph itself is timed (re-captured
 * per trial) under candidate settings; the fastest stay applied to the
 * batch's context and captured.  Outputs are rewritten by every trial. */
int dim3g_batch_autotune(dim3g_batch* b, uint32_t max_trials, dim3g_tuning* out);
/* Shape signature of a workload ("p<lg |P|>_z<lg |z|>_w<lg candidates per
 * row>"), from one count pass; key_len >= 32. */
int dim3g_tuning_key(dim3g_ctx* ctx, const uint32_t* d_R, uint64_t nR, const uint32_t* d_S, uint64_t nS, char* key,
                     uint64_t key_len);
/* Measures, on this context's device, the rates the dense block's cost
 * model decides with, and makes that model use them (replacing the built-in
 * defaults, which were measured once on a GB300): the tcgen05 fp8 product's
 * throughput on all-ones operands at K = 4096 (fp8_tflops: the ceiling of
 * k_dense_mma, dense flops 2 M N K per second), its fixed time per 128 x 256
 * tile at K = 128 (tile_us: TMA fill and epilogue; the difference between
 * grids of 16 and of 8 tiles per SM, so launch costs cancel), and a device-to-device
 * copy's bandwidth (hbm_gbs, read + write bytes).  Allocates about 100 MB of
 * workspace; a few ms. */
typedef struct {
    float fp8_tflops, tile_us, hbm_gbs;
    float sparse_gbs;  /* the sparse kernels' rate in the cost model (4 B a candidate) */
} dim3g_calibration;
int dim3g_calibrate(dim3g_ctx* ctx, dim3g_calibration* out);

/* Text cache of tunings by key (one line each; the last line of a key wins).
 * Host-only; DIM3G_ERR_INVALID when the file or key is absent. */
int dim3g_tuning_save(const char* path, const char* key, const dim3g_tuning* t);
int dim3g_tuning_load(const char* path, const char* key, dim3g_tuning* out);

/* ---- L+S mapper -----------------------------------------------------
 * Replaces LS_mapper<T,H,Tcounter> (Include/L+S_mapper.hpp:11-160): a GPU
 * value -> dense id map.  insert() gives every key its existing id or the
 * next dense id, in the order of first occurrence inside the batch, exactly
 * as a sequence of the reference's insert() calls would; find() gives the id
 * or -1.  Keys are any 32-bit values; ids are int32. */
typedef struct dim3g_mapper dim3g_mapper;
int dim3g_mapper_create(dim3g_ctx* ctx, uint64_t capacity_hint, dim3g_mapper** m);
void dim3g_mapper_destroy(dim3g_mapper* m);
int dim3g_mapper_insert(dim3g_mapper* m, const uint32_t* keys, uint64_t n, int32_t* ids_out);
int dim3g_mapper_find(dim3g_mapper* m, const uint32_t* keys, uint64_t n, int32_t* ids_out);
int64_t dim3g_mapper_size(const dim3g_mapper* m);
/* clear(): drop all keys, keep the id counter (L+S_mapper.hpp:37-40). */
int dim3g_mapper_clear(dim3g_mapper* m);
/* reset_cnt() / __set_cnt(v) (L+S_mapper.hpp:42-48). */
int dim3g_mapper_set_cnt(dim3g_mapper* m, int64_t cnt);

#ifdef __cplusplus
}
#endif
#endif

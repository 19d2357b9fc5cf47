// tune.cu -- the autotuner: measured GB300 timings choose the kernel knobs.
//
// The reference measures host-memory primitives once
// (server_parameter_estimator.cpp:77-269) and feeds the constants to cost
// models (f1/f2/f3, dim3.hpp:42-186) that pick its dense/sparse split.  Here
// the quantities that decide the path are measured directly: the join itself
// is timed on the caller's device-resident input under candidate settings of
// the knobs that set the dense/sparse split, the row classes' thresholds and
// the tile shapes
//   dense_block       heavy rows through the tensor-core product or not
//   dense_k_max       join values in the product (the dense threshold)
//   tile_bits_log2    z-tile width of the bitmap class
//   block_threads     CTA width of the CTA classes
//   block_slots_log2  CTA hash-set size (the class 2 / class 3 threshold)
//   warp_slots_log2   warp hash-set size (the class 1 / class 2 threshold)
//   cta_walk          how CTA rows share their candidates among warps
// by coordinate descent (one knob at a time, the others at their best so
// far; the starting settings are always a trial), and the fastest settings
// are applied to the context.  Results can be kept in a text cache keyed by
// a shape signature of the workload (log2 buckets of the larger relation's
// tuples, the z domain, and candidates per row).
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "../../include/dim3gpu.h"
#include "internal.h"

namespace I = dim3g_internal;

namespace {

struct Knob {
    const char* name;
    std::vector<int64_t> values;
};

int lg_bucket(double v) {
    int b = 0;
    while (v >= 2.0 && b < 63) {
        v /= 2.0;
        b++;
    }
    return b;
}

// One timed trial: device ms of the join under the context's current
// settings (best of `reps` runs).
int trial(dim3g_ctx* ctx, const uint32_t* d_R, uint64_t nR, const uint32_t* d_S, uint64_t nS, uint32_t* d_out,
          uint64_t cap, int reps, float* ms) {
    float best = 1e30f;
    for (int k = 0; k < reps; k++) {
        uint64_t n = 0;
        const int r = dim3g_join_project_device(ctx, d_R, nR, d_S, nS, d_out, cap, &n);
        if (r) return r;
        dim3g_stats st;
        dim3g_get_stats(ctx, &st);
        if (st.ms_total < best) best = st.ms_total;
    }
    *ms = best;
    return DIM3G_OK;
}

int set_all(dim3g_ctx* ctx, const std::vector<Knob>& knobs, const std::vector<int64_t>& v) {
    for (size_t i = 0; i < knobs.size(); i++) {
        const int r = dim3g_set_param(ctx, knobs[i].name, v[i]);
        if (r) return r;
    }
    return DIM3G_OK;
}

}  // namespace

extern "C" {

int dim3g_tuning_key(dim3g_ctx* ctx, const uint32_t* d_R, uint64_t nR, const uint32_t* d_S, uint64_t nS, char* key,
                     uint64_t key_len) {
    if (!ctx || !key || key_len < 32) return DIM3G_ERR_INVALID;
    uint64_t n = 0;
    const int r = dim3g_join_project_count_device(ctx, d_R, nR, d_S, nS, &n);
    if (r) return r;
    dim3g_stats st;
    dim3g_get_stats(ctx, &st);
    const double per_row = st.nx ? (double)st.out_j / (double)st.nx : 0.0;
    snprintf(key, key_len, "p%d_z%d_w%d", lg_bucket((double)st.n_big), lg_bucket((double)st.nz), lg_bucket(per_row));
    return DIM3G_OK;
}

int dim3g_autotune(dim3g_ctx* ctx, const uint32_t* d_R, uint64_t nR, const uint32_t* d_S, uint64_t nS,
                   uint32_t max_trials, dim3g_tuning* out) {
    if (!ctx || !out) return DIM3G_ERR_INVALID;
    memset(out, 0, sizeof *out);
    // the dense/sparse split first (it moves the most time), then the
    // sparse kernels' shapes for whatever rows stay sparse
    std::vector<Knob> knobs = {{"dense_block", {1, 0, 2}},
                               {"dense_k_max", {2048, 512, 128, 4096}},
                               {"tile_bits_log2", {19, 18, 17, 20, 16}},
                               {"block_threads", {512, 256, 1024}},
                               {"block_slots_log2", {14, 13, 12}},
                               {"warp_slots_log2", {11, 10, 9, 12}},
                               {"cta_walk", {3, 2, 0, 1}}};
    enum { kDenseKnob = 0, kDenseKKnob = 1 };
    std::vector<int64_t> cur(knobs.size());
    for (size_t i = 0; i < knobs.size(); i++) {
        const int r = dim3g_get_param(ctx, knobs[i].name, &cur[i]);
        if (r) return r;
    }
    // size of the output: one count pass under the starting settings
    uint64_t n_out = 0;
    int r = dim3g_join_project_count_device(ctx, d_R, nR, d_S, nS, &n_out);
    if (r) return r;
    dim3g_stats st;
    dim3g_get_stats(ctx, &st);
    // the tile width matters only when the z domain needs several tiles at
    // some candidate width
    if (st.nz <= (1u << 16)) knobs[0].values = {cur[0]};
    uint32_t* d_out = nullptr;
    const size_t bytes = (size_t)(n_out ? n_out : 1) * 8;
    if (cudaMalloc(&d_out, bytes) != cudaSuccess) {
        cudaGetLastError();
        return I::fail(ctx, DIM3G_ERR_NOMEM, "autotune: output buffer of %zu bytes", bytes);
    }
    const int reps = 2;
    float best_ms = 0;
    uint32_t trials = 0;
    r = trial(ctx, d_R, nR, d_S, nS, d_out, n_out, reps, &best_ms);
    trials++;
    const float ms_default = best_ms;
    bool dense_ran = false;  // some trial put heavy rows through the product
    std::vector<int64_t> best = cur;
    for (size_t i = 0; i < knobs.size() && !r; i++) {
        // the product's join-value count matters only when the product runs
        if (i == kDenseKKnob && (best[kDenseKnob] == 0 || !dense_ran)) continue;
        for (int64_t v : knobs[i].values) {
            if (v == best[i]) continue;
            if (max_trials && trials >= max_trials) break;
            std::vector<int64_t> cand = best;
            cand[i] = v;
            if (set_all(ctx, knobs, cand)) continue;  // a combination the context rejects
            float ms = 0;
            r = trial(ctx, d_R, nR, d_S, nS, d_out, n_out, reps, &ms);
            trials++;
            if (r) break;
            dim3g_stats ts;
            dim3g_get_stats(ctx, &ts);
            if (ts.rows_dense) dense_ran = true;
            // heavy rows on the sparse kernels: their measured rate becomes
            // the cost model's sparse rate (4 algorithmic bytes a candidate)
            if (i == kDenseKnob && v == 0 && ts.out_j_cls[0] && ts.ms_write_cls[0] > 0)
                I::set_sparse_rate(ctx, 4.0 * (double)ts.out_j_cls[0] / (ts.ms_write_cls[0] * 1e-3));
            if (ms < best_ms) {
                best_ms = ms;
                best = cand;
            }
        }
        if (i == kDenseKnob) {
            dim3g_stats ts;
            dim3g_get_stats(ctx, &ts);
            if (ts.rows_dense) dense_ran = true;
        }
    }
    cudaFree(d_out);
    const int r2 = set_all(ctx, knobs, best);
    if (r) return r;
    if (r2) return r2;
    out->dense_block = (int32_t)best[0];
    out->dense_k_max = (int32_t)best[1];
    out->tile_bits_log2 = (int32_t)best[2];
    out->block_threads = (int32_t)best[3];
    out->block_slots_log2 = (int32_t)best[4];
    out->warp_slots_log2 = (int32_t)best[5];
    out->cta_walk = (int32_t)best[6];
    out->ms = best_ms;
    out->ms_default = ms_default;
    out->trials = trials;
    return DIM3G_OK;
}

int dim3g_tuning_apply(dim3g_ctx* ctx, const dim3g_tuning* t) {
    if (!ctx || !t) return DIM3G_ERR_INVALID;
    int r = dim3g_set_param(ctx, "tile_bits_log2", t->tile_bits_log2);
    if (!r) r = dim3g_set_param(ctx, "block_slots_log2", t->block_slots_log2);
    if (!r) r = dim3g_set_param(ctx, "warp_slots_log2", t->warp_slots_log2);
    if (!r) r = dim3g_set_param(ctx, "block_threads", t->block_threads);
    if (!r) r = dim3g_set_param(ctx, "cta_walk", t->cta_walk);
    if (!r) r = dim3g_set_param(ctx, "dense_block", t->dense_block);
    if (!r) r = dim3g_set_param(ctx, "dense_k_max", t->dense_k_max);
    return r;
}

// Cache file: one line per key, "key tile block_threads block_lg warp_lg
// cta_walk dense_block dense_k_max ms ms_default trials".
int dim3g_tuning_load(const char* path, const char* key, dim3g_tuning* out) {
    if (!path || !key || !out) return DIM3G_ERR_INVALID;
    FILE* f = fopen(path, "r");
    if (!f) return DIM3G_ERR_INVALID;
    char k[128];
    dim3g_tuning t{};
    int found = 0;
    while (fscanf(f, "%127s %d %d %d %d %d %d %d %f %f %u", k, &t.tile_bits_log2, &t.block_threads,
                  &t.block_slots_log2, &t.warp_slots_log2, &t.cta_walk, &t.dense_block, &t.dense_k_max, &t.ms,
                  &t.ms_default, &t.trials) == 11) {
        if (!strcmp(k, key)) {
            *out = t;
            found = 1;  // the last line for a key wins
        }
    }
    fclose(f);
    return found ? DIM3G_OK : DIM3G_ERR_INVALID;
}

int dim3g_tuning_save(const char* path, const char* key, const dim3g_tuning* t) {
    if (!path || !key || !t || strchr(key, ' ') || strlen(key) > 127) return DIM3G_ERR_INVALID;
    FILE* f = fopen(path, "a");
    if (!f) return DIM3G_ERR_INVALID;
    const int w = fprintf(f, "%s %d %d %d %d %d %d %d %.4f %.4f %u\n", key, t->tile_bits_log2, t->block_threads,
                          t->block_slots_log2, t->warp_slots_log2, t->cta_walk, t->dense_block, t->dense_k_max, t->ms,
                          t->ms_default, t->trials);
    fclose(f);
    return w > 0 ? DIM3G_OK : DIM3G_ERR_INVALID;
}

}  // extern "C"

// internal.h -- what the batched / relation-set translation unit needs from a
// context, without exposing the context's layout.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

struct dim3g_ctx;

namespace dim3g_internal {
cudaStream_t stream(const dim3g_ctx* c);
int device(const dim3g_ctx* c);
int sm_count(const dim3g_ctx* c);
void add_launches(dim3g_ctx* c, uint64_t n);
// The dense block's cost model: the sparse kernels' measured rate (4
// algorithmic bytes a candidate, bytes/s).
void set_sparse_rate(dim3g_ctx* c, double bytes_per_s);
// Records a one-line reason on the context; returns code.
int fail(dim3g_ctx* c, int code, const char* fmt, ...);
}  // namespace dim3g_internal

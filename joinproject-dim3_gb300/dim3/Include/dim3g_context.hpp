// dim3g_context.hpp -- the one GPU context a process's drop-in calls share
// (DIM3, DIM3_parallel, DIM3JoinAggregate and every LS_mapper): device 0, or
// the device DIM3G_DEVICE names.  Created on first use, kept until exit;
// creating a context per object would pay the CUDA set-up each time.
#pragma once

#include <cstdio>
#include <cstdlib>

#include "../../../include/dim3gpu.h"

namespace dim3g_dropin {

inline dim3g_ctx* context() {
    static dim3g_ctx* ctx = [] {
        dim3g_ctx* c = nullptr;
        const char* d = getenv("DIM3G_DEVICE");
        int rc = dim3g_create(d ? atoi(d) : 0, &c);
        if (rc != DIM3G_OK) {
            printf("Fail to create the GPU join context (status %d).\n", rc);
            exit(-1);
        }
        return c;
    }();
    return ctx;
}

}  // namespace dim3g_dropin

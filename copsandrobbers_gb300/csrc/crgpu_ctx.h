// crgpu_ctx.h - the context object behind the C ABI (shared by the API translation units).
#pragma once
#include <cuda_runtime.h>

#include <string>

struct cr_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 1;
    bool profiling = false;
    std::string err;
};

// ctx.h -- the engine context behind the opaque tfhe_gpu_ctx handle of the
// C ABI (include/tfhe_gpu.h).  Internal: only the engine's own translation
// units include it.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "../../include/tfhe_gpu.h"
#include "engine.h"

using tfhe_gb300::DevParams;
using tfhe_gb300::kNumForms;
using tfhe_gb300::Tables;

struct tfhe_gpu_ctx {
    tfhe_params P;
    DevParams dp;
    int device = 0;
    cudaStream_t stream = nullptr;
    // fork/join of a gate batch: the key switch of the full blind-rotation
    // waves runs on `side` while the remainder wave leaves SMs idle
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    void* d_tables = nullptr;  // transform tables: FP64 copy then FP32 copy
    Tables tables{};
    void* d_bk[kNumForms] = {nullptr, nullptr};
    int32_t* d_ks = nullptr;
    int32_t ks_row_stride = 0;
    // scratch slots, grown on demand
    void* d_scratch[4] = {nullptr, nullptr, nullptr, nullptr};
    size_t scratch_bytes[4] = {0, 0, 0, 0};
    int groups_per_cta[kNumForms] = {0, 0};  // launch shape per form; 0 = automatic
    int32_t* d_err = nullptr;  // device status word written by bounded waits (3 = timeout)
    std::string last_error;
    size_t key_bytes = 0;
};

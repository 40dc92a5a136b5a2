// noalloc.cu -- a gate-batch entry point that allocates no memory.
//
// tfhe_gpu_bootsGates keeps its intermediate ciphertexts (the combined gate
// inputs and the extracted samples between the blind rotation and the key
// switch) in scratch buffers that the context grows with cudaMalloc on first
// use.  Some callers cannot have that happen inside a call: a serving loop
// that runs under a fixed, pre-reserved memory budget and must not fail with
// an out-of-memory error halfway through a request; a latency-critical loop
// where cudaMalloc / cudaFree (which can synchronise the whole device) would
// stall work that other streams have in flight; a host framework that owns
// all device memory through its own allocator and forbids raw allocations.
// tfhe_gpu_bootsGates_noalloc serves them: the same three launches, with the
// scratch taken from one fixed array compiled into the library.
//
// The array: file-scope, `static __device__`, 256-byte aligned, 3.4 MB
// (847,872 int32 words).  Every GPU that loads the library holds it until the
// process exits.  A call needs count x ((n + 1) + (kN + 1)) words: up to 512
// gates of the default parameter set.  Larger calls are rejected with
// TFHE_GPU_BAD_PARAM and a message naming the limit.
//
// Host code cannot use `g_noalloc_scratch` as an address (in host code the
// name is a stand-in, not device memory).  The device address comes from
// cudaGetSymbolAddress, looked up with the device current on the first call
// of this entry point in each CUDA context of that device, and cached per
// device together with that context's unique id: after cudaDeviceReset, or
// in another context on the same device, the id differs and the address is
// looked up again instead of reusing one that belongs to a destroyed
// context.  Make the first call in a context before capturing any stream
// into a graph (the lookup can load the library's device code).
//
// All calls on a device share the array, and it keeps whatever the last call
// left in it.  No word of it needs to start at zero: each call writes every
// word it later reads (the gate combination writes all n + 1 words of each
// combined sample, the blind rotation writes all kN + 1 words of each
// extracted sample).  Two calls whose work overlaps on the GPU -- on two
// streams, or from two contexts on the same device -- race on the array:
// serialise them.
#include <cuda.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "ctx.h"
#include "engine.h"

namespace {

constexpr size_t kNoAllocWords = 847872;  // 512 x (631 + 1025) int32

static __device__ __align__(256) int32_t g_noalloc_scratch[kNoAllocWords];

constexpr int kMaxDevices = 64;
std::mutex g_lock;
int32_t* g_ptr[kMaxDevices] = {};
unsigned long long g_ctx_id[kMaxDevices] = {};

using CtxGetCurrentFn = CUresult (*)(CUcontext*);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long*);

// Unique id of the current CUDA context (ids are never reused within a
// process, unlike context handles).  The driver functions come through the
// runtime's entry-point query, so the library needs no link-time libcuda.
cudaError_t current_context_id(unsigned long long* id) {
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000,
                                                         cudaEnableDefault, &q1);
        if (e != cudaSuccess) return e;
        e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2);
        if (e != cudaSuccess) return e;
        if (q1 != cudaDriverEntryPointSuccess || q2 != cudaDriverEntryPointSuccess || !f1 || !f2)
            return cudaErrorSymbolNotFound;
        get_current = reinterpret_cast<CtxGetCurrentFn>(f1);
        get_id = reinterpret_cast<CtxGetIdFn>(f2);
    }
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || !c) return cudaErrorInvalidDevice;
    if (get_id(c, id) != CUDA_SUCCESS) return cudaErrorInvalidDevice;
    return cudaSuccess;
}

// Device address of g_noalloc_scratch in the current context of `device`
// (looked up on the first call in each context, then cached).
cudaError_t scratch_for_device(int device, int32_t** out) {
    if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> guard(g_lock);
    unsigned long long id = 0;
    cudaError_t e = current_context_id(&id);
    if (e != cudaSuccess) return e;
    if (!g_ptr[device] || g_ctx_id[device] != id) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_ptr[device] = static_cast<int32_t*>(p);
        g_ctx_id[device] = id;
    }
    *out = g_ptr[device];
    return cudaSuccess;
}

tfhe_gpu_status set_error(tfhe_gpu_ctx* ctx, tfhe_gpu_status s, const std::string& msg) {
    ctx->last_error = msg;
    return s;
}

tfhe_gpu_status cuda_error(tfhe_gpu_ctx* ctx, cudaError_t e, const char* where) {
    return set_error(ctx, e == cudaErrorInvalidValue ? TFHE_GPU_BAD_PARAM : TFHE_GPU_DEVICE_ERROR,
                     std::string(where) + ": " + cudaGetErrorString(e));
}

}  // namespace

extern "C" tfhe_gpu_status tfhe_gpu_bootsGates_noalloc(tfhe_gpu_ctx* ctx, const int32_t* gates,
                                                       int32_t* out, const int32_t* ca,
                                                       const int32_t* cb, int32_t count,
                                                       tfhe_gpu_form form, void* stream) {
    using namespace tfhe_gb300;
    if (!ctx) return TFHE_GPU_BAD_PARAM;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_error(ctx, e, "cudaSetDevice");
    if (form != TFHE_GPU_FP64 && form != TFHE_GPU_SPLIT_FP32)
        return set_error(ctx, TFHE_GPU_BAD_PARAM, "unknown form");
    if (count < 0 || (count && (!gates || !out || !ca || !cb)))
        return set_error(ctx, TFHE_GPU_BAD_PARAM, "bootsGates_noalloc: bad arguments");
    if (!ctx->d_bk[form])
        return set_error(ctx, TFHE_GPU_NO_KEY, "bootstrapping key of this form not uploaded");
    if (!ctx->d_ks) return set_error(ctx, TFHE_GPU_NO_KEY, "key-switching key not uploaded");
    const size_t w_in = (size_t)ctx->P.n + 1;
    const size_t w_ext = (size_t)ctx->P.k * ctx->P.N + 1;
    const size_t need = (size_t)count * (w_in + w_ext);
    if (need > kNoAllocWords) {
        return set_error(ctx, TFHE_GPU_BAD_PARAM,
                         "bootsGates_noalloc: " + std::to_string(count) +
                             " gates need " + std::to_string(need) +
                             " scratch words; the fixed scratch holds " +
                             std::to_string(kNoAllocWords) + " (at most " +
                             std::to_string(kNoAllocWords / (w_in + w_ext)) +
                             " gates for these parameters)");
    }
    if (count == 0) return TFHE_GPU_OK;
    int32_t* scratch = nullptr;
    e = scratch_for_device(ctx->device, &scratch);
    if (e != cudaSuccess) return cuda_error(ctx, e, "cudaGetSymbolAddress(g_noalloc_scratch)");
    int32_t* x = scratch;                       // count x (n + 1) combined samples
    int32_t* u = scratch + (size_t)count * w_in;  // count x (kN + 1) extracted samples
    cudaStream_t st = stream ? reinterpret_cast<cudaStream_t>(stream) : ctx->stream;

    e = launch_gate_combine(ctx->dp, gates, 0, ca, cb, x, count, st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "gate combination");
    EpArgs a{};
    a.err = ctx->d_err;
    a.x = x;
    a.mu = tfhe_client_mod_switch_to_torus32(1, 8);
    a.lwe_out = u;
    a.gsw = ctx->d_bk[form];
    a.count = count;
    e = launch_external_product(ctx->dp, (Form)form, kEpBlindRotate, ctx->tables, a,
                                ctx->groups_per_cta[form], st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "blind rotation");
    e = launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, u, out, count, st);
    if (e != cudaSuccess) return cuda_error(ctx, e, "key switch");
    return TFHE_GPU_OK;
}

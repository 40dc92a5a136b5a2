// capi.cpp -- implementation of the C ABI (include/tfhe_gpu.h).
//
// A context owns: the transform tables, the transform-domain bootstrapping
// keys of the forms built, the padded key-switching table, reusable scratch
// (gate combinations, extracted samples) and a stream.  Entry points check
// their arguments, enqueue launches and return a status; the reference's
// host instead exits the process on an OpenCL error (host.h:13-18).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/tfhe_gpu.h"
#include "ctx.h"
#include "engine.h"

using namespace tfhe_gb300;

namespace {

tfhe_gpu_status fail(tfhe_gpu_ctx* ctx, tfhe_gpu_status s, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return s;
}

tfhe_gpu_status cuda_fail(tfhe_gpu_ctx* ctx, cudaError_t e, const char* where) {
    std::string msg = std::string(where) + ": " + cudaGetErrorString(e);
    if (e == cudaErrorMemoryAllocation) return fail(ctx, TFHE_GPU_OOM, msg);
    if (e == cudaErrorInvalidValue) return fail(ctx, TFHE_GPU_BAD_PARAM, msg);
    return fail(ctx, TFHE_GPU_DEVICE_ERROR, msg);
}

#define CK(ctx, expr)                                          \
    do {                                                       \
        cudaError_t e_ = (expr);                               \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #expr); \
    } while (0)

cudaStream_t pick(tfhe_gpu_ctx* ctx, void* stream) {
    return stream ? reinterpret_cast<cudaStream_t>(stream) : ctx->stream;
}

int32_t auto_split_bits(const tfhe_params& P) {
    // The split K = Khi 2^s + Klo trades two FP32 errors: the high product
    // sum_p D_p * Khi_p must round to exact integers (its size grows with the
    // digits, sqrt((k+1) l N) terms and the 32 - s bits of Khi), while the
    // low product's rounding error grows with 2^s.  Measured on the output
    // phase noise (bench --workload failures / stress --split-bits): the
    // optimum keeps the high product at the same size, s = floor(Bgbit +
    // log2((k+1) l N) / 2 + 10.75): 24 for the default set (sigma 0.00337 /
    // 0.00325 / 0.00330 / 0.00347 turn at s = 23..26) and 26 for n=500, l=2,
    // Bgbit=10 (0.096 / 0.0263 / 0.0291 / 0.0387 at s = 25..28; FP64 0.0253).
    const double terms = (double)(P.k + 1) * P.l * P.N;
    int s = (int)std::floor(P.Bgbit + 0.5 * std::log2(terms) + 10.75);
    if (s < 16) s = 16;
    if (s > 30) s = 30;
    return s;
}

bool params_supported(const tfhe_params* P, std::string* why) {
    if (!P) { *why = "null params"; return false; }
    if (P->N != 1024) { *why = "only N = 1024 is built"; return false; }
    if (P->k != 1) { *why = "only k = 1 is built"; return false; }
    if (P->n < 1 || P->n > 4096) { *why = "n out of range"; return false; }
    if (P->l < 2 || P->l > 3 || P->Bgbit < 1 || P->l * P->Bgbit > 32) {
        *why = "bad decomposition (l in {2, 3} is built, l * Bgbit <= 32)";
        return false;
    }
    if (P->ks_basebit != 2 || P->ks_t < 4 || P->ks_t > 12 || P->ks_t % 4) {
        *why = "key switch built for basebit = 2, t in {4, 8, 12}";
        return false;
    }
    if (P->split_bits < 0 || P->split_bits > 31) { *why = "split_bits out of range"; return false; }
    return true;
}

tfhe_gpu_status ensure_scratch(tfhe_gpu_ctx* ctx, int slot, size_t bytes, void** out) {
    if (ctx->scratch_bytes[slot] < bytes) {
        if (ctx->d_scratch[slot]) {
            CK(ctx, cudaStreamSynchronize(ctx->stream));
            cudaFree(ctx->d_scratch[slot]);
            ctx->d_scratch[slot] = nullptr;
            ctx->scratch_bytes[slot] = 0;
        }
        size_t want = bytes + bytes / 4;
        CK(ctx, cudaMalloc(&ctx->d_scratch[slot], want));
        ctx->scratch_bytes[slot] = want;
    }
    *out = ctx->d_scratch[slot];
    return TFHE_GPU_OK;
}

bool form_ok(int32_t form) { return form == TFHE_GPU_FP64 || form == TFHE_GPU_SPLIT_FP32; }

// After a synchronisation: a kernel whose bounded wait ran out leaves 3 in
// the device status word.  Report it once and clear it.
tfhe_gpu_status check_device_status(tfhe_gpu_ctx* ctx) {
    int32_t v = 0;
    CK(ctx, cudaMemcpy(&v, ctx->d_err, sizeof(v), cudaMemcpyDeviceToHost));
    if (v == 0) return TFHE_GPU_OK;
    CK(ctx, cudaMemset(ctx->d_err, 0, sizeof(int32_t)));
    return fail(ctx, TFHE_GPU_TIMEOUT, "a bounded wait in a kernel gave up (key-row ring stalled)");
}

tfhe_gpu_status need_bk(tfhe_gpu_ctx* ctx, int32_t form) {
    if (!form_ok(form)) return fail(ctx, TFHE_GPU_BAD_PARAM, "unknown form");
    if (!ctx->d_bk[form]) return fail(ctx, TFHE_GPU_NO_KEY, "bootstrapping key of this form not uploaded");
    return TFHE_GPU_OK;
}

tfhe_gpu_status set_device(tfhe_gpu_ctx* ctx) {
    CK(ctx, cudaSetDevice(ctx->device));
    return TFHE_GPU_OK;
}

#define CHECK_CTX(ctx)                                               \
    do {                                                             \
        if (!(ctx)) return TFHE_GPU_BAD_PARAM;                       \
        tfhe_gpu_status s_ = set_device(ctx);                        \
        if (s_ != TFHE_GPU_OK) return s_;                            \
    } while (0)

#define RET(s)                                   \
    do {                                         \
        tfhe_gpu_status r_ = (s);                \
        if (r_ != TFHE_GPU_OK) return r_;        \
    } while (0)

// bootstrap without KS from LWE samples x into extracted samples u
tfhe_gpu_status run_bootstrap_woks(tfhe_gpu_ctx* ctx, const int32_t* x, int32_t mu, int32_t* u,
                                   int32_t count, int32_t form, cudaStream_t st) {
    EpArgs a{};
    a.err = ctx->d_err;
    a.x = x;
    a.mu = mu;
    a.lwe_out = u;
    a.gsw = ctx->d_bk[form];
    a.count = count;
    CK(ctx, launch_external_product(ctx->dp, (Form)form, kEpBlindRotate, ctx->tables, a,
                                    ctx->groups_per_cta[form], st));
    return TFHE_GPU_OK;
}

// combine -> blind rotation + extraction -> key switch, with the gate
// combinations in x (count x (n+1)) and the extracted samples in u
// (count x (kN+1)), both device buffers of the caller.
tfhe_gpu_status run_gates_in(tfhe_gpu_ctx* ctx, const int32_t* gates, int32_t uniform_gate,
                             int32_t* out, const int32_t* ca, const int32_t* cb, int32_t count,
                             int32_t form, int32_t* x, int32_t* u, cudaStream_t st) {
    CK(ctx, launch_gate_combine(ctx->dp, gates, uniform_gate, ca, cb, x, count, st));
    const int32_t mu = tfhe_client_mod_switch_to_torus32(1, 8);
    const int split = blind_rotate_tail_start((Form)form, ctx->groups_per_cta[form], count);
    if (split == 0) {
        RET(run_bootstrap_woks(ctx, x, mu, u, count, form, st));
        CK(ctx, launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, u, out, count, st));
        return TFHE_GPU_OK;
    }
    // The remainder wave of the blind rotation occupies only part of the
    // SMs: issue it right after the full waves, and the full waves' key
    // switch on the side stream, which fills the idle SMs meanwhile.
    const int n = ctx->P.n, nk = ctx->P.k * ctx->P.N;
    RET(run_bootstrap_woks(ctx, x, mu, u, split, form, st));
    CK(ctx, cudaEventRecord(ctx->ev_fork, st));
    CK(ctx, cudaStreamWaitEvent(ctx->side, ctx->ev_fork, 0));
    CK(ctx, launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, u, out, split, ctx->side));
    CK(ctx, cudaEventRecord(ctx->ev_join, ctx->side));
    // from here on the caller's stream joins the side stream on every path
    tfhe_gpu_status s = run_bootstrap_woks(ctx, x + (size_t)split * (n + 1), mu, u + (size_t)split * (nk + 1),
                                           count - split, form, st);
    if (s == TFHE_GPU_OK) {
        const cudaError_t e = launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, u + (size_t)split * (nk + 1),
                                               out + (size_t)split * (n + 1), count - split, st);
        if (e != cudaSuccess) s = cuda_fail(ctx, e, "key switch");
    }
    const cudaError_t e = cudaStreamWaitEvent(st, ctx->ev_join, 0);
    if (s == TFHE_GPU_OK && e != cudaSuccess) s = cuda_fail(ctx, e, "join");
    return s;
}

tfhe_gpu_status run_gates(tfhe_gpu_ctx* ctx, const int32_t* gates, int32_t uniform_gate,
                          int32_t* out, const int32_t* ca, const int32_t* cb, int32_t count,
                          int32_t form, cudaStream_t st) {
    RET(need_bk(ctx, form));
    if (!ctx->d_ks) return fail(ctx, TFHE_GPU_NO_KEY, "key-switching key not uploaded");
    if (count == 0) return TFHE_GPU_OK;
    const int n = ctx->P.n, nk = ctx->P.k * ctx->P.N;
    void *x = nullptr, *u = nullptr;
    RET(ensure_scratch(ctx, 0, (size_t)count * (n + 1) * sizeof(int32_t), &x));
    RET(ensure_scratch(ctx, 1, (size_t)count * (nk + 1) * sizeof(int32_t), &u));
    return run_gates_in(ctx, gates, uniform_gate, out, ca, cb, count, form, (int32_t*)x, (int32_t*)u, st);
}

}  // namespace

extern "C" {

void tfhe_gpu_default_params(tfhe_params* out) {
    if (!out) return;
    std::memset(out, 0, sizeof(*out));
    out->n = 630;
    out->N = 1024;
    out->k = 1;
    out->l = 3;
    out->Bgbit = 7;
    out->ks_t = 8;
    out->ks_basebit = 2;
    out->split_bits = 0;
    out->lwe_alpha = 1.0 / 32768.0;        // 2^-15
    out->tlwe_alpha = 1.0 / 33554432.0;    // 2^-25
}

const char* tfhe_gpu_status_string(tfhe_gpu_status s) {
    switch (s) {
    case TFHE_GPU_OK: return "ok";
    case TFHE_GPU_BAD_PARAM: return "bad parameter";
    case TFHE_GPU_OOM: return "out of memory";
    case TFHE_GPU_TIMEOUT: return "timeout";
    case TFHE_GPU_DEVICE_ERROR: return "device error";
    case TFHE_GPU_NO_KEY: return "key not uploaded";
    }
    return "unknown status";
}

tfhe_gpu_status tfhe_gpu_create(const tfhe_params* params, int32_t device, tfhe_gpu_ctx** out) {
    if (!out) return TFHE_GPU_BAD_PARAM;
    *out = nullptr;
    std::string why;
    if (!params_supported(params, &why)) return TFHE_GPU_BAD_PARAM;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
        return TFHE_GPU_DEVICE_ERROR;
    tfhe_gpu_ctx* ctx = new tfhe_gpu_ctx();
    ctx->P = *params;
    if (ctx->P.split_bits == 0) ctx->P.split_bits = auto_split_bits(ctx->P);
    ctx->dp = DevParams{ctx->P.n, ctx->P.N, ctx->P.k, ctx->P.l, ctx->P.Bgbit,
                        ctx->P.ks_t, ctx->P.ks_basebit, ctx->P.split_bits};
    ctx->device = device;
    auto bail = [&](tfhe_gpu_status s) {
        tfhe_gpu_destroy(ctx);
        return s;
    };
    if (cudaSetDevice(device) != cudaSuccess) return bail(TFHE_GPU_DEVICE_ERROR);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->ev_join, cudaEventDisableTiming) != cudaSuccess)
        return bail(TFHE_GPU_DEVICE_ERROR);
    const int nt = 2 * twiddle_table_entries();
    std::vector<double> h64(nt);
    make_twiddles_host(h64.data());
    std::vector<float> h32(nt);
    for (int i = 0; i < nt; ++i) h32[i] = (float)h64[i];
    const size_t b64 = nt * sizeof(double), b32 = nt * sizeof(float);
    if (cudaMalloc(&ctx->d_tables, b64 + b32) != cudaSuccess) return bail(TFHE_GPU_OOM);
    if (cudaMemcpy(ctx->d_tables, h64.data(), b64, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy((char*)ctx->d_tables + b64, h32.data(), b32, cudaMemcpyHostToDevice) !=
            cudaSuccess)
        return bail(TFHE_GPU_DEVICE_ERROR);
    ctx->tables.tw64 = ctx->d_tables;
    ctx->tables.tw32 = (char*)ctx->d_tables + b64;
    ctx->key_bytes = b64 + b32;
    if (cudaMalloc(&ctx->d_err, sizeof(int32_t)) != cudaSuccess) return bail(TFHE_GPU_OOM);
    if (cudaMemset(ctx->d_err, 0, sizeof(int32_t)) != cudaSuccess) return bail(TFHE_GPU_DEVICE_ERROR);
    *out = ctx;
    return TFHE_GPU_OK;
}

void tfhe_gpu_destroy(tfhe_gpu_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    for (int f = 0; f < kNumForms; ++f)
        if (ctx->d_bk[f]) cudaFree(ctx->d_bk[f]);
    if (ctx->d_ks) cudaFree(ctx->d_ks);
    for (int s = 0; s < 4; ++s)
        if (ctx->d_scratch[s]) cudaFree(ctx->d_scratch[s]);
    if (ctx->d_tables) cudaFree(ctx->d_tables);
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
    if (ctx->ev_join) cudaEventDestroy(ctx->ev_join);
    if (ctx->side) cudaStreamDestroy(ctx->side);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
}

const char* tfhe_gpu_last_error(const tfhe_gpu_ctx* ctx) {
    return ctx ? ctx->last_error.c_str() : "null context";
}

tfhe_gpu_status tfhe_gpu_get_params(const tfhe_gpu_ctx* ctx, tfhe_params* out) {
    if (!ctx || !out) return TFHE_GPU_BAD_PARAM;
    *out = ctx->P;
    return TFHE_GPU_OK;
}

void* tfhe_gpu_stream(const tfhe_gpu_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

tfhe_gpu_status tfhe_gpu_synchronize(tfhe_gpu_ctx* ctx) {
    CHECK_CTX(ctx);
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return check_device_status(ctx);
}

size_t tfhe_gpu_tgsw_fft_bytes(const tfhe_gpu_ctx* ctx, tfhe_gpu_form form) {
    if (!ctx || !form_ok(form)) return 0;
    return tgsw_fft_bytes(ctx->dp, (Form)form);
}

size_t tfhe_gpu_device_bytes(const tfhe_gpu_ctx* ctx) {
    if (!ctx) return 0;
    size_t b = ctx->key_bytes;
    for (int s = 0; s < 4; ++s) b += ctx->scratch_bytes[s];
    return b;
}

tfhe_gpu_status tfhe_gpu_set_groups_per_cta(tfhe_gpu_ctx* ctx, tfhe_gpu_form form,
                                            int32_t groups) {
    if (!ctx || !form_ok(form)) return TFHE_GPU_BAD_PARAM;
    const bool ok = form == TFHE_GPU_FP64 ? (groups == 0 || groups == 3 || groups == 4 || groups == 16)
                                          : ((groups >= 0 && groups <= 16 && groups != 3));
    if (!ok) return fail(ctx, TFHE_GPU_BAD_PARAM, "unsupported groups per CTA for this form");
    ctx->groups_per_cta[form] = groups;
    return TFHE_GPU_OK;
}

int32_t tfhe_gpu_get_groups_per_cta(const tfhe_gpu_ctx* ctx, tfhe_gpu_form form) {
    if (!ctx || !form_ok(form)) return 0;
    return ctx->groups_per_cta[form];
}

// ---- keys -------------------------------------------------------------

static tfhe_gpu_status build_bk_forms(tfhe_gpu_ctx* ctx, const int32_t* d_bk_time,
                                      uint32_t form_mask) {
    for (int f = 0; f < kNumForms; ++f) {
        if (!(form_mask & (1u << f))) continue;
        const size_t bytes = (size_t)ctx->P.n * tgsw_fft_bytes(ctx->dp, (Form)f);
        if (!ctx->d_bk[f]) {
            CK(ctx, cudaMalloc(&ctx->d_bk[f], bytes));
            ctx->key_bytes += bytes;
        }
        CK(ctx, launch_tgsw_to_fft(ctx->dp, (Form)f, ctx->tables, d_bk_time, ctx->d_bk[f],
                                   ctx->P.n, ctx->stream));
    }
    CK(ctx, cudaStreamSynchronize(ctx->stream));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_upload_bootstrapping_key(tfhe_gpu_ctx* ctx, const int32_t* bk,
                                                  uint32_t form_mask) {
    CHECK_CTX(ctx);
    if (!bk || (form_mask & ~3u) || !form_mask) return fail(ctx, TFHE_GPU_BAD_PARAM, "bk/form_mask");
    const size_t words = (size_t)ctx->P.n * (ctx->P.k + 1) * ctx->P.l * (ctx->P.k + 1) * ctx->P.N;
    int32_t* d = nullptr;
    CK(ctx, cudaMalloc(&d, words * sizeof(int32_t)));
    tfhe_gpu_status s = TFHE_GPU_OK;
    cudaError_t e = cudaMemcpy(d, bk, words * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
        s = cuda_fail(ctx, e, "copy bootstrapping key");
    else
        s = build_bk_forms(ctx, d, form_mask);
    cudaFree(d);
    return s;
}

tfhe_gpu_status tfhe_gpu_upload_bootstrapping_key_fft(tfhe_gpu_ctx* ctx, const double* bk_fft,
                                                      uint32_t form_mask) {
    CHECK_CTX(ctx);
    if (!bk_fft || (form_mask & ~3u) || !form_mask)
        return fail(ctx, TFHE_GPU_BAD_PARAM, "bk_fft/form_mask");
    const int npoly = ctx->P.n * (ctx->P.k + 1) * ctx->P.l * (ctx->P.k + 1);
    const size_t words = (size_t)npoly * ctx->P.N;
    double* d_ref = nullptr;
    void* d_eng = nullptr;
    int32_t* d_time = nullptr;
    tfhe_gpu_status s = TFHE_GPU_OK;
    cudaError_t e = cudaMalloc(&d_ref, words * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_eng, words * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&d_time, words * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemcpy(d_ref, bk_fft, words * sizeof(double), cudaMemcpyHostToDevice);
    // reference values are torus/2^32: scale by 2^32 to integer units,
    // transform back and round: the integer key is recovered exactly.
    if (e == cudaSuccess)
        e = launch_lagrange_ref_to_engine64(d_ref, d_eng, npoly, 4294967296.0, ctx->stream);
    if (e == cudaSuccess)
        e = launch_tgsw_from_fft64(ctx->dp, ctx->tables, d_eng, d_time,
                                   npoly / ((ctx->P.k + 1) * ctx->P.l * (ctx->P.k + 1)), ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess)
        s = cuda_fail(ctx, e, "import transform-domain bootstrapping key");
    else
        s = build_bk_forms(ctx, d_time, form_mask);
    cudaFree(d_ref);
    cudaFree(d_eng);
    cudaFree(d_time);
    return s;
}

tfhe_gpu_status tfhe_gpu_upload_keyswitch_key(tfhe_gpu_ctx* ctx, const int32_t* ks) {
    CHECK_CTX(ctx);
    if (!ks) return fail(ctx, TFHE_GPU_BAD_PARAM, "ks");
    const int n = ctx->P.n;
    const int stride = (n + 1 + 3) & ~3;
    const size_t rows = (size_t)ctx->P.k * ctx->P.N * ctx->P.ks_t * (1 << ctx->P.ks_basebit);
    if (!ctx->d_ks) {
        CK(ctx, cudaMalloc(&ctx->d_ks, rows * stride * sizeof(int32_t)));
        ctx->key_bytes += rows * stride * sizeof(int32_t);
    }
    ctx->ks_row_stride = stride;
    CK(ctx, cudaMemset(ctx->d_ks, 0, rows * stride * sizeof(int32_t)));
    CK(ctx, cudaMemcpy2D(ctx->d_ks, stride * sizeof(int32_t), ks, (n + 1) * sizeof(int32_t),
                         (n + 1) * sizeof(int32_t), rows, cudaMemcpyHostToDevice));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_gate_keyset(tfhe_gpu_ctx* ctx, int32_t* lwe_key, int32_t* tlwe_key,
                                     int32_t* ks, int32_t* bk, uint32_t form_mask) {
    CHECK_CTX(ctx);
    if (!lwe_key || !tlwe_key || !ks || (form_mask & ~3u) || !form_mask)
        return fail(ctx, TFHE_GPU_BAD_PARAM, "keyset args");
    const tfhe_params& P = ctx->P;
    const size_t words = (size_t)P.n * (P.k + 1) * P.l * (P.k + 1) * P.N;
    std::vector<int32_t> own;
    int32_t* h_bk = bk;
    if (!h_bk) {
        own.resize(words);
        h_bk = own.data();
    }
    // every random value on the host, in the reference's order
    RET(gate_keyset_host(&P, lwe_key, tlwe_key, ks, h_bk, false));
    int32_t *d_bk = nullptr, *d_keys = nullptr;
    tfhe_gpu_status s = TFHE_GPU_OK;
    cudaError_t e = cudaMalloc(&d_bk, words * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&d_keys, (size_t)(P.k * P.N + P.n) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemcpy(d_bk, h_bk, words * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(d_keys, tlwe_key, (size_t)P.k * P.N * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess)
        e = cudaMemcpy(d_keys + P.k * P.N, lwe_key, (size_t)P.n * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = launch_tgsw_finish(ctx->dp, d_bk, d_keys, d_keys + P.k * P.N, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) s = cuda_fail(ctx, e, "bootstrapping key on the device");
    if (s == TFHE_GPU_OK) s = build_bk_forms(ctx, d_bk, form_mask);
    if (s == TFHE_GPU_OK && bk) {
        e = cudaMemcpy(bk, d_bk, words * sizeof(int32_t), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) s = cuda_fail(ctx, e, "copy bootstrapping key back");
    }
    cudaFree(d_bk);
    cudaFree(d_keys);
    if (s == TFHE_GPU_OK) s = tfhe_gpu_upload_keyswitch_key(ctx, ks);
    return s;
}

tfhe_gpu_status tfhe_gpu_upload_cloud_key(tfhe_gpu_ctx* ctx, const int32_t* bk, const int32_t* ks,
                                          uint32_t form_mask) {
    CHECK_CTX(ctx);
    if (!bk || !ks) return fail(ctx, TFHE_GPU_BAD_PARAM, "bk/ks");
    RET(tfhe_gpu_upload_bootstrapping_key(ctx, bk, form_mask));
    return tfhe_gpu_upload_keyswitch_key(ctx, ks);
}

tfhe_gpu_status tfhe_gpu_tgsw_to_fft(tfhe_gpu_ctx* ctx, const int32_t* tgsw, void* out,
                                     int32_t count, tfhe_gpu_form form, void* stream) {
    CHECK_CTX(ctx);
    if (!form_ok(form) || count < 0 || (count && (!tgsw || !out)))
        return fail(ctx, TFHE_GPU_BAD_PARAM, "tgsw_to_fft args");
    CK(ctx, launch_tgsw_to_fft(ctx->dp, (Form)form, ctx->tables, tgsw, out, count, pick(ctx, stream)));
    return TFHE_GPU_OK;
}

// ---- Lagrange processor ------------------------------------------------

tfhe_gpu_status tfhe_gpu_IntPolynomial_ifft(tfhe_gpu_ctx* ctx, const int32_t* polys, double* out,
                                            int32_t count, void* stream) {
    CHECK_CTX(ctx);
    if (count < 0 || (count && (!polys || !out))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    CK(ctx, launch_poly_to_lagrange(ctx->dp, ctx->tables, polys, out, count, 1.0, pick(ctx, stream)));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_TorusPolynomial_ifft(tfhe_gpu_ctx* ctx, const int32_t* polys,
                                              double* out, int32_t count, void* stream) {
    CHECK_CTX(ctx);
    if (count < 0 || (count && (!polys || !out))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    CK(ctx, launch_poly_to_lagrange(ctx->dp, ctx->tables, polys, out, count, 1.0 / 4294967296.0,
                                    pick(ctx, stream)));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_TorusPolynomial_fft(tfhe_gpu_ctx* ctx, const double* in, int32_t* polys,
                                             int32_t count, void* stream) {
    CHECK_CTX(ctx);
    if (count < 0 || (count && (!polys || !in))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    CK(ctx, launch_lagrange_to_torus(ctx->dp, ctx->tables, in, polys, count, pick(ctx, stream)));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_LagrangeHalfCPolynomialAddMul(tfhe_gpu_ctx* ctx, double* accum,
                                                       const double* a, const double* b,
                                                       int32_t count, void* stream) {
    CHECK_CTX(ctx);
    if (count < 0 || (count && (!accum || !a || !b))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    CK(ctx, launch_lagrange_addmul(a, b, accum, count, ctx->P.N / 2, pick(ctx, stream)));
    return TFHE_GPU_OK;
}

// ---- hot path ------------------------------------------------------------

tfhe_gpu_status tfhe_gpu_tLweMulByXaiMinusOne(tfhe_gpu_ctx* ctx, int32_t* out, const int32_t* ai,
                                              const int32_t* in, int32_t count, void* stream) {
    CHECK_CTX(ctx);
    if (count < 0 || (count && (!out || !ai || !in))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    CK(ctx, launch_mul_by_xai_minus_one(ctx->dp, in, ai, out, count, pick(ctx, stream)));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_tGswFFTExternMulToTLwe(tfhe_gpu_ctx* ctx, int32_t* accum, const void* gsw,
                                                int32_t gsw_per_item, int32_t count,
                                                tfhe_gpu_form form, void* stream) {
    CHECK_CTX(ctx);
    if (!form_ok(form) || count < 0 || (count && (!accum || !gsw)))
        return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    EpArgs a{};
    a.err = ctx->d_err;
    a.acc_in = accum;
    a.acc_out = accum;
    a.gsw = gsw;
    a.gsw_stride = gsw_per_item ? tgsw_fft_bytes(ctx->dp, (Form)form) : 0;
    a.count = count;
    CK(ctx, launch_external_product(ctx->dp, (Form)form, kEpPlain, ctx->tables, a,
                                    ctx->groups_per_cta[form], pick(ctx, stream)));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_tfhe_MuxRotate_FFT(tfhe_gpu_ctx* ctx, int32_t* result,
                                            const int32_t* accum, const void* gsw,
                                            int32_t gsw_per_item, const int32_t* barai,
                                            int32_t count, tfhe_gpu_form form, void* stream) {
    CHECK_CTX(ctx);
    if (!form_ok(form) || count < 0 || (count && (!result || !accum || !gsw || !barai)))
        return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    EpArgs a{};
    a.err = ctx->d_err;
    a.acc_in = accum;
    a.acc_out = result;
    a.bara = barai;
    a.gsw = gsw;
    a.gsw_stride = gsw_per_item ? tgsw_fft_bytes(ctx->dp, (Form)form) : 0;
    a.count = count;
    CK(ctx, launch_external_product(ctx->dp, (Form)form, kEpMuxRotate, ctx->tables, a,
                                    ctx->groups_per_cta[form], pick(ctx, stream)));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_tfhe_blindRotate_FFT(tfhe_gpu_ctx* ctx, int32_t* accum,
                                              const int32_t* bara, int32_t count,
                                              tfhe_gpu_form form, void* stream) {
    CHECK_CTX(ctx);
    RET(need_bk(ctx, form));
    if (count < 0 || (count && (!accum || !bara))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    EpArgs a{};
    a.err = ctx->d_err;
    a.acc_in = accum;
    a.acc_out = accum;
    a.bara = bara;
    a.gsw = ctx->d_bk[form];
    a.count = count;
    CK(ctx, launch_external_product(ctx->dp, (Form)form, kEpBlindRotate, ctx->tables, a,
                                    ctx->groups_per_cta[form], pick(ctx, stream)));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_tLweExtractLweSample(tfhe_gpu_ctx* ctx, int32_t* out,
                                              const int32_t* accum, int32_t count, void* stream) {
    CHECK_CTX(ctx);
    if (count < 0 || (count && (!out || !accum))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    CK(ctx, launch_extract(ctx->dp, accum, out, count, pick(ctx, stream)));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_lweKeySwitch(tfhe_gpu_ctx* ctx, int32_t* out, const int32_t* in,
                                      int32_t count, void* stream) {
    CHECK_CTX(ctx);
    if (!ctx->d_ks) return fail(ctx, TFHE_GPU_NO_KEY, "key-switching key not uploaded");
    if (count < 0 || (count && (!out || !in))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    CK(ctx, launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, in, out, count,
                             pick(ctx, stream)));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_tfhe_bootstrap_woKS_FFT(tfhe_gpu_ctx* ctx, int32_t* out, const int32_t* x,
                                                 int32_t mu, int32_t count, tfhe_gpu_form form,
                                                 void* stream) {
    CHECK_CTX(ctx);
    RET(need_bk(ctx, form));
    if (count < 0 || (count && (!out || !x))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    return run_bootstrap_woks(ctx, x, mu, out, count, form, pick(ctx, stream));
}

tfhe_gpu_status tfhe_gpu_tfhe_bootstrap_FFT(tfhe_gpu_ctx* ctx, int32_t* out, const int32_t* x,
                                            int32_t mu, int32_t count, tfhe_gpu_form form,
                                            void* stream) {
    CHECK_CTX(ctx);
    RET(need_bk(ctx, form));
    if (!ctx->d_ks) return fail(ctx, TFHE_GPU_NO_KEY, "key-switching key not uploaded");
    if (count < 0 || (count && (!out || !x))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    if (count == 0) return TFHE_GPU_OK;
    void* u;
    RET(ensure_scratch(ctx, 1, (size_t)count * (ctx->P.k * ctx->P.N + 1) * sizeof(int32_t), &u));
    cudaStream_t st = pick(ctx, stream);
    RET(run_bootstrap_woks(ctx, x, mu, (int32_t*)u, count, form, st));
    CK(ctx, launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, (const int32_t*)u, out, count,
                             st));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_bootstrap_tv(tfhe_gpu_ctx* ctx, int32_t* out, const int32_t* x,
                                      const int32_t* tv, int32_t tv_stride, int32_t count,
                                      tfhe_gpu_form form, int32_t keyswitch, void* stream) {
    CHECK_CTX(ctx);
    RET(need_bk(ctx, form));
    if (keyswitch && !ctx->d_ks) return fail(ctx, TFHE_GPU_NO_KEY, "key-switching key not uploaded");
    if (count < 0 || (count && (!out || !x || !tv)) || (tv_stride != 0 && tv_stride != ctx->P.N))
        return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    if (count == 0) return TFHE_GPU_OK;
    cudaStream_t st = pick(ctx, stream);
    int32_t* u = out;
    if (keyswitch) {
        void* scratch;
        RET(ensure_scratch(ctx, 1, (size_t)count * (ctx->P.k * ctx->P.N + 1) * sizeof(int32_t), &scratch));
        u = (int32_t*)scratch;
    }
    EpArgs a{};
    a.err = ctx->d_err;
    a.x = x;
    a.tv = tv;
    a.tv_stride = tv_stride;
    a.lwe_out = u;
    a.gsw = ctx->d_bk[form];
    a.count = count;
    CK(ctx, launch_external_product(ctx->dp, (Form)form, kEpBlindRotate, ctx->tables, a,
                                    ctx->groups_per_cta[form], st));
    if (keyswitch)
        CK(ctx, launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, u, out, count, st));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_bootsGate(tfhe_gpu_ctx* ctx, int32_t gate, int32_t* out,
                                   const int32_t* ca, const int32_t* cb, int32_t count,
                                   tfhe_gpu_form form, void* stream) {
    CHECK_CTX(ctx);
    if (gate < 0 || gate > 9 || count < 0 || (count && (!out || !ca || !cb)))
        return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    return run_gates(ctx, nullptr, gate, out, ca, cb, count, form, pick(ctx, stream));
}

tfhe_gpu_status tfhe_gpu_bootsGates(tfhe_gpu_ctx* ctx, const int32_t* gates, int32_t* out,
                                    const int32_t* ca, const int32_t* cb, int32_t count,
                                    tfhe_gpu_form form, void* stream) {
    CHECK_CTX(ctx);
    if (count < 0 || (count && (!gates || !out || !ca || !cb)))
        return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    return run_gates(ctx, gates, 0, out, ca, cb, count, form, pick(ctx, stream));
}

tfhe_gpu_status tfhe_gpu_bootsMUX(tfhe_gpu_ctx* ctx, int32_t* out, const int32_t* a,
                                  const int32_t* b, const int32_t* c, int32_t count,
                                  tfhe_gpu_form form, void* stream) {
    CHECK_CTX(ctx);
    RET(need_bk(ctx, form));
    if (!ctx->d_ks) return fail(ctx, TFHE_GPU_NO_KEY, "key-switching key not uploaded");
    if (count < 0 || (count && (!out || !a || !b || !c))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    if (count == 0) return TFHE_GPU_OK;
    const int n = ctx->P.n, nk = ctx->P.k * ctx->P.N;
    cudaStream_t st = pick(ctx, stream);
    void *x = nullptr, *u = nullptr, *s = nullptr;
    RET(ensure_scratch(ctx, 0, (size_t)2 * count * (n + 1) * sizeof(int32_t), &x));
    RET(ensure_scratch(ctx, 1, (size_t)2 * count * (nk + 1) * sizeof(int32_t), &u));
    RET(ensure_scratch(ctx, 2, (size_t)count * (nk + 1) * sizeof(int32_t), &s));
    int32_t* x1 = (int32_t*)x;
    int32_t* x2 = x1 + (size_t)count * (n + 1);
    // upstream bootsMUX: AND(a, b) and AND(not a, c) bootstrapped without
    // key switch, added with (0, 1/8), then one key switch.
    CK(ctx, launch_gate_combine(ctx->dp, nullptr, TFHE_GATE_AND, a, b, x1, count, st));
    CK(ctx, launch_gate_combine(ctx->dp, nullptr, TFHE_GATE_ANDNY, a, c, x2, count, st));
    const int32_t mu = tfhe_client_mod_switch_to_torus32(1, 8);
    RET(run_bootstrap_woks(ctx, x1, mu, (int32_t*)u, 2 * count, form, st));
    const int32_t* u1 = (const int32_t*)u;
    const int32_t* u2 = u1 + (size_t)count * (nk + 1);
    CK(ctx, launch_lwe_add2_const(u1, u2, (int32_t*)s, nk + 1, mu, count, st));
    CK(ctx, launch_keyswitch(ctx->dp, ctx->d_ks, ctx->ks_row_stride, (const int32_t*)s, out, count,
                             st));
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_bootsGates_host(tfhe_gpu_ctx* ctx, const int32_t* gates,
                                         int32_t uniform_gate, int32_t* out, const int32_t* ca,
                                         const int32_t* cb, int32_t count, tfhe_gpu_form form) {
    CHECK_CTX(ctx);
    if (count < 0 || (count && (!out || !ca || !cb))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    if (!gates && (uniform_gate < 0 || uniform_gate > 9)) return fail(ctx, TFHE_GPU_BAD_PARAM, "gate");
    if (count == 0) return TFHE_GPU_OK;
    const size_t w = (size_t)ctx->P.n + 1;
    const size_t lwe_bytes = (size_t)count * w * sizeof(int32_t);
    void *d_io = nullptr, *d_g = nullptr;
    RET(ensure_scratch(ctx, 3, 3 * lwe_bytes + (gates ? count * sizeof(int32_t) : 0), &d_io));
    int32_t* d_ca = (int32_t*)d_io;
    int32_t* d_cb = d_ca + (size_t)count * w;
    int32_t* d_out = d_cb + (size_t)count * w;
    if (gates) d_g = d_out + (size_t)count * w;
    cudaStream_t st = ctx->stream;
    CK(ctx, cudaMemcpyAsync(d_ca, ca, lwe_bytes, cudaMemcpyHostToDevice, st));
    CK(ctx, cudaMemcpyAsync(d_cb, cb, lwe_bytes, cudaMemcpyHostToDevice, st));
    if (gates) CK(ctx, cudaMemcpyAsync(d_g, gates, count * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    RET(run_gates(ctx, (const int32_t*)d_g, uniform_gate, d_out, d_ca, d_cb, count, form, st));
    CK(ctx, cudaMemcpyAsync(out, d_out, lwe_bytes, cudaMemcpyDeviceToHost, st));
    CK(ctx, cudaStreamSynchronize(st));
    return check_device_status(ctx);
}

// ---- CUDA graph of the gate pipeline, launch-shape autotuner -----------

struct tfhe_gpu_graph {
    tfhe_gpu_ctx* ctx = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int32_t* x = nullptr;  // private scratch: the graph's pointers must stay valid
    int32_t* u = nullptr;
    int32_t kernels = 0;
};

void tfhe_gpu_graph_destroy(tfhe_gpu_graph* g) {
    if (!g) return;
    if (g->ctx) set_device(g->ctx);
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    cudaFree(g->x);
    cudaFree(g->u);
    delete g;
}

tfhe_gpu_status tfhe_gpu_graph_gates_create(tfhe_gpu_ctx* ctx, const int32_t* gates,
                                            int32_t uniform_gate, int32_t* out, const int32_t* ca,
                                            const int32_t* cb, int32_t count, tfhe_gpu_form form,
                                            tfhe_gpu_graph** result) {
    CHECK_CTX(ctx);
    if (!result || count <= 0 || !out || !ca || !cb || !form_ok(form) ||
        (!gates && (uniform_gate < 0 || uniform_gate > 9)))
        return fail(ctx, TFHE_GPU_BAD_PARAM, "graph args");
    *result = nullptr;
    RET(need_bk(ctx, form));
    if (!ctx->d_ks) return fail(ctx, TFHE_GPU_NO_KEY, "key-switching key not uploaded");
    const int n = ctx->P.n, nk = ctx->P.k * ctx->P.N;
    tfhe_gpu_graph* g = new tfhe_gpu_graph();
    g->ctx = ctx;
    cudaStream_t cs = nullptr;
    auto bail = [&](tfhe_gpu_status s) {
        if (cs) cudaStreamDestroy(cs);
        tfhe_gpu_graph_destroy(g);
        return s;
    };
    cudaError_t e = cudaMalloc(&g->x, (size_t)count * (n + 1) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&g->u, (size_t)count * (nk + 1) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "graph buffers"));
    // one eager run: kernel attributes set, errors surface before capture
    tfhe_gpu_status s = run_gates_in(ctx, gates, uniform_gate, out, ca, cb, count, form, g->x, g->u, cs);
    if (s == TFHE_GPU_OK && (e = cudaStreamSynchronize(cs)) != cudaSuccess) s = cuda_fail(ctx, e, "eager run");
    if (s == TFHE_GPU_OK) s = check_device_status(ctx);
    if (s != TFHE_GPU_OK) return bail(s);
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "begin capture"));
    s = run_gates_in(ctx, gates, uniform_gate, out, ca, cb, count, form, g->x, g->u, cs);
    e = cudaStreamEndCapture(cs, &g->graph);
    if (s != TFHE_GPU_OK) return bail(s);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "end capture"));
    e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) return bail(cuda_fail(ctx, e, "instantiate"));
    size_t nodes = 0;
    if (cudaGraphGetNodes(g->graph, nullptr, &nodes) == cudaSuccess && nodes) {
        std::vector<cudaGraphNode_t> list(nodes);
        cudaGraphGetNodes(g->graph, list.data(), &nodes);
        for (cudaGraphNode_t nd : list) {
            cudaGraphNodeType t;
            if (cudaGraphNodeGetType(nd, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++g->kernels;
        }
    }
    cudaStreamDestroy(cs);
    *result = g;
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_graph_launch(tfhe_gpu_graph* g, void* stream) {
    if (!g || !g->exec) return TFHE_GPU_BAD_PARAM;
    CHECK_CTX(g->ctx);
    CK(g->ctx, cudaGraphLaunch(g->exec, pick(g->ctx, stream)));
    return TFHE_GPU_OK;
}

int32_t tfhe_gpu_graph_kernel_count(const tfhe_gpu_graph* g) { return g ? g->kernels : 0; }

tfhe_gpu_status tfhe_gpu_autotune(tfhe_gpu_ctx* ctx, tfhe_gpu_form form, int32_t count,
                                  int32_t* best_shape, float* best_ms) {
    CHECK_CTX(ctx);
    if (!form_ok(form) || count <= 0) return fail(ctx, TFHE_GPU_BAD_PARAM, "autotune args");
    RET(need_bk(ctx, form));
    static const int kFp32[] = {0, 9, 10, 6, 7, 5, 13, 12, 4, 2, 1};
    static const int kFp64[] = {0, 3, 4};
    const int* cand = form == TFHE_GPU_FP64 ? kFp64 : kFp32;
    const int ncand = form == TFHE_GPU_FP64 ? 3 : 11;
    const int n = ctx->P.n, nk = ctx->P.k * ctx->P.N;
    // synthetic inputs: uniform Torus32 samples (a_i = 0 would skip steps)
    std::vector<int32_t> hx((size_t)count * (n + 1));
    uint64_t st = 0x9E3779B97F4A7C15ull;
    for (auto& v : hx) {
        st ^= st << 13;
        st ^= st >> 7;
        st ^= st << 17;
        v = (int32_t)(uint32_t)(st >> 16);
    }
    int32_t *x = nullptr, *u = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    const int keep = ctx->groups_per_cta[form];
    tfhe_gpu_status s = TFHE_GPU_OK;
    cudaError_t e = cudaMalloc(&x, hx.size() * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc(&u, (size_t)count * (nk + 1) * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMemcpy(x, hx.data(), hx.size() * sizeof(int32_t), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaEventCreate(&e0);
    if (e == cudaSuccess) e = cudaEventCreate(&e1);
    if (e != cudaSuccess) s = cuda_fail(ctx, e, "autotune buffers");
    int best = keep;
    float best_t = 0;
    for (int i = 0; s == TFHE_GPU_OK && i < ncand; ++i) {
        const int shape = cand[i];
        if (shape >= 1 && shape <= 2 && count > 2 * kSmCount) continue;  // far slower than the rest
        ctx->groups_per_cta[form] = shape;
        const int32_t mu = tfhe_client_mod_switch_to_torus32(1, 8);
        float t_min = 0;
        for (int rep = 0; rep < 3 && s == TFHE_GPU_OK; ++rep) {
            cudaEventRecord(e0, ctx->stream);
            s = run_bootstrap_woks(ctx, x, mu, u, count, form, ctx->stream);
            cudaEventRecord(e1, ctx->stream);
            if (s == TFHE_GPU_OK && (e = cudaEventSynchronize(e1)) != cudaSuccess) s = cuda_fail(ctx, e, "autotune");
            if (s == TFHE_GPU_OK) s = check_device_status(ctx);
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && (t_min == 0 || ms < t_min)) t_min = ms;  // first run warms up
        }
        // the first candidate is the automatic shape, which also adapts to
        // other batch sizes: another shape replaces it only when it is more
        // than 2 % faster (not on timing noise between identical launches)
        const float margin = best == cand[0] && i > 0 ? 0.98f : 1.0f;
        if (s == TFHE_GPU_OK && (best_t == 0 || t_min < best_t * margin)) {
            best_t = t_min;
            best = shape;
        }
    }
    ctx->groups_per_cta[form] = s == TFHE_GPU_OK ? best : keep;
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(x);
    cudaFree(u);
    if (s != TFHE_GPU_OK) return s;
    if (best_shape) *best_shape = best;
    if (best_ms) *best_ms = best_t;
    return TFHE_GPU_OK;
}

tfhe_gpu_status tfhe_gpu_selftest_timeout(tfhe_gpu_ctx* ctx, tfhe_gpu_form form, int32_t count) {
    CHECK_CTX(ctx);
    if (count <= 0) return fail(ctx, TFHE_GPU_BAD_PARAM, "count");
    RET(need_bk(ctx, form));
    RET(check_device_status(ctx));  // start from a clean status word
    const int n = ctx->P.n, nk = ctx->P.k * ctx->P.N;
    void *x = nullptr, *u = nullptr;
    RET(ensure_scratch(ctx, 0, (size_t)count * (n + 1) * sizeof(int32_t), &x));
    RET(ensure_scratch(ctx, 1, (size_t)count * (nk + 1) * sizeof(int32_t), &u));
    cudaStream_t st = ctx->stream;
    CK(ctx, cudaMemsetAsync(x, 0, (size_t)count * (n + 1) * sizeof(int32_t), st));
    EpArgs a{};
    a.err = ctx->d_err;
    a.x = (const int32_t*)x;
    a.mu = tfhe_client_mod_switch_to_torus32(1, 8);
    a.lwe_out = (int32_t*)u;
    a.gsw = ctx->d_bk[form];
    a.count = count;
    a.stall_keys = 1;
    CK(ctx, launch_external_product(ctx->dp, (Form)form, kEpBlindRotate, ctx->tables, a,
                                    ctx->groups_per_cta[form], st));
    CK(ctx, cudaStreamSynchronize(st));
    return check_device_status(ctx);
}

tfhe_gpu_status tfhe_gpu_bootsMUX_host(tfhe_gpu_ctx* ctx, int32_t* out, const int32_t* a,
                                       const int32_t* b, const int32_t* c, int32_t count,
                                       tfhe_gpu_form form) {
    CHECK_CTX(ctx);
    if (count < 0 || (count && (!out || !a || !b || !c))) return fail(ctx, TFHE_GPU_BAD_PARAM, "args");
    if (count == 0) return TFHE_GPU_OK;
    const size_t lwe_bytes = (size_t)count * (ctx->P.n + 1) * sizeof(int32_t);
    void* d_io = nullptr;
    RET(ensure_scratch(ctx, 3, 4 * lwe_bytes, &d_io));
    char* base = (char*)d_io;
    int32_t* d_a = (int32_t*)base;
    int32_t* d_b = (int32_t*)(base + lwe_bytes);
    int32_t* d_c = (int32_t*)(base + 2 * lwe_bytes);
    int32_t* d_out = (int32_t*)(base + 3 * lwe_bytes);
    cudaStream_t st = ctx->stream;
    CK(ctx, cudaMemcpyAsync(d_a, a, lwe_bytes, cudaMemcpyHostToDevice, st));
    CK(ctx, cudaMemcpyAsync(d_b, b, lwe_bytes, cudaMemcpyHostToDevice, st));
    CK(ctx, cudaMemcpyAsync(d_c, c, lwe_bytes, cudaMemcpyHostToDevice, st));
    RET(tfhe_gpu_bootsMUX(ctx, d_out, d_a, d_b, d_c, count, form, st));
    CK(ctx, cudaMemcpyAsync(out, d_out, lwe_bytes, cudaMemcpyDeviceToHost, st));
    CK(ctx, cudaStreamSynchronize(st));
    return check_device_status(ctx);
}

}  // extern "C"
